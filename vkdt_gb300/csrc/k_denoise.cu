// denoise module kernels, wavelet path (strength > 0, src/pipe/modules/denoise):
// half -> downcov -> down x3 -> assemble (all at the half size W/2 x H/2) ->
// doub (full size). The doub output, the denoised normalised mosaic (f16), is
// what the hilite and develop kernels read in place of denoise/noop.
//
// Every node stores f16 images like the reference. The computations whose
// rounding decides a branch (clipped greens, the structure tensor and the
// choice between its two forms, the hot pixel test, the wavelet threshold
// switch, the sample positions of the bilinear taps) use explicit IEEE
// operations in the shader's order, as the oracle evaluates them.
#include "common.cuh"
#include "kernels.h"
#include "sampler.cuh"

namespace {

DEV float unorm16(uint16_t v) { return __fdiv_rn((float)v, 65535.0f); }

// R16_UNORM mosaic read with MIRRORED_REPEAT over the full input
DEV float raw_m(const dev_denoise_t &p, int x, int y)
{
  x = mirror(x, p.in_w); y = mirror(y, p.in_h);
  return unorm16(__ldg(p.mosaic + (size_t)y * p.pitch + x));
}

// denoise/noise.glsl:1-11, edges applied per channel
DEV void noise_sigma(float out[3], const dev_denoise_t &p, float black, float white, float val)
{
  const float x = fmaxf(0.0f, __fdiv_rn(__fsub_rn(val, black), __fsub_rn(white, black)));
  const float s = __fsqrt_rn(__fadd_rn(p.na, __fmul_rn(x, p.nb)));
#pragma unroll
  for(int k = 0; k < 3; k++) out[k] = gclamp(__fmul_rn(p.edge_gain[k], s), 1e-3f, 1e3f);
}

// the same where the result only feeds continuous arithmetic
DEV void noise_sigma_fast(float out[3], const dev_denoise_t &p, float black, float white, float val)
{
  const float s = sqrtf(p.na + fmaxf(0.0f, (val - black) / (white - black)) * p.nb);
#pragma unroll
  for(int k = 0; k < 3; k++) out[k] = gclamp(p.edge_gain[k] * s, 1e-3f, 1e3f);
}

// denoise/down.comp:102-104: decimated (swizzled) write position
DEV void swz(int &x, int &y, int w, int h)
{
  const int ox = (x & 1) * (w + 1) / 2, oy = (y & 1) * (h + 1) / 2;
  x = x / 2 + ox; y = y / 2 + oy;
}

// x^y for x >= 0 on the special function unit (feeds continuous weights only)
DEV float fpow(float x, float y) { return __powf(x, y); }

// ---------------------------------------------------------------- half
// denoise/half.comp:24-74: bayer R, mean of the greens (a clipped green is
// replaced by the other one), B of the 2x2 block, on the raw unorm values
__global__ void __launch_bounds__(256) k_dn_half(const dev_denoise_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  if(p.filters == 9u)
  { // x-trans: the 3x3 block, greens averaged, red and blue by block parity (texelFetch reads)
    const int bx = p.cx + 3 * x, by = p.cy + 3 * y;
    float c[9];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++)
      {
        const int X = bx + i, Y = by + j;
        c[3 * i + j] = (X < p.in_w && Y < p.in_h) ? unorm16(__ldg(p.mosaic + (size_t)Y * p.pitch + X)) : 0.0f;
      }
    const float c0 = __fmul_rn(__fadd_rn(c[1], c[7]), 0.5f), c1 = __fmul_rn(__fadd_rn(c[3], c[5]), 0.5f);
    const bool odd = ((x + y + p.cx + p.cy) & 1) > 0;
    const float g = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(c[0], c[2]), c[4]), c[6]), c[8]), 5.0f);
    p.half_img[(size_t)y * p.hw + x] = mk_half4(odd ? c0 : c1, g, odd ? c1 : c0, 1.0f);
    return;
  }
  const int i0 = p.cx + 2 * x, j0 = p.cy + 2 * y;
  float cx = raw_m(p, i0, j0 + 1), cy = raw_m(p, i0 + 1, j0 + 1);
  float cz = raw_m(p, i0 + 1, j0), cw = raw_m(p, i0, j0);
  if(cx >= p.white[1]) cx = cz;
  if(cz >= p.white[1]) cz = cx;
  p.half_img[(size_t)y * p.hw + x] = mk_half4(cw, __fmul_rn(__fadd_rn(cx, cz), 0.5f), cy, 1.0f);
}

// ---------------------------------------------------------------- downcov
// denoise/downcov.comp:41-63 with cov.glsl:159-276 response(): a 5x5 luminance
// structure tensor in two forms (weighted by px^2 and by 1/px^2), the one with
// the smaller determinant decomposed, then an anisotropic gaussian over the
// 5x5 window that skips hot pixels. One 16x16 tile per CTA, the 20x20 input
// window (mirrored) in shared memory.
constexpr int DC_T = 16, DC_N = DC_T + 4;

// The structure tensor decides two branches of the shader (the form taken and
// the hot pixel skip): its sums are IEEE operations in the shader's order
// without contraction, as the oracle evaluates them, from per texel terms made
// once per staged texel: l = luminance, 1/l, l^2, 1/l^2 and l/25. i/l for the
// integer offsets i in [-2, 2] is i (1/l) exactly (scaling by 1 or 2).
__global__ void __launch_bounds__(256) k_dn_downcov(const dev_denoise_t p)
{
  __shared__ float sr[DC_N][DC_N + 1], sg[DC_N][DC_N + 1], sbl[DC_N][DC_N + 1];
  __shared__ float sl[DC_N][DC_N + 1], sil[DC_N][DC_N + 1], sl2[DC_N][DC_N + 1], sil2[DC_N][DC_N + 1];
  __shared__ float sl25[DC_N][DC_N + 1];
  const int X0 = blockIdx.x * DC_T, Y0 = blockIdx.y * DC_T;
  for(int i = threadIdx.x; i < DC_N * DC_N; i += 256)
  {
    const int tx = i % DC_N, ty = i / DC_N;
    // slots an output reads are within 2 of the image (mirror exact); the
    // clamp only keeps the unused slots of images narrower than a tile in bounds
    const int x = min(max(mirror(X0 - 2 + tx, p.hw), 0), p.hw - 1);
    const int y = min(max(mirror(Y0 - 2 + ty, p.hh), 0), p.hh - 1);
    float v[4];
    ld4(p.half_img, p.hw, x, y, v);
    sr[ty][tx] = v[0]; sg[ty][tx] = v[1]; sbl[ty][tx] = v[2];
    const float l = lum2020(v[0], v[1], v[2]);
    const float l2 = __fmul_rn(l, l);
    sl[ty][tx] = l; sil[ty][tx] = __frcp_rn(l); sl2[ty][tx] = l2; sil2[ty][tx] = __frcp_rn(l2);
    sl25[ty][tx] = __fdiv_rn(l, 25.0f);
  }
  __syncthreads();
  const int lx = threadIdx.x % DC_T, ly = threadIdx.x / DC_T;
  const int x = X0 + lx, y = Y0 + ly;
  if(x >= p.hw || y >= p.hh) return;
  // first moments of the luminance (Sw) and of its inverse (Sb)
  float mw0 = 0.0f, mw1 = 0.0f, mb0 = 0.0f, mb1 = 0.0f, smw = 0.0f, smb = 0.0f;
#pragma unroll
  for(int j = -2; j <= 2; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      const float px = sl[ly + 2 + j][lx + 2 + i], ipx = sil[ly + 2 + j][lx + 2 + i];
      if(i) { mw0 = __fadd_rn(mw0, __fmul_rn((float)i, px)); mb0 = __fadd_rn(mb0, __fmul_rn((float)i, ipx)); }
      if(j) { mw1 = __fadd_rn(mw1, __fmul_rn((float)j, px)); mb1 = __fadd_rn(mb1, __fmul_rn((float)j, ipx)); }
      smw = __fadd_rn(smw, px); smb = __fadd_rn(smb, ipx);
    }
  mw0 = __fdiv_rn(mw0, smw); mw1 = __fdiv_rn(mw1, smw);
  mb0 = __fdiv_rn(mb0, smb); mb1 = __fdiv_rn(mb1, smb);
  // second moments
  float mean_b = 0.0f;
  float Sw00 = 0.0f, Sw01 = 0.0f, Sw10 = 0.0f, Sw11 = 0.0f, Sb00 = 0.0f, Sb01 = 0.0f, Sb10 = 0.0f, Sb11 = 0.0f;
  float sw = 0.0f, sb = 0.0f;
#pragma unroll
  for(int j = -2; j <= 2; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      mean_b = __fadd_rn(mean_b, sl25[ly + 2 + j][lx + 2 + i]);
      const float p2 = sl2[ly + 2 + j][lx + 2 + i], b2 = sil2[ly + 2 + j][lx + 2 + i];
      const float q0 = __fsub_rn((float)i, mw0), q1 = __fsub_rn((float)j, mw1);
      Sw00 = __fadd_rn(Sw00, __fmul_rn(__fmul_rn(p2, q0), q0));
      Sw01 = __fadd_rn(Sw01, __fmul_rn(__fmul_rn(p2, q0), q1));
      Sw10 = __fadd_rn(Sw10, __fmul_rn(__fmul_rn(p2, q1), q0));
      Sw11 = __fadd_rn(Sw11, __fmul_rn(__fmul_rn(p2, q1), q1));
      sw = __fadd_rn(sw, p2);
      const float r0 = __fsub_rn((float)i, mb0), r1 = __fsub_rn((float)j, mb1);
      Sb00 = __fadd_rn(Sb00, __fmul_rn(__fmul_rn(b2, r0), r0));
      Sb01 = __fadd_rn(Sb01, __fmul_rn(__fmul_rn(b2, r0), r1));
      Sb10 = __fadd_rn(Sb10, __fmul_rn(__fmul_rn(b2, r1), r0));
      Sb11 = __fadd_rn(Sb11, __fmul_rn(__fmul_rn(b2, r1), r1));
      sb = __fadd_rn(sb, b2);
    }
  Sw00 = __fdiv_rn(Sw00, sw); Sw01 = __fdiv_rn(Sw01, sw); Sw10 = __fdiv_rn(Sw10, sw); Sw11 = __fdiv_rn(Sw11, sw);
  Sb00 = __fdiv_rn(Sb00, sb); Sb01 = __fdiv_rn(Sb01, sb); Sb10 = __fdiv_rn(Sb10, sb); Sb11 = __fdiv_rn(Sb11, sb);
  // cov.glsl: the form with the smaller determinant
  const float detw = __fsub_rn(__fmul_rn(Sw00, Sw11), __fmul_rn(Sw10, Sw01));
  const float detb = __fsub_rn(__fmul_rn(Sb00, Sb11), __fmul_rn(Sb10, Sb01));
  const bool usew = detw < detb;
  float eval[2], e0[2], e1[2];
  if(usew) evd2x2(eval, e0, e1, Sw00, Sw10, Sw11);
  else     evd2x2(eval, e0, e1, Sb00, Sb10, Sb11);
  eval[1] *= 0.05f;
  eval[0] = gclamp(eval[0], 0.01f, 25.0f); eval[1] = gclamp(eval[1], 0.01f, 25.0f);
  const float ie0 = 1.0f / eval[0], ie1 = 1.0f / eval[1];
  // anisotropic gaussian over the window, hot pixels (r > 2 mean) left out.
  // exp(-0.5 (x0^2 / e0 + x1^2 / e1)), x0 = e0 . (i, j), x1 = e1 . (i, j), as the
  // quadratic form exp2(qa i^2 + qb i j + qc j^2) with coefficients made once
  // (continuous weights: the products round differently, the weights agree)
  const float kq = -0.5f * 1.4426950408889634f;
  const float qa = kq * (e0[0] * e0[0] * ie0 + e1[0] * e1[0] * ie1);
  const float qb = kq * 2.0f * (e0[0] * e0[1] * ie0 + e1[0] * e1[1] * ie1);
  const float qc = kq * (e0[1] * e0[1] * ie0 + e1[1] * e1[1] * ie1);
  const float hot = __fmul_rn(2.0f, mean_b);
  float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, wt = 0.0f;
  uint32_t skip = 0;
#pragma unroll
  for(int j = -2; j <= 2; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      const float pr = sr[ly + 2 + j][lx + 2 + i];
      if(pr > hot) { skip |= 1u << ((i + 2) + 5 * (j + 2)); continue; }
      float ex;
      asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(ex) : "f"(qa * (float)(i * i) + qb * (float)(i * j) + qc * (float)(j * j)));
      const float ww = fmaxf(1e-9f, ex);
      r0 += ww * pr; r1 += ww * sg[ly + 2 + j][lx + 2 + i]; r2 += ww * sbl[ly + 2 + j][lx + 2 + i];
      wt += ww;
    }
  if(p.dbg_cov) p.dbg_cov[(size_t)y * p.hw + x] = skip | (usew ? 1u << 25 : 0u);
  const float d = 1.0f / fmaxf(wt, 1e-8f);
  float edge = gclamp(75.0f * fmaxf(0.0f, eval[1] - 0.09f), 0.0f, 1.0f);
  edge = smoothstep(0.4f, 0.75f, edge);
  edge = gclamp(0.02f + edge, 0.0f, 1.0f);
  int X = x, Y = y;
  swz(X, Y, p.hw, p.hh);
  p.lvl[0][(size_t)Y * p.hw + X] = mk_half4(r0 * d, r1 * d, r2 * d, edge);
}

// ---------------------------------------------------------------- down
// denoise/down.comp:59-108 (levels 1..3): four bilinear taps in a flower
// around the texel, weighted by how close their x^0.8 values are relative to
// the noise (0.7^level sigma / block); the centre keeps weight 0.2
__global__ void __launch_bounds__(256) k_dn_down(const dev_denoise_t p, const half4 *__restrict__ in,
    half4 *__restrict__ out, float pl)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  const float t = 0.2f;
  float c[4];
  ld4(in, p.hw, x, y, c);
  float ns[3];
  noise_sigma_fast(ns, p, p.black[1], p.white[1], c[0]);
  float wc[3], g1[3], sum[3], wgt[3];
#pragma unroll
  for(int k = 0; k < 3; k++)
  {
    wc[k] = 1.0f / (pl * ns[k] / p.block_f);
    g1[k] = c[k] < 0.0f ? c[k] : fpow(c[k], 0.8f);
    sum[k] = t * c[k]; wgt[k] = t;
  }
  // offsets of the taps (0.5 + o): (1.7, 0.9), (-0.7, 0.1), (0.9, -0.7), (0.1, 1.7). Below
  // 8192 texels the sampler's position of every tap (rounded to 1/256) is the texel x + dx
  // plus the fraction ax whatever x is (checked for every x): the taps read those directly.
  const float ox[4] = { 0.5f + 1.2f, 0.5f - 1.2f, 0.5f + 0.4f, 0.5f - 0.4f };
  const float oy[4] = { 0.5f + 0.4f, 0.5f - 0.4f, 0.5f - 1.2f, 0.5f + 1.2f };
  const int tdx[4] = { 1, -2, 0, -1 }, tdy[4] = { 0, -1, -2, 1 };
  const float tax[4] = { 51.0f / 256.0f, 205.0f / 256.0f, 102.0f / 256.0f, 154.0f / 256.0f };
  const float tay[4] = { 102.0f / 256.0f, 154.0f / 256.0f, 205.0f / 256.0f, 51.0f / 256.0f };
  const bool fixed = p.hw < 8192 && p.hh < 8192;
#pragma unroll
  for(int o = 0; o < 4; o++)
  {
    float col[4];
    if(fixed) bilinear_at(in, p.hw, p.hh, x + tdx[o], y + tdy[o], tax[o], tay[o], col);
    else bilinear(in, p.hw, p.hh, __fadd_rn((float)x, ox[o]), __fadd_rn((float)y, oy[o]), col);
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      const float g0 = col[k] < 0.0f ? col[k] : fpow(col[k], 0.8f);
      const float e = gclamp(1.0f - 0.5f * (wc[k] * fabsf(g0 - g1[k])), 0.0f, 1.0f);
      const float w = e * (1.0f - t) / 4.0f;
      sum[k] += w * col[k];
      wgt[k] += w;
    }
  }
  int X = x, Y = y;
  swz(X, Y, p.hw, p.hh);
  out[(size_t)Y * p.hw + X] = mk_half4(sum[0] / wgt[0], sum[1] / wgt[1], sum[2] / wgt[2], 1.0f);
}

// ---------------------------------------------------------------- assemble
// denoise/assemble.comp:151-273: gather the 4 scales through the swizzle,
// detail coefficients normalised by the noise, a slope based detail mask,
// soft shrinkage at strength^4 (off where the coarse coefficient is large),
// recomposition and a luma blend in YUV
DEV void fetch_z(const half4 *img, int w, int h, int x, int y, float v[3])
{
  if(x < 0 || y < 0 || x >= w || y >= h) { v[0] = v[1] = v[2] = 0.0f; return; }
  float a;
  ld_half4(img + (size_t)y * w + x, v[0], v[1], v[2], a);
}

DEV void m3v(const float *A, const float v[3], float o[3])
{
#pragma unroll
  for(int i = 0; i < 3; i++) o[i] = A[3 * i + 0] * v[0] + A[3 * i + 1] * v[1] + A[3 * i + 2] * v[2];
}

__global__ void __launch_bounds__(256) k_dn_assemble(const dev_denoise_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  const int szx = p.hw + 1, szy = p.hh + 1;
  float d[5][3], orig[3];
  fetch_z(p.half_img, p.hw, p.hh, x, y, orig);
#pragma unroll
  for(int k = 0; k < 3; k++) d[0][k] = orig[k];
  int ex = x, ey = y;
#pragma unroll
  for(int l = 1; l <= 4; l++)
  {
    ex = ex / 2 + (ex & 1) * szx / 2;
    ey = ey / 2 + (ey & 1) * szy / 2;
    fetch_z(p.lvl[l - 1], p.hw, p.hh, ex, ey, d[l]);
  }
  float sigma[3];
  noise_sigma(sigma, p, p.black[1], p.white[1], fmaxf(d[2][0], 0.0f));
  const float *b = p.bscale;
  // channel 0 decides the threshold switch below: IEEE; the others feed continuous math only
#pragma unroll
  for(int l = 0; l < 4; l++)
  {
    d[l][0] = __fdiv_rn(__fsub_rn(d[l][0], d[l + 1][0]), __fmul_rn(sigma[0], b[l]));
#pragma unroll
    for(int k = 1; k < 3; k++) d[l][k] = (d[l][k] - d[l + 1][k]) / (sigma[k] * b[l]);
  }
  float len[4];
#pragma unroll
  for(int l = 0; l < 4; l++) len[l] = sqrtf(d[l][0] * d[l][0] + d[l][1] * d[l][1] + d[l][2] * d[l][2]);
  const float slope = ((len[3] - len[0]) / 3.0f + (len[2] - len[1]) + (len[1] - len[0]) + (len[3] - len[2])
                     + (len[2] - len[0]) / 2.0f + (len[3] - len[1]) / 2.0f) / 6.0f;
  float test = fmaxf(0.0f, -slope);
  test = fmaxf(0.0f, 1.0f - test);
  test = test * test; test = test * test; test = test * test; test = test * test;   // pow(test, 16)
  test = gclamp(1.5f * test, 0.0f, 1.0f);
  const float thrs0 = p.thrs0;
  uint32_t sw = 0;
#pragma unroll
  for(int l = 3; l >= 0; l--)
  {
    const bool big = fabsf(d[l][0]) > 10.0f;
    sw |= big ? 1u << l : 0u;
    const float thrs = big ? 10000.0f : thrs0;
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      const float a = fabsf(d[l][k]);
      const float tt = fminf(1.0f, a / (2.0f * thrs));
      d[4][k] += sigma[k] * b[l] * gsign(d[l][k]) * gmix(fmaxf(a - thrs, 0.0f), a, tt);
    }
  }
  float v4[3], vo[3];
#pragma unroll
  for(int k = 0; k < 3; k++)
  {
    const float iwb = p.wb[k] / (p.white[k] - p.black[k]);
    v4[k] = (d[4][k] - p.black[k]) * iwb;
    vo[k] = (orig[k] - p.black[k]) * iwb;
  }
  float yuv[3], yuvo[3], rgb[3];
  m3v(p.rgb_to_yuv, v4, yuv);
  m3v(p.rgb_to_yuv, vo, yuvo);
  yuv[0] = gmix(yuvo[0], yuv[0], p.luma);
  m3v(p.yuv_to_rgb, yuv, rgb);
  float o[3];
#pragma unroll
  for(int k = 0; k < 3; k++) o[k] = rgb[k] / p.wb[k] * (p.white[k] - p.black[k]) + p.black[k];
  p.asm_img[(size_t)y * p.hw + x] = mk_half4(o[0], o[1], o[2], test);
  if(p.dbg_thr) p.dbg_thr[(size_t)y * p.hw + x] = (uint8_t)sw;
}

// ---------------------------------------------------------------- doub
// denoise/doub.comp:35-116 (no gain map): per CFA sample, shrink the
// full resolution residual against the bilinear up-sampled noisy coarse
// level, protected by the detail mask, and normalise to [0, 1]
__global__ void __launch_bounds__(256) k_dn_doub(const dev_denoise_t p)
{
  const int x = blockIdx.x * 32 + threadIdx.x % 32, y = blockIdx.y * 8 + threadIdx.x / 32;
  if(x >= p.W || y >= p.H) return;
  const float ux = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)p.W);
  const float uy = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)p.H);
  const float tx = __fmul_rn(ux, (float)p.hw), ty = __fmul_rn(uy, (float)p.hh);
  float upsm[4], down[4];
  bilinear(p.asm_img, p.hw, p.hh, tx, ty, upsm);
  bilinear(p.half_img, p.hw, p.hh, tx, ty, down);
  const int col = p.filters == 9u ? cfa_xtrans(x, y) : cfa_bayer(x, y);
  const float black = p.black[col], white = p.white[col];
  const float crs = col == 0 ? upsm[0] : (col == 1 ? upsm[1] : upsm[2]);
  const float crs1 = col == 0 ? down[0] : (col == 1 ? down[1] : down[2]);
  float Tt = 0.5f * p.strength * upsm[3];
  if(p.filters == 9u && col != 1) Tt /= fmaxf(1e-4f, upsm[3]);
  const float blendw = 0.5f * ((col == 1 ? p.luma : 1.0f) + 1.0f);
  float sigma[3];
  noise_sigma_fast(sigma, p, black, white, crs);
  float val = raw_m(p, x + p.cx, y + p.cy);
  if(val < white)
  {
    const float wav = (val - crs1) / fmaxf(sigma[0] + sigma[2], 1e-8f);
    const float tt = fminf(1.0f, wav / fmaxf(2.0f * Tt, 1e-8f));
    float uw = fminf(1.0f, upsm[3]);
    uw = uw * uw; uw = uw * uw;                      // pow(min(1, w), 4)
    uw = 1.0f - (1.0f - uw) * p.detail;
    const float aw = fabsf(wav);
    val = gmix(val, fmaxf(0.0f, crs + sigma[1] * gsign(wav) * gmix(fmaxf(0.0f, aw - Tt), aw, tt)), uw * blendw);
  }
  val = fmaxf(0.0f, (val - black) / (white - black));
  p.dn[(size_t)y * p.W + x] = f2h(val);
}

} // namespace

cudaError_t launch_denoise(const dev_denoise_t &p, int stage, cudaStream_t s)
{
  const dim3 gh((p.hw + 15) / 16, (p.hh + 15) / 16);
  switch(stage)
  {
    case 0: k_dn_half<<<gh, 256, 0, s>>>(p); break;
    case 1: k_dn_downcov<<<dim3((p.hw + DC_T - 1) / DC_T, (p.hh + DC_T - 1) / DC_T), 256, 0, s>>>(p); break;
    case 2: case 3: case 4:
      k_dn_down<<<gh, 256, 0, s>>>(p, p.lvl[stage - 2], p.lvl[stage - 1], p.pl[stage - 1]); break;
    case 5: k_dn_assemble<<<gh, 256, 0, s>>>(p); break;
    case 6: k_dn_doub<<<dim3((p.W + 31) / 32, (p.H + 7) / 8), 256, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
