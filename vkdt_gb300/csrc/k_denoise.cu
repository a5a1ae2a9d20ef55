// denoise module kernels, wavelet path (strength > 0, src/pipe/modules/denoise):
// half -> downcov -> down x3 -> assemble (all at the half size W/2 x H/2) ->
// doub (full size); on bayer mosaics half is made inside the downcov launch. The doub output, the denoised normalised mosaic (f16), is
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
#include "denoise.cuh"
#include "gauss.cuh"

namespace {

// R16_UNORM: v / 65535 correctly rounded (unorm16_exact, equal to the IEEE quotient on every code)
DEV float unorm16(uint16_t v) { return unorm16_exact(v); }

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

// GLSL pow(x, y) = exp2(y log2(x)) for x >= 0 on the special function unit with
// denormals flushed: the bases are blends of f16 image values, far above the
// f32 denormal range (feeds continuous weights only)
DEV float fpow(float x, float y)
{
  float l, r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(x));
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y * l));
  return r;
}

// square root on the special function unit (feeds continuous values only)
DEV float sqrt_fast(float x) { float r; asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }

// channel k (compile time) of a half4 texel loaded as two words
DEV float hch(uint2 v, int k)
{
  const uint32_t w = k < 2 ? v.x : v.y;
  const __half2 h = *reinterpret_cast<const __half2 *>(&w);
  return (k & 1) ? __high2float(h) : __low2float(h);
}

// texture()'s blend at fractions (ax, ay) of the four texels, as bilinear_at
DEV float blend4(float t00, float t10, float t01, float t11, float ax, float ay)
{
  return (t00 * (1.0f - ax) + t10 * ax) * (1.0f - ay) + (t01 * (1.0f - ax) + t11 * ax) * ay;
}

// blend4 of two channels side by side (paired FP32: each component rounds as the scalar form)
DEV float2 blend4x2(float2 t00, float2 t10, float2 t01, float2 t11, float ax, float ay)
{
  const float2 a = make_float2(ax, ax), b = make_float2(1.0f - ax, 1.0f - ax);
  const float2 top = __ffma2_rn(t10, a, __fmul2_rn(t00, b)), bot = __ffma2_rn(t11, a, __fmul2_rn(t01, b));
  return __ffma2_rn(bot, make_float2(ay, ay), __fmul2_rn(top, make_float2(1.0f - ay, 1.0f - ay)));
}

// ---------------------------------------------------------------- half
// the bayer half texel (x, y): R, the mean of the greens, B of its 2x2 block.
// The block lies in the mosaic (the crop window is even and inside it): no
// mirrored read.
struct bayer_block_t { uint16_t c[4]; };   // the 2x2 codes: (0,0), (1,0), (0,1), (1,1)
DEV bayer_block_t half_bayer_load(const dev_denoise_t &p, int x, int y)
{
  const uint16_t *r0 = p.mosaic + (size_t)(p.cy + 2 * y) * p.pitch + p.cx + 2 * x, *r1 = r0 + p.pitch;
  bayer_block_t b;
  b.c[0] = __ldg(r0); b.c[1] = __ldg(r0 + 1); b.c[2] = __ldg(r1); b.c[3] = __ldg(r1 + 1);
  return b;
}
DEV void half_bayer_eval(const dev_denoise_t &p, const bayer_block_t &b, float v[3])
{
  float cx = unorm16_exact(b.c[2]), cy = unorm16_exact(b.c[3]);
  float cz = unorm16_exact(b.c[1]), cw = unorm16_exact(b.c[0]);
  if(cx >= p.white[1]) cx = cz;
  if(cz >= p.white[1]) cz = cx;
  v[0] = cw; v[1] = __fmul_rn(__fadd_rn(cx, cz), 0.5f); v[2] = cy;
}
DEV void half_bayer(const dev_denoise_t &p, int x, int y, float v[3]) { half_bayer_eval(p, half_bayer_load(p, x, y), v); }

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
  float v[3];
  half_bayer(p, x, y, v);
  p.half_img[(size_t)y * p.hw + x] = mk_half4(v[0], v[1], v[2], 1.0f);
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
// once per staged texel: l = luminance, 1/l, l^2, 1/l^2 and l/25. The two
// forms (w: l, b: 1/l) are built side by side as pairs where a paired FP32
// instruction rounds each component as the scalar IEEE operation does (as in
// gauss.cuh): i (l, 1/l) + m is one paired fma, exact as the product by the
// integer offset i in [-2, 2] is; the differences to the means, the products
// and the quotients (div2_ry from one correctly rounded reciprocal per sum)
// are paired. The code generator contracts a paired product into the paired
// sum that takes it, so the products the sums take are paired fmas with an
// opaque -0 addend (exact), checked against the scalar IEEE form on the device.
// HALF (bayer): the window is made from the mosaic here (half_bayer, rounded to
// f16 as the stored half image) and the tile's own texels of the half image are
// written, in place of a launch of k_dn_half.
#ifndef VKDT_DOWNCOV_CTAS
#define VKDT_DOWNCOV_CTAS 5    // CTAs per SM the register budget is cut for
#endif
template<bool HALF>
__global__ void __launch_bounds__(256, VKDT_DOWNCOV_CTAS) k_dn_downcov(const dev_denoise_t p)
{
  __shared__ float2 s_l[DC_N][DC_N];    // (l, 1/l)
  __shared__ float4 s_q[DC_N][DC_N];    // (l^2, 1/l^2, l/25, -)
  __shared__ float4 s_c[DC_N][DC_N];    // (r, g, b, -)
  const int X0 = blockIdx.x * DC_T, Y0 = blockIdx.y * DC_T;
  // the window's slots, two per thread: all loads issued before the first is used
  constexpr int NS = (DC_N * DC_N + 255) / 256;
  const bool inner = X0 >= 2 && Y0 >= 2 && X0 + DC_N - 2 <= p.hw && Y0 + DC_N - 2 <= p.hh;
  bayer_block_t blk[NS];
  uint2 tex[NS];
#pragma unroll
  for(int r = 0; r < NS; r++)
  {
    const int i = threadIdx.x + 256 * r;
    if(i >= DC_N * DC_N) break;
    const int tx = i % DC_N, ty = i / DC_N;
    int x = X0 - 2 + tx, y = Y0 - 2 + ty;
    if(!inner)
    { // slots an output reads are within 2 of the image (mirror exact); the
      // clamp only keeps the unused slots of images narrower than a tile in bounds
      x = min(max(mirror(x, p.hw), 0), p.hw - 1);
      y = min(max(mirror(y, p.hh), 0), p.hh - 1);
    }
    if(HALF) blk[r] = half_bayer_load(p, x, y);
    else tex[r] = __ldg(reinterpret_cast<const uint2 *>(p.half_img + (size_t)y * p.hw + x));
  }
#pragma unroll
  for(int r = 0; r < NS; r++)
  {
    const int i = threadIdx.x + 256 * r;
    if(i >= DC_N * DC_N) break;
    const int tx = i % DC_N, ty = i / DC_N;
    float v[4];
    if(HALF)
    {
      half_bayer_eval(p, blk[r], v);
      const int x = X0 - 2 + tx, y = Y0 - 2 + ty;
      if(tx >= 2 && ty >= 2 && tx < DC_T + 2 && ty < DC_T + 2 && x < p.hw && y < p.hh)
        p.half_img[(size_t)y * p.hw + x] = mk_half4(v[0], v[1], v[2], 1.0f);
#pragma unroll
      for(int k = 0; k < 3; k++) v[k] = f16r(v[k]);
    }
    else { v[0] = hch(tex[r], 0); v[1] = hch(tex[r], 1); v[2] = hch(tex[r], 2); }
    s_c[ty][tx] = make_float4(v[0], v[1], v[2], 0.0f);
    const float l = lum2020(v[0], v[1], v[2]);
    const float l2 = __fmul_rn(l, l);
    s_l[ty][tx] = make_float2(l, __frcp_rn(l));
    s_q[ty][tx] = make_float4(l2, __frcp_rn(l2), div_ry(l, 25.0f, 1.0f / 25.0f, true), 0.0f);
  }
  __syncthreads();
  const int lx = threadIdx.x % DC_T, ly = threadIdx.x / DC_T;
  const int x = X0 + lx, y = Y0 + ly;
  if(x >= p.hw || y >= p.hh) return;
  // first moments of the luminance (w) and of its inverse (b)
  float2 m0 = make_float2(0.0f, 0.0f), m1 = m0, sm = m0;
#pragma unroll
  for(int j = -2; j <= 2; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      const float2 pv = s_l[ly + 2 + j][lx + 2 + i];
      if(i) m0 = __ffma2_rn(make_float2((float)i, (float)i), pv, m0);
      if(j) m1 = __ffma2_rn(make_float2((float)j, (float)j), pv, m1);
      sm = __fadd2_rn(sm, pv);
    }
  {
    const bool okw = div_ok(sm.x), okb = div_ok(sm.y);
    const float2 ys = make_float2(__frcp_rn(sm.x), __frcp_rn(sm.y));
    m0 = div2_ry(m0, sm, ys, okw, okb);
    m1 = div2_ry(m1, sm, ys, okw, okb);
  }
  // second moments
  const float2 n0 = make_float2(-m0.x, -m0.y), n1 = make_float2(-m1.x, -m1.y);   // i - m as i + (-m): exact
  // the last products as paired fmas with an addend of -0 the compiler cannot see
  // (p.neg_zero; x + -0 = x for every x): the sums that take them are paired adds
  // with no product to contract with
  const float2 nz = make_float2(p.neg_zero, p.neg_zero);
  float mean_b = 0.0f;
  float2 S00 = make_float2(0.0f, 0.0f), S01 = S00, S10 = S00, S11 = S00, ss = S00;   // (w, b)
#pragma unroll
  for(int j = -2; j <= 2; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      const float4 q = s_q[ly + 2 + j][lx + 2 + i];
      mean_b = __fadd_rn(mean_b, q.z);
      const float2 P = make_float2(q.x, q.y);
      const float2 q0 = __fadd2_rn(make_float2((float)i, (float)i), n0);
      const float2 q1 = __fadd2_rn(make_float2((float)j, (float)j), n1);
      const float2 a = __fmul2_rn(P, q0), b = __fmul2_rn(P, q1);
      S00 = __fadd2_rn(S00, __ffma2_rn(a, q0, nz));
      S01 = __fadd2_rn(S01, __ffma2_rn(a, q1, nz));
      S10 = __fadd2_rn(S10, __ffma2_rn(b, q0, nz));
      S11 = __fadd2_rn(S11, __ffma2_rn(b, q1, nz));
      ss = __fadd2_rn(ss, P);
    }
  float Sw00, Sw01, Sw10, Sw11, Sb00, Sb01, Sb10, Sb11;
  {
    const bool okw = div_ok(ss.x), okb = div_ok(ss.y);
    const float2 ys = make_float2(__frcp_rn(ss.x), __frcp_rn(ss.y));
    float2 r;
    r = div2_ry(S00, ss, ys, okw, okb); Sw00 = r.x; Sb00 = r.y;
    r = div2_ry(S01, ss, ys, okw, okb); Sw01 = r.x; Sb01 = r.y;
    r = div2_ry(S10, ss, ys, okw, okb); Sw10 = r.x; Sb10 = r.y;
    r = div2_ry(S11, ss, ys, okw, okb); Sw11 = r.x; Sb11 = r.y;
  }
  // cov.glsl: the form with the smaller determinant
  const float detw = __fsub_rn(__fmul_rn(Sw00, Sw11), __fmul_rn(Sw10, Sw01));
  const float detb = __fsub_rn(__fmul_rn(Sb00, Sb11), __fmul_rn(Sb10, Sb01));
  const bool usew = detw < detb;
  float eval[2], e0[2], e1[2];
  if(usew) evd2x2(eval, e0, e1, Sw00, Sw10, Sw11);
  else     evd2x2(eval, e0, e1, Sb00, Sb10, Sb11);
  eval[1] *= 0.05f;
  eval[0] = gclamp(eval[0], 0.01f, 25.0f); eval[1] = gclamp(eval[1], 0.01f, 25.0f);
  const float ie0 = __fdividef(1.0f, eval[0]), ie1 = __fdividef(1.0f, eval[1]);
  // anisotropic gaussian over the window, hot pixels (r > 2 mean) left out.
  // exp(-0.5 (x0^2 / e0 + x1^2 / e1)), x0 = e0 . (i, j), x1 = e1 . (i, j), as the
  // quadratic form exp2(qa i^2 + qb i j + qc j^2) with coefficients made once
  // (continuous weights: the products round differently, the weights agree)
  const float kq = -0.5f * 1.4426950408889634f;
  const float qa = kq * (e0[0] * e0[0] * ie0 + e1[0] * e1[0] * ie1);
  const float qb = kq * 2.0f * (e0[0] * e0[1] * ie0 + e1[0] * e1[1] * ie1);
  const float qc = kq * (e0[1] * e0[1] * ie0 + e1[1] * e1[1] * ie1);
  const float hot = __fmul_rn(2.0f, mean_b);
  float2 rg = make_float2(0.0f, 0.0f), bw = rg;    // (r, g) and (b, weight) sums
  uint32_t skip = 0;
  // the taps (i, j) and (-i, -j) share their weight: one exponential per pair
#pragma unroll
  for(int j = -2; j <= 0; j++)
#pragma unroll
    for(int i = -2; i <= 2; i++)
    {
      if(j == 0 && i > 0) continue;
      float ex;
      asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(ex) : "f"(qa * (float)(i * i) + qb * (float)(i * j) + qc * (float)(j * j)));
      const float ww = fmaxf(1e-9f, ex);
      const float2 w2 = make_float2(ww, ww);
#pragma unroll
      for(int h = 0; h < 2; h++)
      {
        if(h && i == 0 && j == 0) break;
        const int ti = h ? -i : i, tj = h ? -j : j;
        const float4 c = s_c[ly + 2 + tj][lx + 2 + ti];
        if(c.x > hot) { skip |= 1u << ((ti + 2) + 5 * (tj + 2)); continue; }
        rg = __ffma2_rn(w2, make_float2(c.x, c.y), rg);
        bw = __ffma2_rn(w2, make_float2(c.z, 1.0f), bw);
      }
    }
  if(p.dbg_cov) p.dbg_cov[(size_t)y * p.hw + x] = skip | (usew ? 1u << 25 : 0u);
  const float d = __fdividef(1.0f, fmaxf(bw.y, 1e-8f));
  float edge = gclamp(75.0f * fmaxf(0.0f, eval[1] - 0.09f), 0.0f, 1.0f);
  edge = smoothstep(0.4f, 0.75f, edge);
  edge = gclamp(0.02f + edge, 0.0f, 1.0f);
  int X = x, Y = y;
  swz(X, Y, p.hw, p.hh);
  p.lvl[0][(size_t)Y * p.hw + X] = mk_half4(rg.x * d, rg.y * d, bw.x * d, edge);
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
      const float e = __saturatef(1.0f - 0.5f * (wc[k] * fabsf(g0 - g1[k])));
      const float w = e * (1.0f - t) / 4.0f;
      sum[k] += w * col[k];
      wgt[k] += w;
    }
  }
  int X = x, Y = y;
  swz(X, Y, p.hw, p.hh);
  out[(size_t)Y * p.hw + X] = mk_half4(sum[0] / wgt[0], sum[1] / wgt[1], sum[2] / wgt[2], 1.0f);
}

// the same below 8192 texels (taps at fixed places), one 16x16 tile per CTA:
// the 20x20 window the taps reach (x-2..x+2, mirrored) staged once as f32
// rgb, every tap's four texels read from shared memory at offsets fixed at
// compile time. The weights are continuous: fast quotients.
constexpr int DW_T = 16, DW_N = DW_T + 4;

__global__ void __launch_bounds__(256, 6) k_dn_down_tile(const dev_denoise_t p, const half4 *__restrict__ in,
    half4 *__restrict__ out, float pl)
{
  __shared__ float4 win[DW_N][DW_N];
  const int X0 = blockIdx.x * DW_T, Y0 = blockIdx.y * DW_T;
  // the window's slots, two per thread: both loads issued before the first is used
  constexpr int NS = (DW_N * DW_N + 255) / 256;
  const bool inner = X0 >= 2 && Y0 >= 2 && X0 + DW_N - 2 <= p.hw && Y0 + DW_N - 2 <= p.hh;
  uint2 tex[NS];
#pragma unroll
  for(int r = 0; r < NS; r++)
  {
    const int k = threadIdx.x + 256 * r;
    if(k >= DW_N * DW_N) break;
    const int tx = k % DW_N, ty = k / DW_N;
    int x = X0 - 2 + tx, y = Y0 - 2 + ty;
    if(!inner)
    { // slots an output reads are within 2 of the image (mirror exact); the clamp
      // only keeps the unused slots of images narrower than a tile in bounds
      x = min(max(mirror(x, p.hw), 0), p.hw - 1);
      y = min(max(mirror(y, p.hh), 0), p.hh - 1);
    }
    tex[r] = __ldg(reinterpret_cast<const uint2 *>(in + (size_t)y * p.hw + x));
  }
#pragma unroll
  for(int r = 0; r < NS; r++)
  {
    const int k = threadIdx.x + 256 * r;
    if(k >= DW_N * DW_N) break;
    win[k / DW_N][k % DW_N] = make_float4(hch(tex[r], 0), hch(tex[r], 1), hch(tex[r], 2), 0.0f);
  }
  __syncthreads();
  const int lx = threadIdx.x % DW_T, ly = threadIdx.x / DW_T;
  const int x = X0 + lx, y = Y0 + ly;
  if(x >= p.hw || y >= p.hh) return;
  const float t = 0.2f;
  const float4 cc = win[ly + 2][lx + 2];
  const float c[3] = { cc.x, cc.y, cc.z };
  const float s = sqrt_fast(p.na + fmaxf(0.0f, __fdividef(c[0] - p.black[1], p.white[1] - p.black[1])) * p.nb);
  float wc[3], g1[3], sum[3], wgt[3];
#pragma unroll
  for(int k = 0; k < 3; k++)
  {
    const float ns = gclamp(p.edge_gain[k] * s, 1e-3f, 1e3f);
    wc[k] = __fdividef(p.block_f, pl * ns);
    g1[k] = c[k] < 0.0f ? c[k] : fpow(c[k], 0.8f);
    sum[k] = t * c[k]; wgt[k] = t;
  }
  // the taps of k_dn_down's fixed form: texel (x + tdx, y + tdy) and its right and lower neighbours
  const int tdx[4] = { 1, -2, 0, -1 }, tdy[4] = { 0, -1, -2, 1 };
  const float tax[4] = { 51.0f / 256.0f, 205.0f / 256.0f, 102.0f / 256.0f, 154.0f / 256.0f };
  const float tay[4] = { 102.0f / 256.0f, 154.0f / 256.0f, 205.0f / 256.0f, 51.0f / 256.0f };
#pragma unroll
  for(int o = 0; o < 4; o++)
  {
    const int sx = lx + 2 + tdx[o], sy = ly + 2 + tdy[o];
    const float4 t00 = win[sy][sx], t10 = win[sy][sx + 1], t01 = win[sy + 1][sx], t11 = win[sy + 1][sx + 1];
    const float2 rg = blend4x2(make_float2(t00.x, t00.y), make_float2(t10.x, t10.y), make_float2(t01.x, t01.y),
                               make_float2(t11.x, t11.y), tax[o], tay[o]);
    const float col[3] = { rg.x, rg.y, blend4(t00.z, t10.z, t01.z, t11.z, tax[o], tay[o]) };
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      const float g0 = col[k] < 0.0f ? col[k] : fpow(col[k], 0.8f);
      const float e = __saturatef(1.0f - 0.5f * (wc[k] * fabsf(g0 - g1[k])));
      const float w = e * (1.0f - t) / 4.0f;
      sum[k] += w * col[k];
      wgt[k] += w;
    }
  }
  int X = x, Y = y;
  swz(X, Y, p.hw, p.hh);
  out[(size_t)Y * p.hw + X] = mk_half4(__fdividef(sum[0], wgt[0]), __fdividef(sum[1], wgt[1]),
                                       __fdividef(sum[2], wgt[2]), 1.0f);
}

// ---------------------------------------------------------------- assemble
// denoise/assemble.comp:151-273: gather the 4 scales through the swizzle,
// detail coefficients normalised by the noise, a slope based detail mask,
// soft shrinkage at strength^4 (off where the coarse coefficient is large),
// recomposition and a luma blend in YUV
DEV void fetch_z(const half4 *img, int w, int h, int x, int y, float v[3])
{
  if((unsigned)x >= (unsigned)w || (unsigned)y >= (unsigned)h) { v[0] = v[1] = v[2] = 0.0f; return; }
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
    ex = (ex >> 1) + (ex & 1) * (szx >> 1);   // ex / 2 + (ex & 1) * szx / 2, ex >= 0
    ey = (ey >> 1) + (ey & 1) * (szy >> 1);
    fetch_z(p.lvl[l - 1], p.hw, p.hh, ex, ey, d[l]);
  }
  float sigma[3];
  noise_sigma(sigma, p, p.black[1], p.white[1], fmaxf(d[2][0], 0.0f));
  const float *b = p.bscale;
  // channel 0 decides the threshold switch below: IEEE; the others feed continuous
  // math only (fast reciprocals, square roots and constant quotients)
#pragma unroll
  for(int l = 0; l < 4; l++)
  {
    d[l][0] = __fdiv_rn(__fsub_rn(d[l][0], d[l + 1][0]), __fmul_rn(sigma[0], b[l]));
#pragma unroll
    for(int k = 1; k < 3; k++) d[l][k] = (d[l][k] - d[l + 1][k]) * __fdividef(1.0f, sigma[k] * b[l]);
  }
  float len[4];
#pragma unroll
  for(int l = 0; l < 4; l++) len[l] = sqrt_fast(d[l][0] * d[l][0] + d[l][1] * d[l][1] + d[l][2] * d[l][2]);
  const float slope = ((len[3] - len[0]) * (1.0f / 3.0f) + (len[2] - len[1]) + (len[1] - len[0]) + (len[3] - len[2])
                     + (len[2] - len[0]) * 0.5f + (len[3] - len[1]) * 0.5f) * (1.0f / 6.0f);
  float test = fmaxf(0.0f, -slope);
  test = fmaxf(0.0f, 1.0f - test);
  test = test * test; test = test * test; test = test * test; test = test * test;   // pow(test, 16)
  test = gclamp(1.5f * test, 0.0f, 1.0f);
  const float thrs0 = p.thrs0, ith0 = __fdividef(0.5f, thrs0);
  uint32_t sw = 0;
#pragma unroll
  for(int l = 3; l >= 0; l--)
  {
    const bool big = fabsf(d[l][0]) > 10.0f;
    sw |= big ? 1u << l : 0u;
    const float thrs = big ? 10000.0f : thrs0, ith = big ? 0.5f / 10000.0f : ith0;
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
      const float a = fabsf(d[l][k]);
      const float tt = fminf(1.0f, a * ith);
      // sign(d) mix(max(a - thrs, 0), a, tt) for a = |d|: the mix is >= 0 and 0 at d = 0
      const float m = fmaxf(a - thrs, 0.0f);
      d[4][k] += copysignf(sigma[k] * b[l] * fmaf(a - m, tt, m), d[l][k]);
    }
  }
  float v4[3], vo[3];
#pragma unroll
  for(int k = 0; k < 3; k++)
  {
    v4[k] = (d[4][k] - p.black[k]) * p.wb_norm[k];
    vo[k] = (orig[k] - p.black[k]) * p.wb_norm[k];
  }
  float yuv[3], yuvo[3], rgb[3];
  m3v(p.rgb_to_yuv, v4, yuv);
  m3v(p.rgb_to_yuv, vo, yuvo);
  yuv[0] = gmix(yuvo[0], yuv[0], p.luma);
  m3v(p.yuv_to_rgb, yuv, rgb);
  float o[3];
#pragma unroll
  for(int k = 0; k < 3; k++) o[k] = rgb[k] * p.wb_denorm[k] + p.black[k];
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

// doub for bayer mosaics (W = 2 hw, H = 2 hh) where the bilinear taps of every
// row and column were found on the host to sit at fixed places: output
// position 2i reads texels i-1, i at fraction 0.75 (texel space i - 0.25), 2i+1
// texels i, i+1 at 0.25. One thread per 2x2 quad (R G / G B) reads the 3x3
// texels of both coarse images around its quad once and blends only the
// channels each pixel uses. The branch val < white is on the exact unorm value;
// the rest is continuous and takes the fast quotients.
__global__ void __launch_bounds__(256) k_dn_doub_quad(const dev_denoise_t p)
{
  const int i = blockIdx.x * 32 + threadIdx.x % 32, j = blockIdx.y * 8 + threadIdx.x / 32;
  if(i >= p.hw || j >= p.hh) return;
  // MIRRORED_REPEAT of i - 1 >= -1 and i + 1 <= hw
  const int xs[3] = { i > 0 ? i - 1 : 0, i, i + 1 < p.hw ? i + 1 : p.hw - 1 };
  const int ys[3] = { j > 0 ? j - 1 : 0, j, j + 1 < p.hh ? j + 1 : p.hh - 1 };
  uint2 ta[3][3], th[3][3];
#pragma unroll
  for(int r = 0; r < 3; r++)
  {
    const uint2 *ra = reinterpret_cast<const uint2 *>(p.asm_img + (size_t)ys[r] * p.hw);
    const uint2 *rh = reinterpret_cast<const uint2 *>(p.half_img + (size_t)ys[r] * p.hw);
#pragma unroll
    for(int c = 0; c < 3; c++) { ta[r][c] = __ldg(ra + xs[c]); th[r][c] = __ldg(rh + xs[c]); }
  }
  const float Ts = 0.5f * p.strength;
#pragma unroll
  for(int b = 0; b < 2; b++)
  {
    const int y = 2 * j + b;
    const uint16_t *mrow = p.mosaic + (size_t)(y + p.cy) * p.pitch + 2 * i + p.cx;
    const uint32_t code[2] = { __ldg(mrow), __ldg(mrow + 1) };
    const float ay = b ? 0.25f : 0.75f;
    float out[2];
#pragma unroll
    for(int a = 0; a < 2; a++)
    {
      const int col = a != b ? 1 : (a ? 2 : 0);      // cfa_bayer(2i + a, 2j + b)
      const float ax = a ? 0.25f : 0.75f;
      const uint2 a00 = ta[b][a], a10 = ta[b][a + 1], a01 = ta[b + 1][a], a11 = ta[b + 1][a + 1];
      const uint2 h00 = th[b][a], h10 = th[b][a + 1], h01 = th[b + 1][a], h11 = th[b + 1][a + 1];
      const float crs = blend4(hch(a00, col), hch(a10, col), hch(a01, col), hch(a11, col), ax, ay);
      const float mask = blend4(hch(a00, 3), hch(a10, 3), hch(a01, 3), hch(a11, 3), ax, ay);
      const float crs1 = blend4(hch(h00, col), hch(h10, col), hch(h01, col), hch(h11, col), ax, ay);
      const float black = p.black[col], white = p.white[col];
      const float Tt = Ts * mask;
      const float blendw = 0.5f * ((col == 1 ? p.luma : 1.0f) + 1.0f);
      const float s = sqrt_fast(p.na + fmaxf(0.0f, __fdividef(crs - black, white - black)) * p.nb);
      const float s0 = gclamp(p.edge_gain[0] * s, 1e-3f, 1e3f), s1 = gclamp(p.edge_gain[1] * s, 1e-3f, 1e3f);
      const float s2 = gclamp(p.edge_gain[2] * s, 1e-3f, 1e3f);
      float val = unorm16_exact(code[a]);
      if(val < white)
      {
        const float wav = __fdividef(val - crs1, fmaxf(s0 + s2, 1e-8f));
        const float tt = fminf(1.0f, __fdividef(wav, fmaxf(2.0f * Tt, 1e-8f)));
        float uw = fminf(1.0f, mask);
        uw = uw * uw; uw = uw * uw;                      // pow(min(1, w), 4)
        uw = 1.0f - (1.0f - uw) * p.detail;
        const float aw = fabsf(wav);
        // tt follows the sign of wav: the mix extrapolates for wav < 0 (as in the shader)
        val = gmix(val, fmaxf(0.0f, crs + s1 * gsign(wav) * gmix(fmaxf(0.0f, aw - Tt), aw, tt)), uw * blendw);
      }
      out[a] = fmaxf(0.0f, __fdividef(val - black, white - black));
    }
    *reinterpret_cast<__half2 *>(p.dn + (size_t)y * p.W + 2 * i) = __halves2half2(f2h(out[0]), f2h(out[1]));
  }
}

} // namespace

cudaError_t launch_denoise(const dev_denoise_t &p, int stage, cudaStream_t s)
{
  const dim3 gh((p.hw + 15) / 16, (p.hh + 15) / 16);
  switch(stage)
  {
    case 0: if(p.fuse_half) return cudaErrorInvalidValue; k_dn_half<<<gh, 256, 0, s>>>(p); break;
    case 1:
    {
      const dim3 grid((p.hw + DC_T - 1) / DC_T, (p.hh + DC_T - 1) / DC_T);
      if(p.fuse_half) k_dn_downcov<true><<<grid, 256, 0, s>>>(p);
      else k_dn_downcov<false><<<grid, 256, 0, s>>>(p);
      break;
    }
    case 2: case 3: case 4:
      if(p.hw < 8192 && p.hh < 8192)
        k_dn_down_tile<<<dim3((p.hw + DW_T - 1) / DW_T, (p.hh + DW_T - 1) / DW_T), 256, 0, s>>>(
            p, p.lvl[stage - 2], p.lvl[stage - 1], p.pl[stage - 1]);
      else k_dn_down<<<gh, 256, 0, s>>>(p, p.lvl[stage - 2], p.lvl[stage - 1], p.pl[stage - 1]);
      break;
    case 5: k_dn_assemble<<<gh, 256, 0, s>>>(p); break;
    case 6:
      if(p.doub_fixed) k_dn_doub_quad<<<dim3((p.hw + 31) / 32, (p.hh + 7) / 8), 256, 0, s>>>(p);
      else k_dn_doub<<<dim3((p.W + 31) / 32, (p.H + 7) / 8), 256, 0, s>>>(p);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
