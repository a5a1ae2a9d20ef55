// llap module kernels (src/pipe/modules/llap): the pyramid reduce and
// assemble levels below level 1 and the final full resolution pass
// (assemble of level 0 fused with llap/colour). Pyramid levels are stored as
// 11 f16 planes (NUM_GAMMA curves + grey) each, planar.
//
// The assemble kernels stage the coarse level (its 11 planes and the coarse
// assembled image) of a 32x32 output tile in shared memory and hand each warp
// outputs of one (x, y) parity, so all lanes of a warp share the tap pattern
// of the gauss_expand they evaluate.
#include "common.cuh"
#include "hilite.cuh"
#include "kernels.h"
#include "pixel.cuh"

namespace {

constexpr int NPL = 11;
constexpr int NG = 10;
constexpr int FT = 32;            // output tile
constexpr int FS = FT / 2 + 4;    // coarse slots per side: virtual [X0/2-2, X0/2+FT/2+2)

DEV int mirror1(int i, int n)
{ // mirrored repeat for |overshoot| < n, clamped for slots no output reads
  if(i < 0) i = -1 - i;
  if(i >= n) i = 2 * n - 1 - i;
  return min(max(i, 0), n - 1);
}

// llap/llap.glsl:16-21: the first hi in [1, NUM_GAMMA-1) with gamma(hi) > v;
// the gammas increase, so this counts gamma(1..8) <= v
DEV int gamma_hi_from_v(float v)
{
  int hi = 1;
#pragma unroll
  for(int i = 1; i < NG - 1; i++) hi += (llap_gamma(i) <= v) ? 1 : 0;
  return hi;
}

// one bilinear tap of the reference sampler at a half-texel multiple: x0 the
// left texel, hx whether the x weight is 0.5 (else 0); same for y. fetch(x, y)
// returns the mirrored texel. The arithmetic is the oracle's
// (t00 (1-ax) + t10 ax)(1-ay) + (t01 (1-ax) + t11 ax) ay with the zero-weight
// terms dropped, which is exact for finite texels.
template<class F> DEV float tap(F fetch, int x0, bool hx, int y0, bool hy)
{
  const float r0 = hx ? fetch(x0, y0) * 0.5f + fetch(x0 + 1, y0) * 0.5f : fetch(x0, y0);
  if(!hy) return r0;
  const float r1 = hx ? fetch(x0, y0 + 1) * 0.5f + fetch(x0 + 1, y0 + 1) * 0.5f : fetch(x0, y0 + 1);
  return r0 * 0.5f + r1 * 0.5f;
}

// llap/assemble.comp:54-58 gauss_expand = shared.glsl:99-127 sample_soft at
// (o/2 + 0.5): three taps per axis at o/2+0.5 + {-1.5, 0, 1.5}
template<class F> DEV float expand(F fetch, int ox, int oy)
{
  int x0[3], y0[3];
  bool hx[3], hy[3];
  const int kx = ox >> 1, ky = oy >> 1;
  if(ox & 1) { x0[0] = kx - 1; hx[0] = false; x0[1] = kx; hx[1] = true; x0[2] = kx + 2; hx[2] = false; }
  else       { x0[0] = kx - 2; hx[0] = true;  x0[1] = kx; hx[1] = false; x0[2] = kx + 1; hx[2] = true; }
  if(oy & 1) { y0[0] = ky - 1; hy[0] = false; y0[1] = ky; hy[1] = true; y0[2] = ky + 2; hy[2] = false; }
  else       { y0[0] = ky - 2; hy[0] = true;  y0[1] = ky; hy[1] = false; y0[2] = ky + 1; hy[2] = true; }
  float r = 0.0f;
#pragma unroll
  for(int j = 0; j < 3; j++)
#pragma unroll
  for(int i = 0; i < 3; i++) r += tap(fetch, x0[i], hx[i], y0[j], hy[j]);
  return r / 9.0f;
}

// llap/reduce.comp:17-35 (sample_semisoft), all planes of one level. The four
// half-texel bilinear taps equal ((P00+P10)/4 ...) with the horizontal pair
// sums P (halving is exact), as in the develop kernel.
__global__ void __launch_bounds__(256) k_llap_reduce(const __half *__restrict__ in, int iw, int ih, size_t ip,
    __half *__restrict__ out, int ow, int oh, size_t op)
{
  const int x = blockIdx.x * 32 + threadIdx.x % 32, y = blockIdx.y * 8 + threadIdx.x / 32;
  if(x >= ow || y >= oh) return;
  int xs[3], ys[3];
  for(int a = 0; a < 3; a++) { xs[a] = mirror_full(2 * x - 1 + a, iw); ys[a] = mirror_full(2 * y - 1 + a, ih); }
  for(int k = 0; k < NPL; k++)
  {
    const __half *pl = in + k * ip;
    float P[3][2];
    for(int b = 0; b < 3; b++)
    {
      const __half *row = pl + (size_t)ys[b] * iw;
      const float t0 = h2f(row[xs[0]]), t1 = h2f(row[xs[1]]), t2 = h2f(row[xs[2]]);
      P[b][0] = t0 + t1;
      P[b][1] = t1 + t2;
    }
    const float q00 = (P[0][0] + P[1][0]) * 0.25f, q10 = (P[0][1] + P[1][1]) * 0.25f;
    const float q01 = (P[1][0] + P[2][0]) * 0.25f, q11 = (P[1][1] + P[2][1]) * 0.25f;
    out[k * op + (size_t)y * ow + x] = f2h((((q00 + q10) + q01) + q11) / 4.0f);
  }
}

// stage the 11 planes of the coarse level and the coarse assembled image of
// one output tile: slot (sx, sy) holds the mirrored texel (bx+sx, by+sy)
DEV void stage_coarse(__half (*sl)[FS][FS + 2], const __half *l1, int w1, int h1, size_t p1,
    const __half *coarse, int bx, int by)
{
  for(int i = threadIdx.x; i < (NPL + 1) * FS * FS; i += blockDim.x)
  {
    const int k = i / (FS * FS), r = i % (FS * FS);
    const int sx = r % FS, sy = r / FS;
    const int gx = mirror1(bx + sx, w1), gy = mirror1(by + sy, h1);
    const __half *pl = k < NPL ? l1 + k * p1 : coarse;
    sl[k][sy][sx] = pl[(size_t)gy * w1 + gx];
  }
}

// output pixel of the tile for item t: warps take one (x, y) parity class
DEV bool tile_item(int t, int X0, int Y0, int w0, int h0, int &x, int &y)
{
  constexpr int NB = (FT / 2) * (FT / 2);
  const int ph = t / NB, b = t % NB;
  x = X0 + 2 * (b % (FT / 2)) + (ph & 1);
  y = Y0 + 2 * (b / (FT / 2)) + (ph >> 1);
  return x < w0 && y < h0;
}

// llap/assemble.comp:89-123 for a stored level: output at the size of l0
__global__ void __launch_bounds__(256) k_llap_assemble(const __half *__restrict__ coarse, int first,
    const __half *__restrict__ l0, int w0, int h0, size_t p0,
    const __half *__restrict__ l1, int w1, int h1, size_t p1, __half *__restrict__ out)
{
  __shared__ __half sl[NPL + 1][FS][FS + 2];
  const int X0 = blockIdx.x * FT, Y0 = blockIdx.y * FT;
  const int bx = X0 / 2 - 2, by = Y0 / 2 - 2;
  stage_coarse(sl, l1, w1, h1, p1, first ? l1 + NG * p1 : coarse, bx, by);
  __syncthreads();
  for(int t = threadIdx.x; t < FT * FT; t += blockDim.x)
  {
    int x, y;
    if(!tile_item(t, X0, Y0, w0, h0, x, y)) continue;
    auto fs = [&](int k) { return [=](int ix, int iy) { return h2f(sl[k][iy - by][ix - bx]); }; };
    const float res = expand(fs(NPL), x, y);
    const size_t o = (size_t)y * w0 + x;
    const float v = h2f(l0[NG * p0 + o]);
    const int hi = gamma_hi_from_v(v);
    const float glo = (float)(hi - 1) / (10.0f - 1.0f), ghi = (float)hi / (10.0f - 1.0f);
    const float a = gclamp((v - glo) / (ghi - glo), 0.0f, 1.0f);
    const float la = h2f(l0[(hi - 1) * p0 + o]) - expand(fs(hi - 1), x, y);
    const float lb = h2f(l0[hi * p0 + o]) - expand(fs(hi), x, y);
    out[o] = f2h(res + la * (1.0f - a) + lb * a);
  }
}

// llap/assemble.comp for level 0 (l0 recomputed from the filmcurv output like
// llap/curve.comp) fused with llap/colour.comp:141-160
__global__ void __launch_bounds__(256) k_llap_final(const dev_llap_k3_t p)
{
  __shared__ __half sl[NPL + 1][FS][FS + 2];
  const int X0 = blockIdx.x * FT, Y0 = blockIdx.y * FT;
  const int bx = X0 / 2 - 2, by = Y0 / 2 - 2;
  stage_coarse(sl, p.l1, p.l1w, p.l1h, p.l1plane, p.coarse, bx, by);
  __syncthreads();
  const float sig = p.ll_sigma;
  const float r2s = 1.0f / (2.0f * sig), rden = 1.0f / (2.0f * sig * sig / 3.0f);
  for(int t = threadIdx.x; t < FT * FT; t += blockDim.x)
  {
    int x, y;
    if(!tile_item(t, X0, Y0, p.W, p.H, x, y)) continue;
    float rgb[4];
    ld_half4(p.rgbf + (size_t)y * p.W + x, rgb[0], rgb[1], rgb[2], rgb[3]);
    const float yv = lum2020(gclamp(rgb[0], -1000.0f, 1000.0f), gclamp(rgb[1], -1000.0f, 1000.0f), gclamp(rgb[2], -1000.0f, 1000.0f));
    const float v = f16r(yv);
    const int hi = gamma_hi_from_v(v);
    const float glo = (float)(hi - 1) / (10.0f - 1.0f), ghi = (float)hi / (10.0f - 1.0f);
    const float a = gclamp((v - glo) / (ghi - glo), 0.0f, 1.0f);
    auto fs = [&](int k) { return [=](int ix, int iy) { return h2f(sl[k][iy - by][ix - bx]); }; };
    const float res = expand(fs(NPL), x, y);
    const float c0 = f16r(llap_curve_rcp(yv, glo, sig, r2s, rden, p.ll_shadows, p.ll_highlights, p.ll_clarity));
    const float c1 = f16r(llap_curve_rcp(yv, ghi, sig, r2s, rden, p.ll_shadows, p.ll_highlights, p.ll_clarity));
    const float la = c0 - expand(fs(hi - 1), x, y);
    const float lb = c1 - expand(fs(hi), x, y);
    float yo_ = f16r(res + la * (1.0f - a) + lb * a);
    // llap/colour.comp
    const float yo = fmaxf(lum2020(rgb[0], rgb[1], rgb[2]), 1e-8f);
    if(yo_ < yo) yo_ = yo * expf(1.0f * (yo_ - yo));
    float o[3];
    for(int k = 0; k < 3; k++) o[k] = fmaxf(0.0f, rgb[k] * yo_ / yo);
    p.out[(size_t)y * p.W + x] = mk_half4(o[0], o[1], o[2], 1.0f);
  }
}

} // namespace

cudaError_t launch_llap_reduce(const __half *in, int iw, int ih, size_t iplane,
    __half *out, int ow, int oh, size_t oplane, cudaStream_t s)
{
  dim3 grid((ow + 31) / 32, (oh + 7) / 8);
  k_llap_reduce<<<grid, 256, 0, s>>>(in, iw, ih, iplane, out, ow, oh, oplane);
  return cudaGetLastError();
}

cudaError_t launch_llap_assemble(const __half *coarse, int first, const __half *l0, int w0, int h0, size_t p0,
    const __half *l1, int w1, int h1, size_t p1, __half *out, cudaStream_t s)
{
  dim3 grid((w0 + FT - 1) / FT, (h0 + FT - 1) / FT);
  k_llap_assemble<<<grid, 256, 0, s>>>(coarse, first, l0, w0, h0, p0, l1, w1, h1, p1, out);
  return cudaGetLastError();
}

cudaError_t launch_llap_final(const dev_llap_k3_t &p, cudaStream_t s)
{
  dim3 grid((p.W + FT - 1) / FT, (p.H + FT - 1) / FT);
  k_llap_final<<<grid, 256, 0, s>>>(p);
  return cudaGetLastError();
}
