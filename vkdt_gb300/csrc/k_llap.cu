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

// llap/assemble.comp:54-58 gauss_expand = shared.glsl:99-127 sample_soft at
// (o/2 + 0.5): three bilinear taps per axis at o/2+0.5 + {-1.5, 0, 1.5}, which
// land on texel centres or half way between two. Summed per axis the texel
// weights are (.5 .5 1 .5 .5) around k = o/2 for even o and (1 .5 .5 1) from
// k-1 for odd o; the expand is the separable sum of those, divided by 9.
// PX, PY: parities of the output position. fetch(x, y) returns the texel.
template<int PX, int PY, class F> DEV float expand(F fetch, int kx, int ky)
{
  constexpr int NX = PX ? 4 : 5, NY = PY ? 4 : 5;
  constexpr int BXO = PX ? -1 : -2, BYO = PY ? -1 : -2;
  float r = 0.0f;
#pragma unroll
  for(int b = 0; b < NY; b++)
  {
    float row = 0.0f;
#pragma unroll
    for(int a = 0; a < NX; a++)
    {
      const float w = PX ? ((a == 0 || a == 3) ? 1.0f : 0.5f) : (a == 2 ? 1.0f : 0.5f);
      row += w * fetch(kx + BXO + a, ky + BYO + b);
    }
    const float wy = PY ? ((b == 0 || b == 3) ? 1.0f : 0.5f) : (b == 2 ? 1.0f : 0.5f);
    r += wy * row;
  }
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
    out[k * op + (size_t)y * ow + x] = f2h((((q00 + q10) + q01) + q11) * 0.25f);
  }
}

// stage the 11 planes of the coarse level and the coarse assembled image of
// one output tile: slot (sx, sy) holds the mirrored texel (bx+sx, by+sy)
DEV void stage_coarse(float (*sl)[FS][FS + 1], const __half *l1, int w1, int h1, size_t p1,
    const __half *coarse, int bx, int by)
{ // the mirrored position once per slot, then the same texel of every plane
  for(int r = threadIdx.x; r < FS * FS; r += blockDim.x)
  {
    const int sx = r % FS, sy = r / FS;
    const size_t o = (size_t)mirror1(by + sy, h1) * w1 + mirror1(bx + sx, w1);
#pragma unroll
    for(int k = 0; k < NPL; k++) sl[k][sy][sx] = h2f(__ldg(l1 + k * p1 + o));
    sl[NPL][sy][sx] = h2f(__ldg(coarse + o));
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

// llap/assemble.comp:89-123 at one output pixel of parity (PX, PY). l0(k)
// returns the fine level plane k at the pixel, sl holds the coarse level.
template<int PX, int PY, class L0> DEV float assemble_px(L0 l0, float v, const float (*sl)[FS][FS + 1], int x, int y, int bx, int by)
{
  const int kx = x >> 1, ky = y >> 1;
  auto fs = [&](int k) { return [=](int ix, int iy) { return sl[k][iy - by][ix - bx]; }; };
  const float res = expand<PX, PY>(fs(NPL), kx, ky);
  const int hi = gamma_hi_from_v(v);
  const float glo = llap_gamma(hi - 1), ghi = llap_gamma(hi);
  const float a = gclamp((v - glo) / (ghi - glo), 0.0f, 1.0f);
  const float la = l0(hi - 1, glo) - expand<PX, PY>(fs(hi - 1), kx, ky);
  const float lb = l0(hi, ghi) - expand<PX, PY>(fs(hi), kx, ky);
  return res + la * (1.0f - a) + lb * a;
}

// llap/assemble.comp:89-123 for a stored level: output at the size of l0
template<int PX, int PY> DEV void assemble_stored(const float (*sl)[FS][FS + 1], const __half *l0, size_t p0,
    int w0, int x, int y, int bx, int by, __half *out)
{
  const size_t o = (size_t)y * w0 + x;
  const float v = h2f(l0[NG * p0 + o]);
  const float r = assemble_px<PX, PY>([&](int k, float) { return h2f(l0[k * p0 + o]); }, v, sl, x, y, bx, by);
  out[o] = f2h(r);
}

__global__ void __launch_bounds__(256) k_llap_assemble(const __half *__restrict__ coarse, int first,
    const __half *__restrict__ l0, int w0, int h0, size_t p0,
    const __half *__restrict__ l1, int w1, int h1, size_t p1, __half *__restrict__ out)
{
  __shared__ float sl[NPL + 1][FS][FS + 1];
  const int X0 = blockIdx.x * FT, Y0 = blockIdx.y * FT;
  const int bx = X0 / 2 - 2, by = Y0 / 2 - 2;
  stage_coarse(sl, l1, w1, h1, p1, first ? l1 + NG * p1 : coarse, bx, by);
  __syncthreads();
  for(int t = threadIdx.x; t < FT * FT; t += blockDim.x)
  {
    int x, y;
    if(!tile_item(t, X0, Y0, w0, h0, x, y)) continue;
    switch((x & 1) + 2 * (y & 1))
    { // uniform per warp (tile_item hands a warp one parity class)
      case 0: assemble_stored<0, 0>(sl, l0, p0, w0, x, y, bx, by, out); break;
      case 1: assemble_stored<1, 0>(sl, l0, p0, w0, x, y, bx, by, out); break;
      case 2: assemble_stored<0, 1>(sl, l0, p0, w0, x, y, bx, by, out); break;
      default: assemble_stored<1, 1>(sl, l0, p0, w0, x, y, bx, by, out); break;
    }
  }
}

// llap/assemble.comp for level 0, the fine planes recomputed from the
// filmcurv output like llap/curve.comp, fused with llap/colour.comp:141-160
template<int PX, int PY> DEV void final_px(const dev_llap_k3_t &p, const float (*sl)[FS][FS + 1], int x, int y,
    int bx, int by, float r2s, float rden)
{
  float rgb[4];
  ld_half4(p.rgbf + (size_t)y * p.W + x, rgb[0], rgb[1], rgb[2], rgb[3]);
  const float yv = lum2020(gclamp(rgb[0], -1000.0f, 1000.0f), gclamp(rgb[1], -1000.0f, 1000.0f), gclamp(rgb[2], -1000.0f, 1000.0f));
  const float v = f16r(yv);
  float yo_ = f16r(assemble_px<PX, PY>([&](int, float g) {
      return f16r(llap_curve_rcp(yv, g, p.ll_sigma, r2s, rden, p.ll_shadows, p.ll_highlights, p.ll_clarity)); },
    v, sl, x, y, bx, by));
  const float yo = fmaxf(lum2020(rgb[0], rgb[1], rgb[2]), 1e-8f);
  if(yo_ < yo) yo_ = yo * expf(1.0f * (yo_ - yo));
  float o[3];
  for(int k = 0; k < 3; k++) o[k] = fmaxf(0.0f, rgb[k] * yo_ / yo);
  p.out[(size_t)y * p.W + x] = mk_half4(o[0], o[1], o[2], 1.0f);
}

__global__ void __launch_bounds__(256) k_llap_final(const dev_llap_k3_t p)
{
  __shared__ float sl[NPL + 1][FS][FS + 1];
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
    switch((x & 1) + 2 * (y & 1))
    {
      case 0: final_px<0, 0>(p, sl, x, y, bx, by, r2s, rden); break;
      case 1: final_px<1, 0>(p, sl, x, y, bx, by, r2s, rden); break;
      case 2: final_px<0, 1>(p, sl, x, y, bx, by, r2s, rden); break;
      default: final_px<1, 1>(p, sl, x, y, bx, by, r2s, rden); break;
    }
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
