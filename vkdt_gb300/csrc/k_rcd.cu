// Demosaic by ratio corrected directional interpolation (RCD, demosaic
// method 1, the default of vkdt's raw video graphs): demosaic/rcd_conv.comp
// and demosaic/rcd_fill.comp on the bayer output of hilite/doub.
//
// k_rcd_conv: per pixel the vertical/horizontal discriminator (full size),
// per red/blue pixel the diagonal one and per green pixel the low pass of its
// red/blue neighbour (half width images), from a mirrored shared tile.
//
// k_rcd_fill: one CTA of 32x32 threads per 64x32 tile, stepping 58x26 as the
// reference's workgroups do (demosaic/config.h): the tile geometry is part of
// the result, because the reference interpolates with a border of 3 while its
// last two stages each read 3 pixels out, so the pixels near a tile seam see
// neighbours that the tile computed from a truncated neighbourhood. The three
// f16 planes of the tile are indexed linearly like the shader's shared
// arrays (an offset past a tile edge wraps into the adjacent row) and are
// padded with zeros, which is what the rows outside the arrays read (the
// reference leaves those reads undefined; the oracle reads 0 as well).
//
// All arithmetic is IEEE single precision in the shader's order
// (__fadd_rn/__fmul_rn/__fdiv_rn, no contraction) and the shader's f16
// operations are f16 operations (__hsub), so the output equals the oracle's
// bit for bit.
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int RC_CX = 64, RC_CY = 16, RC_H = 4;           // conv tile and halo
constexpr int RF_TX = 64, RF_TY = 32, RF_B = 3;            // fill tile and border (demosaic/config.h)
constexpr int RF_SX = RF_TX - 2 * RF_B, RF_SY = RF_TY - 2 * RF_B;
constexpr int RF_N = RF_TX * RF_TY, RF_PAD = 256;          // reads reach 3 rows + 3 columns past the plane

DEV float fadd(float a, float b) { return __fadd_rn(a, b); }
DEV float fsub(float a, float b) { return __fsub_rn(a, b); }
DEV float fmul(float a, float b) { return __fmul_rn(a, b); }
DEV float fdiv(float a, float b) { return __fdiv_rn(a, b); }
DEV float fmixr(float x, float y, float a) { return fadd(fmul(x, fsub(1.0f, a)), fmul(y, a)); }
DEV int mirror_any(int i, int n)
{ // MIRRORED_REPEAT for any i: the tiles compute pixels up to a tile past the image
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  return t < n ? t : m - 1 - t;
}

// demosaic/rcd_conv.comp:8-49
__global__ void __launch_bounds__(256) k_rcd_conv(const dev_rcd_t p)
{
  __shared__ float t[RC_CY + 2 * RC_H][RC_CX + 2 * RC_H + 1];
  const int x0 = blockIdx.x * RC_CX, y0 = blockIdx.y * RC_CY;
  for(int i = threadIdx.x; i < (RC_CY + 2 * RC_H) * (RC_CX + 2 * RC_H); i += 256)
  { // the mosaic through the sampler at texel centres: mirrored
    const int ly = i / (RC_CX + 2 * RC_H), lx = i % (RC_CX + 2 * RC_H);
    const int gx = mirror_any(x0 + lx - RC_H, p.W), gy = mirror_any(y0 + ly - RC_H, p.H);
    t[ly][lx] = h2f(p.cfa[(size_t)gy * p.W + gx]);
  }
  __syncthreads();
  const int lx = threadIdx.x % RC_CX, x = x0 + lx;
  if(x >= p.W) return;
  const int hw = p.W / 2;
  for(int ly = threadIdx.x / RC_CX; ly < RC_CY; ly += 256 / RC_CX)
  {
    const int y = y0 + ly;
    if(y >= p.H) return;
    auto c = [&](int i, int j) { return t[ly + RC_H + j][lx + RC_H + i]; };
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for(int i = -1; i <= 1; i++)
    {
      float a = fadd(fsub(fsub(fadd(fsub(fsub(c(i, -3), fmul(3.0f, c(i, -2))), c(i, -1)), fmul(6.0f, c(i, 0))), c(i, 1)), fmul(3.0f, c(i, 2))), c(i, 3));
      float b = fadd(fsub(fsub(fadd(fsub(fsub(c(-3, i), fmul(3.0f, c(-2, i))), c(-1, i)), fmul(6.0f, c(0, i))), c(1, i)), fmul(3.0f, c(2, i))), c(3, i));
      s0 = fadd(s0, a); s1 = fadd(s1, b);
    }
    s0 = fmul(s0, s0); s1 = fmul(s1, s1);
    p.vh[(size_t)y * p.W + x] = f2h(fdiv(s0, fadd(fadd(1e-5f, s0), s1)));
    if(((x + y) & 1) == 0)
    { // red/blue: diagonal discriminator
      float q0 = 1e-5f, q1 = 1e-5f;
#pragma unroll
      for(int i = -1; i <= 1; i++)
      {
        q0 = fadd(q0, fadd(fsub(fadd(fsub(fsub(c(-3 + i, -3 + i), c(1 + i, -1 + i)), c(1 + i, 1 + i)), c(3 + i, 3 + i)),
                                fmul(3.0f, fadd(c(-2 + i, -2 + i), c(2 + i, 2 + i)))), fmul(6.0f, c(i, i))));
        q1 = fadd(q1, fadd(fsub(fadd(fsub(fsub(c(3 + i, -3 - i), c(1 + i, -1 - i)), c(-1 + i, 1 - i)), c(-3 + i, 3 - i)),
                                fmul(3.0f, fadd(c(2 + i, -2 - i), c(-2 + i, 2 - i)))), fmul(6.0f, c(i, -i))));
      }
      q0 = fmul(q0, q0); q1 = fmul(q1, q1);
      p.pq[(size_t)y * hw + x / 2] = f2h(fdiv(q0, fadd(q0, q1)));
    }
    else
    { // green: 3x3 low pass (weights .5 1 .5 in each direction) around the red/blue neighbour of the row
      const int off = (x & 1) ? -1 : 1;
      float l = 0.0f;
#pragma unroll
      for(int j = -1; j <= 1; j++)
#pragma unroll
        for(int i = -1; i <= 1; i++)
          l = fadd(l, fmul((j == 0 ? 1.0f : 0.5f) * (i == 0 ? 1.0f : 0.5f), c(i + off, j)));
      p.lp[(size_t)y * hw + x / 2] = f2h(fmaxf(1e-6f, l));
    }
  }
}

// demosaic/rcd_fill.comp:20-162
__global__ void __launch_bounds__(1024) k_rcd_fill(const dev_rcd_t p)
{
  __shared__ __half sh[3][RF_PAD + RF_N + RF_PAD];   // shm_r, shm_g, shm_b
  const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * 32 + lx;
  for(int i = tid; i < RF_PAD; i += 1024)
#pragma unroll
    for(int c = 0; c < 3; c++) { sh[c][i] = __float2half_rn(0.0f); sh[c][RF_PAD + RF_N + i] = __float2half_rn(0.0f); }
  const int ix = blockIdx.x * RF_SX + 2 * lx - RF_B, iy = blockIdx.y * RF_SY + ly - RF_B;   // ipos
  const int base = RF_PAD + RF_TX * ly + 2 * lx;
  const int hw = p.W / 2;
  auto cf = [&](int x, int y) -> float {   // texelFetch of the mosaic, 0 outside
    return (x < 0 || y < 0 || x >= p.W || y >= p.H) ? 0.0f : h2f(p.cfa[(size_t)y * p.W + x]);
  };
  auto vhf = [&](int x, int y) { return h2f(p.vh[(size_t)mirror_any(y, p.H) * p.W + mirror_any(x, p.W)]); };
  auto hidx = [&](int x, int y) { return mirror_any((x + ((y & 1) == 1 ? 0 : 1)) / 2, hw); };   // truncating division
  auto pqf = [&](int x, int y) { return h2f(p.pq[(size_t)mirror_any(y, p.H) * hw + hidx(x, y)]); };
  auto lpf = [&](int x, int y) { return h2f(p.lp[(size_t)mirror_any(y, p.H) * hw + hidx(x, y)]); };
  const float eps = 1e-5f;
  { // fill the tile, white balanced, f16
#pragma unroll
    for(int k = 0; k < 2; k++)
    {
      const int c = cfa_bayer(ix + k, iy);
      const float v = gclamp(cf(ix + k, iy), 0.0f, 65535.0f);
#pragma unroll
      for(int ch = 0; ch < 3; ch++) sh[ch][base + k] = __float2half_rn(c == ch ? fmul(p.wb[ch], v) : 0.0f);
    }
  }
  __syncthreads();
  const int k_rb = cfa_bayer(ix, iy) == 1 ? 1 : 0;   // the red/blue pixel of the pair
  { // green at red/blue
    const int x = ix + k_rb, y = iy;
    const float vhc = vhf(x, y);
    const float vhn = fmul(0.25f, fadd(fadd(fadd(vhf(x - 1, y - 1), vhf(x + 1, y - 1)), vhf(x - 1, y + 1)), vhf(x + 1, y + 1)));
    const float vhd = fabsf(fsub(0.5f, vhc)) < fabsf(fsub(0.5f, vhn)) ? vhn : vhc;
    const float cn1 = cf(x, y - 1), cs1 = cf(x, y + 1), cw1 = cf(x - 1, y), ce1 = cf(x + 1, y), c0 = cf(x, y);
    const float cn2 = cf(x, y - 2), cs2 = cf(x, y + 2), cw2 = cf(x - 2, y), ce2 = cf(x + 2, y);
    const float Ng = fadd(fadd(fadd(fadd(eps, fabsf(fsub(cn1, cs1))), fabsf(fsub(c0, cn2))), fabsf(fsub(cn1, cf(x, y - 3)))), fabsf(fsub(cn2, cf(x, y - 4))));
    const float Sg = fadd(fadd(fadd(fadd(eps, fabsf(fsub(cn1, cs1))), fabsf(fsub(c0, cs2))), fabsf(fsub(cs1, cf(x, y + 3)))), fabsf(fsub(cs2, cf(x, y + 4))));
    const float Wg = fadd(fadd(fadd(fadd(eps, fabsf(fsub(cw1, ce1))), fabsf(fsub(c0, cw2))), fabsf(fsub(cw1, cf(x - 3, y)))), fabsf(fsub(cw2, cf(x - 4, y))));
    const float Eg = fadd(fadd(fadd(fadd(eps, fabsf(fsub(cw1, ce1))), fabsf(fsub(c0, ce2))), fabsf(fsub(ce1, cf(x + 3, y)))), fabsf(fsub(ce2, cf(x + 4, y))));
    const float l0 = lpf(x, y);
    const float Ne = fdiv(fmul(fmul(cn1, 2.0f), l0), fadd(fadd(eps, l0), lpf(x, y - 2)));
    const float Se = fdiv(fmul(fmul(cs1, 2.0f), l0), fadd(fadd(eps, l0), lpf(x, y + 2)));
    const float We = fdiv(fmul(fmul(cw1, 2.0f), l0), fadd(fadd(eps, l0), lpf(x - 2, y)));
    const float Ee = fdiv(fmul(fmul(ce1, 2.0f), l0), fadd(fadd(eps, l0), lpf(x + 2, y)));
    const float ve = gclamp(fdiv(fadd(fmul(Sg, Ne), fmul(Ng, Se)), fadd(Ng, Sg)), 0.0f, 65534.0f);
    const float he = gclamp(fdiv(fadd(fmul(Wg, Ee), fmul(Eg, We)), fadd(Eg, Wg)), 0.0f, 65534.0f);
    sh[1][base + k_rb] = __float2half_rn(fmixr(ve, he, vhd));
  }
  __syncthreads();
  { // blue at red, red at blue: along the diagonals
    const int x = ix + k_rb, y = iy, o = base + k_rb;
    const bool red = cfa_bayer(x, y) == 0;
    const __half *sc = sh[red ? 2 : 0], *sg = sh[1];
    auto S = [&](const __half *a, int dx, int dy) { return a[o + RF_TX * dy + dx]; };
    auto hd = [&](__half a, __half b) { return __half2float(__habs(__hsub(a, b))); };
    const float pqc = pqf(x, y);
    const float pqn = fmul(0.25f, fadd(fadd(fadd(pqf(x - 1, y - 1), pqf(x + 1, y - 1)), pqf(x - 1, y + 1)), pqf(x + 1, y + 1)));
    const float pqd = fabsf(fsub(0.5f, pqc)) < fabsf(fsub(0.5f, pqn)) ? pqn : pqc;
    const __half g0 = S(sg, 0, 0);
    const __half cnw = S(sc, -1, -1), cne = S(sc, 1, -1), csw = S(sc, -1, 1), cse = S(sc, 1, 1);
    const float NWg = fadd(fadd(fadd(eps, hd(cnw, cse)), hd(cnw, S(sc, -3, -3))), hd(g0, S(sg, -2, -2)));
    const float NEg = fadd(fadd(fadd(eps, hd(cne, csw)), hd(cne, S(sc, 3, -3))), hd(g0, S(sg, 2, -2)));
    const float SWg = fadd(fadd(fadd(eps, hd(cne, csw)), hd(csw, S(sc, -3, 3))), hd(g0, S(sg, -2, 2)));
    const float SEg = fadd(fadd(fadd(eps, hd(cnw, cse)), hd(cse, S(sc, 3, 3))), hd(g0, S(sg, 2, 2)));
    const float NWe = __half2float(__hsub(cnw, S(sg, -1, -1))), NEe = __half2float(__hsub(cne, S(sg, 1, -1)));
    const float SWe = __half2float(__hsub(csw, S(sg, -1, 1))), SEe = __half2float(__hsub(cse, S(sg, 1, 1)));
    const float pe = fdiv(fadd(fmul(NWg, SEe), fmul(SEg, NWe)), fadd(NWg, SEg));
    const float qe = fdiv(fadd(fmul(NEg, SWe), fmul(SWg, NEe)), fadd(NEg, SWg));
    sh[red ? 2 : 0][o] = __float2half_rn(gclamp(fadd(__half2float(g0), fmixr(pe, qe, pqd)), 0.0f, 65535.0f));
  }
  __syncthreads();
  { // red and blue at green
    const int kg = 1 - k_rb, x = ix + kg, y = iy, o = base + kg;
    const __half *sg = sh[1];
    auto S = [&](const __half *a, int dx, int dy) { return a[o + RF_TX * dy + dx]; };
    auto hd = [&](__half a, __half b) { return __half2float(__habs(__hsub(a, b))); };
    const float vhc = vhf(x, y);
    const float vhn = fmul(0.25f, fadd(fadd(fadd(vhf(x - 1, y - 1), vhf(x + 1, y - 1)), vhf(x - 1, y + 1)), vhf(x + 1, y + 1)));
    const float vhd = fabsf(fsub(0.5f, vhc)) < fabsf(fsub(0.5f, vhn)) ? vhn : vhc;
    const __half g0 = S(sg, 0, 0);
    const float N1 = fadd(eps, hd(g0, S(sg, 0, -2))), S1 = fadd(eps, hd(g0, S(sg, 0, 2)));
    const float W1 = fadd(eps, hd(g0, S(sg, -2, 0))), E1 = fadd(eps, hd(g0, S(sg, 2, 0)));
    float res[2];
#pragma unroll
    for(int c = 0; c < 2; c++)
    {
      const __half *sc = sh[c == 0 ? 0 : 2];
      const __half cn = S(sc, 0, -1), cs = S(sc, 0, 1), cw = S(sc, -1, 0), ce = S(sc, 1, 0);
      const float SN = hd(cn, cs), EW = hd(cw, ce);
      const float Ng = fadd(fadd(N1, SN), hd(cn, S(sc, 0, -3)));
      const float Sg = fadd(fadd(S1, SN), hd(cs, S(sc, 0, 3)));
      const float Wg = fadd(fadd(W1, EW), hd(cw, S(sc, -3, 0)));
      const float Eg = fadd(fadd(E1, EW), hd(ce, S(sc, 3, 0)));
      const float Ne = __half2float(__hsub(cn, S(sg, 0, -1))), Se = __half2float(__hsub(cs, S(sg, 0, 1)));
      const float We = __half2float(__hsub(cw, S(sg, -1, 0))), Ee = __half2float(__hsub(ce, S(sg, 1, 0)));
      const float ve = fdiv(fadd(fmul(Ng, Se), fmul(Sg, Ne)), fadd(Ng, Sg));
      const float he = fdiv(fadd(fmul(Eg, We), fmul(Wg, Ee)), fadd(Eg, Wg));
      res[c] = gclamp(fadd(__half2float(g0), fmixr(ve, he, vhd)), 0.0f, 65535.0f);
      // the shader stores red before it computes blue; blue reads no red of this pixel
      if(c == 0) sh[0][o] = __float2half_rn(res[0]);
    }
    sh[2][o] = __float2half_rn(res[1]);
  }
  __syncthreads();
  // the inner 58x26 pixels, divided by the white balance again
#pragma unroll
  for(int k = 0; k < 2; k++)
  {
    const int gx = ix + k, lxx = 2 * lx + k;
    if(lxx >= RF_B && ly >= RF_B && lxx < RF_TX - RF_B && ly < RF_TY - RF_B && gx < p.W && iy < p.H)
    {
      const int o = base + k;
      p.out[(size_t)iy * p.W + gx] = mk_half4(fdiv(h2f(sh[0][o]), p.wb[0]), fdiv(h2f(sh[1][o]), p.wb[1]),
                                              fdiv(h2f(sh[2][o]), p.wb[2]), 1.0f);
    }
  }
}

} // namespace

cudaError_t launch_rcd(const dev_rcd_t &p, int stage, cudaStream_t s)
{
  if(stage == 0)
    k_rcd_conv<<<dim3((p.W + RC_CX - 1) / RC_CX, (p.H + RC_CY - 1) / RC_CY), 256, 0, s>>>(p);
  else if(stage == 1)
    k_rcd_fill<<<dim3((p.W + RF_SX - 1) / RF_SX, (p.H + RF_SY - 1) / RF_SY), dim3(32, 32), 0, s>>>(p);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}
