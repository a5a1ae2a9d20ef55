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
#include "develop_px.cuh"
#include "kernels.h"
#include "pixel.cuh"

namespace {

constexpr int RC_CX = 64, RC_CY = 16, RC_H = 4;           // conv tile and halo
constexpr int RF_TX = 64, RF_TY = 32, RF_B = 3;            // fill tile and border (demosaic/config.h)
constexpr int RF_SX = RF_TX - 2 * RF_B, RF_SY = RF_TY - 2 * RF_B;
constexpr int RF_N = RF_TX * RF_TY, RF_PAD = 256;          // reads reach 3 rows + 3 columns past the plane
// the fill kernel's staged inputs, in tile coordinates (0,0 = the tile's first pixel)
constexpr int CF_X0 = -4, CF_W = 72, CF_Y0 = -4, CF_H = 40;   // mosaic, 0 outside the image
constexpr int VH_X0 = -1, VH_W = 66, VH_Y0 = -1, VH_H = 34;   // vh, mirrored
constexpr int HQ_W = 40, HQ_Y0 = -2, HQ_H = 36;               // pq and lp by half index, mirrored

DEV float fadd(float a, float b) { return __fadd_rn(a, b); }
DEV float fsub(float a, float b) { return __fsub_rn(a, b); }
DEV float fmul(float a, float b) { return __fmul_rn(a, b); }
DEV float fdiv(float a, float b) { return __fdiv_rn(a, b); }
DEV float fmixr(float x, float y, float a) { return fadd(fmul(x, fsub(1.0f, a)), fmul(y, a)); }
DEV int mirror_any(int i, int n)
{ // MIRRORED_REPEAT for any i: the tiles compute pixels up to a tile past the image
  if((unsigned)i < (unsigned)n) return i;
  if(i >= -n && i < 2 * n) return i < 0 ? -1 - i : 2 * n - 1 - i;
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  return t < n ? t : m - 1 - t;
}

// demosaic/rcd_conv.comp:8-49. The sums over the three offsets i of the
// shader are sums of one filter response taken at three neighbouring
// positions (a column, a row or a diagonal), so each response is computed
// once per position and shared; every response and every sum is formed in
// the shader's order.
__global__ void __launch_bounds__(256) k_rcd_conv(const dev_rcd_t p)
{
  __shared__ float t[RC_CY + 2 * RC_H][RC_CX + 2 * RC_H + 1];   // mosaic, mirrored, tile +-4
  __shared__ float fv[RC_CY][RC_CX + 2];                        // vertical response, columns -1..64
  __shared__ float fh[RC_CY + 2][RC_CX];                        // horizontal response, rows -1..16
  __shared__ float d1[RC_CY + 2][RC_CX + 2], d2[RC_CY + 2][RC_CX + 2];   // diagonal responses, -1..64 x -1..16
  const int x0 = blockIdx.x * RC_CX, y0 = blockIdx.y * RC_CY, tid = threadIdx.x;
#pragma unroll 4
  for(int i = tid; i < (RC_CY + 2 * RC_H) * (RC_CX + 2 * RC_H); i += 256)
  { // the mosaic through the sampler at texel centres: mirrored
    const int ly = i / (RC_CX + 2 * RC_H), lx = i % (RC_CX + 2 * RC_H);
    const int gx = mirror_any(x0 + lx - RC_H, p.W), gy = mirror_any(y0 + ly - RC_H, p.H);
    t[ly][lx] = h2f(p.cfa[(size_t)gy * p.W + gx]);
  }
  __syncthreads();
  auto c = [&](int x, int y) { return t[y + RC_H][x + RC_H]; };   // tile coordinates
  for(int i = tid; i < RC_CY * (RC_CX + 2); i += 256)
  {
    const int y = i / (RC_CX + 2), x = i % (RC_CX + 2) - 1;
    fv[y][x + 1] = fadd(fsub(fsub(fadd(fsub(fsub(c(x, y - 3), fmul(3.0f, c(x, y - 2))), c(x, y - 1)), fmul(6.0f, c(x, y))), c(x, y + 1)),
                             fmul(3.0f, c(x, y + 2))), c(x, y + 3));
  }
  for(int i = tid; i < (RC_CY + 2) * RC_CX; i += 256)
  {
    const int y = i / RC_CX - 1, x = i % RC_CX;
    fh[y + 1][x] = fadd(fsub(fsub(fadd(fsub(fsub(c(x - 3, y), fmul(3.0f, c(x - 2, y))), c(x - 1, y)), fmul(6.0f, c(x, y))), c(x + 1, y)),
                             fmul(3.0f, c(x + 2, y))), c(x + 3, y));
  }
  for(int i = tid; i < (RC_CY + 2) * (RC_CX + 2); i += 256)
  {
    const int y = i / (RC_CX + 2) - 1, x = i % (RC_CX + 2) - 1;
    if(((x0 + x + y0 + y) & 1) != 0) continue;   // red/blue positions only
    d1[y + 1][x + 1] = fadd(fsub(fadd(fsub(fsub(c(x - 3, y - 3), c(x + 1, y - 1)), c(x + 1, y + 1)), c(x + 3, y + 3)),
                                 fmul(3.0f, fadd(c(x - 2, y - 2), c(x + 2, y + 2)))), fmul(6.0f, c(x, y)));
    d2[y + 1][x + 1] = fadd(fsub(fadd(fsub(fsub(c(x + 3, y - 3), c(x + 1, y - 1)), c(x - 1, y + 1)), c(x - 3, y + 3)),
                                 fmul(3.0f, fadd(c(x + 2, y - 2), c(x - 2, y + 2)))), fmul(6.0f, c(x, y)));
  }
  __syncthreads();
  const int lx = tid % RC_CX, x = x0 + lx;
  if(x >= p.W) return;
  const int hw = p.W / 2;
  for(int ly = tid / RC_CX; ly < RC_CY; ly += 256 / RC_CX)
  {
    const int y = y0 + ly;
    if(y >= p.H) return;
    float s0 = fadd(fadd(fadd(0.0f, fv[ly][lx]), fv[ly][lx + 1]), fv[ly][lx + 2]);
    float s1 = fadd(fadd(fadd(0.0f, fh[ly][lx]), fh[ly + 1][lx]), fh[ly + 2][lx]);
    s0 = fmul(s0, s0); s1 = fmul(s1, s1);
    p.vh[(size_t)y * p.W + x] = f2h(fdiv(s0, fadd(fadd(1e-5f, s0), s1)));
    if(((x + y) & 1) == 0)
    { // red/blue: diagonal discriminator
      float q0 = fadd(fadd(fadd(1e-5f, d1[ly][lx]), d1[ly + 1][lx + 1]), d1[ly + 2][lx + 2]);
      float q1 = fadd(fadd(fadd(1e-5f, d2[ly + 2][lx]), d2[ly + 1][lx + 1]), d2[ly][lx + 2]);
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
          l = fadd(l, fmul((j == 0 ? 1.0f : 0.5f) * (i == 0 ? 1.0f : 0.5f), c(lx + i + off, ly + j)));
      p.lp[(size_t)y * hw + x / 2] = f2h(fmaxf(1e-6f, l));
    }
  }
}

// demosaic/rcd_fill.comp:20-162. 256 threads per tile, each working on the
// pixel pairs of four tile rows; the mosaic, vh, pq and lp the tile reads
// are staged in shared memory first (mirrored or zero filled as the shader
// reads them).
template<bool POST> __global__ void __launch_bounds__(256, 5) k_rcd_fill(const dev_rcd_t p, const dev_image_t d)
{
  __shared__ __half sh[3][RF_PAD + RF_N + RF_PAD];   // shm_r, shm_g, shm_b
  __shared__ uint32_t hist[257];
  __shared__ __half scf[CF_H][CF_W], svh[VH_H][VH_W], spq[HQ_H][HQ_W], slp[HQ_H][HQ_W];
  const int tid = threadIdx.x, lx = tid & 31, ly0 = tid >> 5;
  const int ox = blockIdx.x * RF_SX - RF_B, oy = blockIdx.y * RF_SY - RF_B;   // the tile's first pixel
  const int hw = p.W / 2;
  const int hmin = ((ox - 2) >> 1) - 1;            // below every half index the tile reads
  const __half zero = __float2half_rn(0.0f);
  for(int i = tid; i < RF_PAD; i += 256)
#pragma unroll
    for(int c = 0; c < 3; c++) { sh[c][i] = zero; sh[c][RF_PAD + RF_N + i] = zero; }
  if(POST && d.hist) for(int i = tid; i < 257; i += 256) hist[i] = 0;
#pragma unroll 4
  for(int i = tid; i < CF_H * CF_W; i += 256)
  { // texelFetch of the mosaic: 0 outside
    const int yy = i / CF_W, xx = i % CF_W;
    const int gx = ox + CF_X0 + xx, gy = oy + CF_Y0 + yy;
    scf[yy][xx] = (gx >= 0 && gy >= 0 && gx < p.W && gy < p.H) ? p.cfa[(size_t)gy * p.W + gx] : zero;
  }
#pragma unroll 4
  for(int i = tid; i < VH_H * VH_W; i += 256)
  { // texture() at texel centres: mirrored
    const int yy = i / VH_W, xx = i % VH_W;
    svh[yy][xx] = p.vh[(size_t)mirror_any(oy + VH_Y0 + yy, p.H) * p.W + mirror_any(ox + VH_X0 + xx, p.W)];
  }
#pragma unroll 2
  for(int i = tid; i < HQ_H * HQ_W; i += 256)
  {
    const int yy = i / HQ_W, xx = i % HQ_W;
    const size_t o = (size_t)mirror_any(oy + HQ_Y0 + yy, p.H) * hw + mirror_any(hmin + xx, hw);
    spq[yy][xx] = p.pq[o];
    slp[yy][xx] = p.lp[o];
  }
  __syncthreads();
  // tile coordinates (x, y) -> staged values
  auto cf = [&](int x, int y) { return h2f(scf[y - CF_Y0][x - CF_X0]); };
  auto vhf = [&](int x, int y) { return h2f(svh[y - VH_Y0][x - VH_X0]); };
  auto hq = [&](int x, int y) { const int gx = ox + x, gy = oy + y; return (gx + ((gy & 1) == 1 ? 0 : 1)) / 2 - hmin; };   // truncating division
  auto pqf = [&](int x, int y) { return h2f(spq[y - HQ_Y0][hq(x, y)]); };
  auto lpf = [&](int x, int y) { return h2f(slp[y - HQ_Y0][hq(x, y)]); };
  const float eps = 1e-5f;
#pragma unroll 1
  for(int ly = ly0; ly < RF_TY; ly += 8)
  { // fill the tile, white balanced, f16
#pragma unroll
    for(int k = 0; k < 2; k++)
    {
      const int x = 2 * lx + k;
      const int c = cfa_bayer(ox + x, oy + ly);
      const float v = gclamp(cf(x, ly), 0.0f, 65535.0f);
#pragma unroll
      for(int ch = 0; ch < 3; ch++) sh[ch][RF_PAD + RF_TX * ly + x] = __float2half_rn(c == ch ? fmul(p.wb[ch], v) : 0.0f);
    }
  }
  __syncthreads();
#pragma unroll 1
  for(int ly = ly0; ly < RF_TY; ly += 8)
  { // green at red/blue
    const int k_rb = cfa_bayer(ox + 2 * lx, oy + ly) == 1 ? 1 : 0;   // the red/blue pixel of the pair
    const int x = 2 * lx + k_rb, y = ly;
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
    sh[1][RF_PAD + RF_TX * y + x] = __float2half_rn(fmixr(ve, he, vhd));
  }
  __syncthreads();
#pragma unroll 1
  for(int ly = ly0; ly < RF_TY; ly += 8)
  { // blue at red, red at blue: along the diagonals
    const int k_rb = cfa_bayer(ox + 2 * lx, oy + ly) == 1 ? 1 : 0;
    const int x = 2 * lx + k_rb, y = ly, o = RF_PAD + RF_TX * y + x;
    const bool red = cfa_bayer(ox + x, oy + y) == 0;
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
#pragma unroll 1
  for(int ly = ly0; ly < RF_TY; ly += 8)
  { // red and blue at green; the last stage: only the pixels the tile writes
    const int kg = cfa_bayer(ox + 2 * lx, oy + ly) == 1 ? 0 : 1;
    const int x = 2 * lx + kg, y = ly, o = RF_PAD + RF_TX * y + x;
    if(x < RF_B || y < RF_B || x >= RF_TX - RF_B || y >= RF_TY - RF_B) continue;
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
  // the inner 58x26 pixels, divided by the white balance again (the demosaic output,
  // f16); with POST, colour/main, the histogram and filmcurv/main follow per pixel
#pragma unroll 1
  for(int ly = ly0; ly < RF_TY; ly += 8)
  {
    const int gy = oy + ly;
#pragma unroll
    for(int k = 0; k < 2; k++)
    {
      const int x = 2 * lx + k, gx = ox + x;
      if(x >= RF_B && ly >= RF_B && x < RF_TX - RF_B && ly < RF_TY - RF_B && gx < p.W && gy < p.H)
      {
        const int o = RF_PAD + RF_TX * ly + x;
        const float dm[3] = { f16r(fdiv(h2f(sh[0][o]), p.wb[0])), f16r(fdiv(h2f(sh[1][o]), p.wb[1])),
                              f16r(fdiv(h2f(sh[2][o]), p.wb[2])) };
        if(p.out) p.out[(size_t)gy * p.W + gx] = mk_half4(dm[0], dm[1], dm[2], 1.0f);
        if(POST)
        {
          float co[3], fc[3];
          colour_px(d, dm, co);
          if(d.dbg_colour) d.dbg_colour[(size_t)gy * p.W + gx] = mk_half4(co[0], co[1], co[2], 1.0f);
          if(d.hist)
          {
            const uint32_t bin = hist_bin(co[0], co[1], co[2]);
            if(bin > 0) { atomicAdd(&hist[bin], 1u); atomicAdd(&hist[256], 1u); }
          }
          filmcurv_px(d, co, fc);
          d.rgbf[(size_t)gy * p.W + gx] = mk_half4(fc[0], fc[1], fc[2], 1.0f);
        }
      }
    }
  }
  if(POST && d.hist)
  {
    __syncthreads();
    for(int i = tid; i < 257; i += 256) if(hist[i]) atomicAdd(d.hist + i, hist[i]);
  }
}

} // namespace

cudaError_t launch_rcd(const dev_rcd_t &p, const dev_image_t *post, int stage, cudaStream_t s)
{
  const dim3 gf((p.W + RF_SX - 1) / RF_SX, (p.H + RF_SY - 1) / RF_SY);
  if(stage == 0)
    k_rcd_conv<<<dim3((p.W + RC_CX - 1) / RC_CX, (p.H + RC_CY - 1) / RC_CY), 256, 0, s>>>(p);
  else if(stage == 1 && p.post && post)
    k_rcd_fill<true><<<gf, 256, 0, s>>>(p, *post);
  else if(stage == 1 && !p.post)
  {
    dev_image_t none;
    memset(&none, 0, sizeof(none));
    k_rcd_fill<false><<<gf, 256, 0, s>>>(p, none);
  }
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}
