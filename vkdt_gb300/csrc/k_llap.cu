// llap module kernels (src/pipe/modules/llap): the pyramid reduce and
// assemble levels below level 1 and the final full resolution pass
// (assemble of level 0 fused with llap/colour). Pyramid levels are stored as
// 11 f16 planes (NUM_GAMMA curves + grey) each, planar.
//
// The assemble kernels stage the coarse level (its planes and the coarse
// assembled image) of a 64x16 output tile in shared memory. A thread takes two
// horizontally adjacent outputs (one of each x parity, both centred on the
// same coarse column) and a warp one row of 32 such pairs: the lanes read 32
// consecutive coarse slots (no bank conflicts), the rgba images move as 16
// byte words, and all lanes of a warp evaluate the same tap pattern.
#include "common.cuh"
#include "hilite.cuh"
#include "kernels.h"
#include "pixel.cuh"

#include <cudaTypedefs.h>
#include <cstring>

namespace {

constexpr int NPL = 11;
constexpr int NG = 10;
constexpr int FTX = 64, FTY = 16;              // output tile
constexpr int NKX = FTX / 2;                   // coarse columns the tile's outputs centre on
constexpr int FSX = NKX + 4, FSY = FTY / 2 + 4; // coarse slots: virtual [X0/2-2, X0/2+NKX+2) x [Y0/2-2, Y0/2+FTY/2+2)

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
  for(int i = 1; i < NG - 1; i++) hi += (kLlapGamma[i] <= v) ? 1 : 0;
  return hi;
}

// llap/assemble.comp:54-58 gauss_expand = shared.glsl:99-127 sample_soft at
// (o/2 + 0.5): three bilinear taps per axis at o/2+0.5 + {-1.5, 0, 1.5}, which
// land on texel centres or half way between two. Summed per axis the texel
// weights are (.5 .5 1 .5 .5) around k = o/2 for even o and (1 .5 .5 1) from
// k-1 for odd o; the expand is the separable sum of those, row sums first,
// divided by 9. PX, PY: parities of the output position.
//
// hrow: the row sum for x parity PX around column kx, fetch(x) the texel
template<int PX, class F> DEV float hrow(F fetch, int kx)
{
  constexpr int NX = PX ? 4 : 5, BXO = PX ? -1 : -2;
  float row = 0.0f;
#pragma unroll
  for(int a = 0; a < NX; a++)
  {
    const float w = PX ? ((a == 0 || a == 3) ? 1.0f : 0.5f) : (a == 2 ? 1.0f : 0.5f);
    row += w * fetch(kx + BXO + a);
  }
  return row;
}

// vcol: the sum of the row sums rowsum(y) for y parity PY around row ky, / 9
template<int PY, class R> DEV float vcol(R rowsum, int ky)
{
  constexpr int NY = PY ? 4 : 5, BYO = PY ? -1 : -2;
  float r = 0.0f;
#pragma unroll
  for(int b = 0; b < NY; b++)
  {
    const float wy = PY ? ((b == 0 || b == 3) ? 1.0f : 0.5f) : (b == 2 ? 1.0f : 0.5f);
    r += wy * rowsum(ky + BYO + b);
  }
  return r / 9.0f;
}

// expand of two planes at once (fetch returns both texels as a float2): the
// same sums in the same order as hrow and vcol for each of the two, as paired
// FP32 operations (one instruction for both planes; the weights are powers of
// two, so each fused step rounds only its sum, as the separate ones do)
template<int PX, int PY, class F> DEV float2 expand2(F fetch, int kx, int ky)
{
  constexpr int NX = PX ? 4 : 5, NY = PY ? 4 : 5;
  constexpr int BXO = PX ? -1 : -2, BYO = PY ? -1 : -2;
  float2 r = make_float2(0.0f, 0.0f);
#pragma unroll
  for(int b = 0; b < NY; b++)
  {
    float2 row = make_float2(0.0f, 0.0f);
#pragma unroll
    for(int a = 0; a < NX; a++)
    {
      const float w = PX ? ((a == 0 || a == 3) ? 1.0f : 0.5f) : (a == 2 ? 1.0f : 0.5f);
      row = __ffma2_rn(make_float2(w, w), fetch(kx + BXO + a, ky + BYO + b), row);
    }
    const float wy = PY ? ((b == 0 || b == 3) ? 1.0f : 0.5f) : (b == 2 ? 1.0f : 0.5f);
    r = __ffma2_rn(make_float2(wy, wy), row, r);
  }
  return make_float2(r.x / 9.0f, r.y / 9.0f);
}

// llap/reduce.comp:17-35 (sample_semisoft), the planes of one level. The four
// half-texel bilinear taps are the chain of pair sums scaled once by 1/16, as
// in llap_reduce_px. A CTA makes a 32 x 16 tile of outputs for a group of
// RPG planes (blockIdx.z): per plane it stages the input texels
// [2 OX - 8, 2 OX + 64) x [2 OY - 1, 2 OY + 32) once (the outputs read
// [2 OX - 1, 2 OX + 64); the box starts 16 bytes lower, where a TMA copy may
// start). Where those texels lie inside the level, one thread stages the
// whole box of all the group's planes with a TMA copy (cp.async.bulk.tensor on
// a 3D tensor map over the level: x, y, plane), its completion counted on an
// mbarrier; without a tensor map, asynchronous 4 byte copies. At the level's
// border mirrored single loads (the taps overshoot the input by at most one
// texel). Two plane groups per tile: 29 KB per CTA, 7 CTAs per SM.
constexpr int RT_X = 32, RT_Y = 16, RB_X = 2 * RT_X + 8, RI_Y = 2 * RT_Y + 1, RPG = (NPL + 1) / 2;
constexpr int RB_OFF = 6;                                        // slot of input column 2 OX - 2
constexpr uint32_t RED_BOX_BYTES = RPG * RI_Y * RB_X * sizeof(__half);
// bounded waits: polls of the copy's mbarrier before the CTA gives up (a completed copy takes
// microseconds; this is seconds), and again for the copy to land before the CTA exits
constexpr int TMA_WAIT_POLLS = 1 << 24;

DEV bool mbar_wait(uint32_t bar, int polls)
{
  uint32_t done = 0;
  for(int i = 0; i < polls && !done; i++)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(bar) : "memory");
  return done != 0;
}

__global__ void __launch_bounds__(256, 7) k_llap_reduce(const __grid_constant__ CUtensorMap map, int use_map,
    const __half *__restrict__ in, int iw, int ih, int ipitch, size_t ip,
    __half *__restrict__ out, int ow, int oh, int opitch, size_t op, uint32_t *status)
{
  __shared__ __align__(128) __half t[RPG][RI_Y][RB_X];   // the group's planes at once: every load in flight together
  __shared__ __align__(8) uint64_t bar;
  const int k0 = blockIdx.z * RPG, nk = min(RPG, NPL - k0);
  const int OX = blockIdx.x * RT_X, OY = blockIdx.y * RT_Y;
  const int bx0 = 2 * OX - 8, gx0 = 2 * OX - 2, gy0 = 2 * OY - 1;   // box origin, first texel read
  const bool inside = bx0 >= 0 && gy0 >= 0 && 2 * OX + RB_X - 8 <= iw && gy0 + RI_Y <= ih;
  if(inside && use_map)
  { // one TMA copy of the box (6 planes x 33 rows x 72 texels; planes past the last read as 0)
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar), dst = (uint32_t)__cvta_generic_to_shared(&t[0][0][0]);
    if(threadIdx.x == 0)
    {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(b) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncthreads();
    if(threadIdx.x == 0)
    {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(b), "r"(RED_BOX_BYTES) : "memory");
      asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
                   :: "r"(dst), "l"(reinterpret_cast<uint64_t>(&map)), "r"(bx0), "r"(gy0), "r"(k0), "r"(b) : "memory");
    }
    if(!mbar_wait(b, TMA_WAIT_POLLS))
    { // the copy did not complete: record it, give the copy a last bounded chance to land, leave
      if(threadIdx.x == 0) atomicOr(status, 1u);
      mbar_wait(b, TMA_WAIT_POLLS);
      return;
    }
  }
  else if(inside)
  { // asynchronous 4 byte copies (even texel offsets: the row pitch is a multiple of 8 texels)
    for(int i = threadIdx.x; i < RI_Y * (RB_X / 2 - 3); i += blockDim.x)
    {
      const int r = i / (RB_X / 2 - 3), c = i % (RB_X / 2 - 3);
      const size_t o = (size_t)(gy0 + r) * ipitch + gx0 + 2 * c;
#pragma unroll
      for(int k = 0; k < RPG; k++)
        if(k < nk)
        {
          const unsigned dst = (unsigned)__cvta_generic_to_shared(&t[k][r][RB_OFF + 2 * c]);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" :: "r"(dst), "l"(in + (k0 + k) * ip + o) : "memory");
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
  }
  else
    for(int i = threadIdx.x; i < RI_Y * (RB_X - RB_OFF); i += blockDim.x)
    {
      const int r = i / (RB_X - RB_OFF), c = i % (RB_X - RB_OFF);
      const size_t o = (size_t)mirror1(gy0 + r, ih) * ipitch + mirror1(gx0 + c, iw);
#pragma unroll
      for(int k = 0; k < RPG; k++)
        if(k < nk) t[k][r][RB_OFF + c] = __ldg(in + (k0 + k) * ip + o);
    }
  __syncthreads();
  const int lx = threadIdx.x % RT_X, ly = threadIdx.x / RT_X;
#pragma unroll
  for(int h = 0; h < 2; h++)
  {
    const int oy = OY + ly + 8 * h, ox = OX + lx;
    if(ox >= ow || oy >= oh) continue;
    for(int k = 0; k < nk; k++)
    {
      float P[3][2];
#pragma unroll
      for(int b = 0; b < 3; b++)
      { // input rows 2 oy - 1 + b, columns 2 ox - 1 .. 2 ox + 1
        const __half *row = &t[k][2 * (ly + 8 * h) + b][RB_OFF + 2 * lx + 1];
        const float t0 = h2f(row[0]), t1 = h2f(row[1]), t2 = h2f(row[2]);
        P[b][0] = t0 + t1;
        P[b][1] = t1 + t2;
      }
      out[(k0 + k) * op + (size_t)oy * opitch + ox] =
          f2h(((((P[0][0] + P[1][0]) + (P[0][1] + P[1][1])) + (P[1][0] + P[2][0])) + (P[1][1] + P[2][1])) * 0.0625f);
    }
  }
}

// the coarse level around one output tile: slot (sx, sy) holds the mirrored
// texel (bx+sx, by+sy). An output mixes the two adjacent planes around its
// grey value, so the planes are staged in pairs (k, k+1), one 8 byte word per
// slot (f16 values as floats: exact, one load and no conversion per tap),
// beside the coarse assembled image. The coarse image enters every output, so
// its row sums are made once per tile.
struct coarse_t
{
  float2 pr[NG - 1][FSY][FSX];    // planes (k, k+1), k = 0 .. NG-2
  float c[FSY][FSX];              // the coarse assembled image (the grey plane on the first level)
  float hc[2][FSY][NKX];          // hrow of c for even / odd outputs: [x parity][slot row][column - X0/2]
};

DEV void stage_coarse(coarse_t &sc, const __half *l1, int w1, int h1, int pitch1, size_t p1,
    const __half *coarse, int bx, int by)
{ // the mirrored position once per slot, then the same texel of every plane
  for(int r = threadIdx.x; r < FSX * FSY; r += blockDim.x)
  {
    const int sx = r % FSX, sy = r / FSX;
    const size_t o = (size_t)mirror1(by + sy, h1) * pitch1 + mirror1(bx + sx, w1);
    float h[NG];
#pragma unroll
    for(int k = 0; k < NG; k++) h[k] = h2f(__ldg(l1 + k * p1 + o));
#pragma unroll
    for(int k = 0; k < NG - 1; k++) sc.pr[k][sy][sx] = make_float2(h[k], h[k + 1]);
    sc.c[sy][sx] = h2f(__ldg(coarse + o));
  }
  __syncthreads();
  // coarse column X0/2 + lx sits in slot lx + 2
  for(int i = threadIdx.x; i < 2 * FSY * NKX; i += blockDim.x)
  {
    const int lx = i % NKX, sy = (i / NKX) % FSY, px = i / (NKX * FSY);
    const float *row = sc.c[sy];
    sc.hc[px][sy][lx] = px ? hrow<1>([&](int sx) { return row[sx]; }, lx + 2)
                           : hrow<0>([&](int sx) { return row[sx]; }, lx + 2);
  }
}

// llap/assemble.comp:89-123 at one output of parity (PX, PY) centred on coarse
// column slot lx + 2 and row slot sy. l0(hi, glo, ghi) returns the fine level
// planes hi - 1 and hi (of gamma glo and ghi) at the output.
template<int PX, int PY, class L0> DEV float assemble_px(L0 l0, float v, const coarse_t &sc, int lx, int sy)
{
  const float res = vcol<PY>([&](int iy) { return sc.hc[PX][iy][lx]; }, sy);
  const int hi = gamma_hi_from_v(v);
  const float glo = kLlapGamma[hi - 1], ghi = kLlapGamma[hi];
  const float a = gclamp((v - glo) / (ghi - glo), 0.0f, 1.0f);
  const float2 (*pr)[FSX] = sc.pr[hi - 1];
  const float2 e = expand2<PX, PY>([&](int ix, int iy) { return pr[iy][ix]; }, lx + 2, sy);
  const float2 f = l0(hi, glo, ghi);
  const float la = f.x - e.x;
  const float lb = f.y - e.y;
  return res + la * (1.0f - a) + lb * a;
}

// llap/assemble.comp:89-123 for a stored level: output o at the size of l0
template<int PX, int PY> DEV void assemble_stored(const coarse_t &sl, const __half *l0, size_t p0,
    size_t o, int lx, int sy, __half *out)
{
  const float v = h2f(l0[NG * p0 + o]);
  const float r = assemble_px<PX, PY>([&](int hi, float, float) {
      return make_float2(h2f(l0[(hi - 1) * p0 + o]), h2f(l0[hi * p0 + o])); }, v, sl, lx, sy);
  out[o] = f2h(r);
}

__global__ void __launch_bounds__(256) k_llap_assemble(const __half *__restrict__ coarse, int first,
    const __half *__restrict__ l0, int w0, int h0, int pitch0, size_t p0,
    const __half *__restrict__ l1, int w1, int h1, int pitch1, size_t p1, __half *__restrict__ out)
{
  __shared__ coarse_t sl;
  const int X0 = blockIdx.x * FTX, Y0 = blockIdx.y * FTY;
  stage_coarse(sl, l1, w1, h1, pitch1, p1, first ? l1 + NG * p1 : coarse, X0 / 2 - 2, Y0 / 2 - 2);
  __syncthreads();
  for(int t = threadIdx.x; t < NKX * FTY; t += blockDim.x)
  { // the pair (x, x + 1) of row y; a warp takes one row
    const int lx = t % NKX, ry = t / NKX;
    const int x = X0 + 2 * lx, y = Y0 + ry;
    if(x >= w0 || y >= h0) continue;
    const int sy = (ry >> 1) + 2;
    const size_t o = (size_t)y * pitch0 + x;
    const bool two = x + 1 < w0;
    if(y & 1)
    {
      assemble_stored<0, 1>(sl, l0, p0, o, lx, sy, out);
      if(two) assemble_stored<1, 1>(sl, l0, p0, o + 1, lx, sy, out);
    }
    else
    {
      assemble_stored<0, 0>(sl, l0, p0, o, lx, sy, out);
      if(two) assemble_stored<1, 0>(sl, l0, p0, o + 1, lx, sy, out);
    }
  }
}

// grade/main.comp:23-64 on the llap output (rounded to f16 as the reference
// stores it): lift / gamma / gain / offset per channel, or their zoned form
// weighted by a log luminance; pow and log2 as the accurate functions
DEV void grade_px(const dev_llap_k3_t &p, float rgb[3])
{
  float gain[3], lift[3], gamma[3];
  for(int k = 0; k < 3; k++) { gain[k] = p.gr_gain[k]; lift[k] = p.gr_lift[k]; gamma[k] = p.gr_gamma[k]; }
  if(p.grade == 2)
  {
    float L = 0.0f;
    L = L + fmaxf(rgb[0], 0.0f) * 0.2126f;
    L = L + fmaxf(rgb[1], 0.0f) * 0.7152f;
    L = L + fmaxf(rgb[2], 0.0f) * 0.0722f;
    L = gclamp(0.67f + log2f(fmaxf(L, 1e-6f)) * 0.11f, 0.0f, 1.0f);
    const float sp = gclamp(p.gr_sp, 1e-3f, 1.0f - 1e-3f);
    const float hp = gclamp(p.gr_hp, sp + 1e-3f, 1.0f);
    const float ws = 1.0f - smoothstep(0.0f, sp, L);
    const float wh = smoothstep(hp, 1.0f, L);
    const float wm = 1.0f - ws - wh;
    for(int k = 0; k < 3; k++)
    {
      gain[k] = gmix(1.0f, gain[k], wh);
      lift[k] = lift[k] * ws;
      gamma[k] = gmix(1.0f, gamma[k], wm);
    }
  }
  for(int k = 0; k < 3; k++)
  {
    float v = gain[k] * rgb[k];
    v = v * (1.0f - lift[k]) + lift[k];
    // pow(x, 1) is x: the default gamma (and the mid zone's weight 0) costs no pow
    v = gamma[k] == 1.0f ? fmaxf(v, 0.0f) : powf(fmaxf(v, 0.0f), 1.0f / gamma[k]);
    rgb[k] = v + p.gr_off[k];
  }
}

// llap/assemble.comp for level 0, the fine planes recomputed from the
// filmcurv output like llap/curve.comp, fused with llap/colour.comp:141-160
// (and grade when the graph connects it)
template<int PX, int PY> DEV half4 final_px(const dev_llap_k3_t &p, const coarse_t &sl, const float rgb[3],
    int lx, int sy, float r2s, float rden)
{
  const float yv = lum2020(gclamp(rgb[0], -1000.0f, 1000.0f), gclamp(rgb[1], -1000.0f, 1000.0f), gclamp(rgb[2], -1000.0f, 1000.0f));
  const float v = f16r(yv);
  const bool unit_curve = p.ll_shadows == 1.0f && p.ll_highlights == 1.0f;
  float yo_ = f16r(assemble_px<PX, PY>([&](int, float glo, float ghi) {
      if(unit_curve)
      { // both planes as one pair, as k_post makes the level-0 planes (llap_curve_unit2)
        const float2 X = make_float2(yv, yv);
        const float2 c = __fadd2_rn(X, make_float2(-glo, -ghi));
        const float2 na = __fmul2_rn(__fmul2_rn(c, c), make_float2(-rden, -rden));
        const float2 e = make_float2(curve_exp(na.x), curve_exp(na.y));
        const float2 r = __ffma2_rn(__fmul2_rn(make_float2(p.ll_clarity, p.ll_clarity), c), e, X);
        return make_float2(f16r(r.x), f16r(r.y));
      }
      return make_float2(f16r(llap_curve_rcp(yv, glo, p.ll_sigma, r2s, rden, p.ll_shadows, p.ll_highlights, p.ll_clarity)),
                         f16r(llap_curve_rcp(yv, ghi, p.ll_sigma, r2s, rden, p.ll_shadows, p.ll_highlights, p.ll_clarity))); },
    v, sl, lx, sy));
  // llap/colour.comp: the output luminance over the input's (continuous: the fast exponential and one quotient)
  const float yo = fmaxf(lum2020(rgb[0], rgb[1], rgb[2]), 1e-8f);
  if(yo_ < yo) yo_ = yo * __expf(yo_ - yo);
  const float s = __fdividef(yo_, yo);
  float o[3] = { fmaxf(0.0f, rgb[0] * s), fmaxf(0.0f, rgb[1] * s), fmaxf(0.0f, rgb[2] * s) };
  if(p.grade)
  { // grade reads the llap output as stored (f16)
    for(int k = 0; k < 3; k++) o[k] = f16r(o[k]);
    grade_px(p, o);
  }
  return mk_half4(o[0], o[1], o[2], 1.0f);
}

DEV void unpack_half4(uint2 u, float rgb[3])
{
  const __half2 lo = *reinterpret_cast<const __half2 *>(&u.x), hi = *reinterpret_cast<const __half2 *>(&u.y);
  rgb[0] = __low2float(lo); rgb[1] = __high2float(lo); rgb[2] = __low2float(hi);
}

DEV uint2 pack_half4(half4 h) { return *reinterpret_cast<const uint2 *>(&h); }

__global__ void __launch_bounds__(256, 6) k_llap_final(const dev_llap_k3_t p)
{
  __shared__ coarse_t sl;
  const int X0 = blockIdx.x * FTX, Y0 = blockIdx.y * FTY;
  stage_coarse(sl, p.l1, p.l1w, p.l1h, p.l1pitch, p.l1plane, p.coarse, X0 / 2 - 2, Y0 / 2 - 2);
  __syncthreads();
  const float sig = p.ll_sigma;
  const float r2s = 1.0f / (2.0f * sig), rden = 1.0f / (2.0f * sig * sig / 3.0f);
  // the pair as one 16 byte word where it starts 16 byte aligned in both images (every pair of
  // rows of even length; every other row of odd length, the crop window's 5993 for one)
  const bool vec_base = !((reinterpret_cast<uintptr_t>(p.rgbf) | reinterpret_cast<uintptr_t>(p.out)) & 15);
  for(int t = threadIdx.x; t < NKX * FTY; t += blockDim.x)
  { // the pair (x, x + 1) of row y; a warp takes one row
    const int lx = t % NKX, ry = t / NKX;
    const int x = X0 + 2 * lx, y = Y0 + ry;
    if(x >= p.W || y >= p.H) continue;
    const int sy = (ry >> 1) + 2;
    const size_t o = (size_t)y * p.W + x;
    const bool two = x + 1 < p.W;
    const bool vec = vec_base && two && !(o & 1);
    uint4 u = make_uint4(0u, 0u, 0u, 0u);
    if(vec) u = __ldg(reinterpret_cast<const uint4 *>(p.rgbf + o));
    else
    {
      const uint2 a = __ldg(reinterpret_cast<const uint2 *>(p.rgbf + o));
      u.x = a.x; u.y = a.y;
      if(two) { const uint2 b = __ldg(reinterpret_cast<const uint2 *>(p.rgbf + o + 1)); u.z = b.x; u.w = b.y; }
    }
    float ca[3], cb[3];
    unpack_half4(make_uint2(u.x, u.y), ca);
    unpack_half4(make_uint2(u.z, u.w), cb);
    half4 ha, hb;
    if(y & 1)
    {
      ha = final_px<0, 1>(p, sl, ca, lx, sy, r2s, rden);
      if(two) hb = final_px<1, 1>(p, sl, cb, lx, sy, r2s, rden);
    }
    else
    {
      ha = final_px<0, 0>(p, sl, ca, lx, sy, r2s, rden);
      if(two) hb = final_px<1, 0>(p, sl, cb, lx, sy, r2s, rden);
    }
    if(vec)
    {
      const uint2 a = pack_half4(ha), b = pack_half4(hb);
      *reinterpret_cast<uint4 *>(p.out + o) = make_uint4(a.x, a.y, b.x, b.y);
    }
    else
    {
      p.out[o] = ha;
      if(two) p.out[o + 1] = hb;
    }
  }
}

} // namespace

cudaError_t init_llap()
{ // the reduce stages 6 planes of a tile (26 KB): 8 CTAs per SM with the full carveout;
  // the assemble kernels 36 KB: 6 CTAs per SM
  cudaError_t e = cudaFuncSetAttribute(k_llap_reduce, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if(e == cudaSuccess) e = cudaFuncSetAttribute(k_llap_assemble, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if(e == cudaSuccess) e = cudaFuncSetAttribute(k_llap_final, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  return e;
}

// the 3D tensor map (x, y, plane) over a level's 11 planes that k_llap_reduce stages its
// input boxes through; out of range texels and planes read 0 (the kernel uses none of them)
// the driver's cuTensorMapEncodeTiled, looked up once through the runtime (no link to libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if(!encode)
  {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if(e == cudaSuccess && q == cudaDriverEntryPointSuccess && fn) encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  return encode;
}

cudaError_t llap_reduce_tensor_map(const llap_level_t &in, CUtensorMap *map)
{
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if(!encode) return cudaErrorNotSupported;
  const cuuint64_t dim[3] = { (cuuint64_t)in.w, (cuuint64_t)in.h, (cuuint64_t)NPL };
  const cuuint64_t stride[2] = { (cuuint64_t)in.pitch * sizeof(__half), (cuuint64_t)in.plane * sizeof(__half) };
  const cuuint32_t box[3] = { (cuuint32_t)RB_X, (cuuint32_t)RI_Y, (cuuint32_t)RPG };
  const cuuint32_t estride[3] = { 1, 1, 1 };
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, (void *)in.p, dim, stride, box, estride,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_llap_reduce(const llap_level_t &in, const llap_level_t &out, const CUtensorMap *map,
    uint32_t *status, cudaStream_t s)
{
  dim3 grid((out.w + RT_X - 1) / RT_X, (out.h + RT_Y - 1) / RT_Y, (NPL + RPG - 1) / RPG);
  CUtensorMap none;
  memset(&none, 0, sizeof(none));
  k_llap_reduce<<<grid, 256, 0, s>>>(map ? *map : none, map ? 1 : 0, in.p, in.w, in.h, in.pitch, in.plane,
                                     out.p, out.w, out.h, out.pitch, out.plane, status);
  return cudaGetLastError();
}

cudaError_t launch_llap_assemble(const __half *coarse, int first, const llap_level_t &l0, const llap_level_t &l1,
    __half *out, cudaStream_t s)
{
  dim3 grid((l0.w + FTX - 1) / FTX, (l0.h + FTY - 1) / FTY);
  k_llap_assemble<<<grid, 256, 0, s>>>(coarse, first, l0.p, l0.w, l0.h, l0.pitch, l0.plane,
                                       l1.p, l1.w, l1.h, l1.pitch, l1.plane, out);
  return cudaGetLastError();
}

cudaError_t launch_llap_final(const dev_llap_k3_t &p, cudaStream_t s)
{
  dim3 grid((p.W + FTX - 1) / FTX, (p.H + FTY - 1) / FTY);
  k_llap_final<<<grid, 256, 0, s>>>(p);
  return cudaGetLastError();
}
