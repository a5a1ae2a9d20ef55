// The fused full resolution pass of the path (bayer):
//   hilite/doub (with the level 0 hilite/assemble and denoise/noop recomputed
//   from the mosaic) -> demosaic/gauss -> demosaic/splat -> demosaic/fix ->
//   colour/main -> [OpenDRT/hist] -> filmcurv/main -> llap/curve -> the first
//   llap/reduce level.
// Every intermediate image the reference stores (all f16) is rounded to f16
// at the same point here, but lives only in shared memory. HBM sees the u16
// mosaic in, the filmcurv output (rgba f16, needed by llap/colour) and the 11
// level 1 planes of the llap pyramid out.
//
// A crop after demosaic that moves the image by whole texels (crop/main.comp
// fetching texel (x + dx, y + dy) for every output pixel: no rotation, the
// untouched quad) is applied on the way out: the colour, histogram and
// filmcurv outputs of the window's pixels are written at crop coordinates. The
// llap levels then belong to the cropped image, whose tiles do not align with
// these (an odd shift moves them off the CFA blocks): with a crop the kernel
// ends at filmcurv and the llap curve and first reduce run on its output.
//
// Staging: an interior tile's mosaic window (48 x 40 codes from 16 bytes left
// of its 4 pixel halo) arrives by one TMA copy (cp.async.bulk.tensor on a 2D
// tensor map over the mosaic, completion on an mbarrier) while the CTA loads
// the hilite coarse level; border tiles and mosaics the map cannot describe
// read the codes with plain loads.
//
// Tiling: one CTA computes a TX x TY tile of output pixels. Every stage is
// evaluated on the halo its consumer needs (slots indexed by "virtual"
// positions that hold the value of the mirrored real position, which is what
// a MIRRORED_REPEAT texture read returns). The last tile of a row/column is
// shifted inwards so that the 6 pixel wrap of demosaic/splat.comp:153-156
// always lands inside the tile's slots; outputs are written by the owner only.
//
// Work mapping: the per pixel stages (splat, fix and everything after) hand
// a warp pixels of one CFA phase, so the colour dependent branches of the
// shaders are uniform in a warp; the shared arrays those stages read with a
// stride of two pixels are stored split by x parity (no bank conflicts).
//
// Gaussian weights of demosaic/splat and demosaic/fix: the eigenvectors of
// the bayer covariance are snapped to the axes (gauss.comp:72-73), so per
// covariance entry the weight exp(-0.5 dot(E o / eval, E o)) takes only the
// values for dot = 0, 1/e0, 1/e1, 1/e0 + 1/e1 (E o has entries in {-1,0,1}).
// They are computed once per entry with the same operations as the shader
// (the products by +-1 and 0 are exact), so the weights are bit identical.
#include "common.cuh"
#include "hilite.cuh"
#include "kernels.h"
#include "pixel.cuh"
#include "develop_px.cuh"
#include "gauss.cuh"

#include <cstring>

namespace {

constexpr int TX = 32, TY = 32;
constexpr int NT = 256;
constexpr int MB = TX / 2 + 4;       // hilite output mosaic: virtual blocks [X0/2-2, X0/2+TX/2+2)
constexpr int MX = 2 * MB;           // pixel slots per side (virtual [X0-4, X0+TX+4))
constexpr int CX = TX / 2 + 2;       // demosaic/gauss: half positions [X0/2-1, X0/2+TX/2+1)
constexpr int GX = TX + 3;           // demosaic/splat: virtual [X0-2, X0+TX+1)
constexpr int GH = (GX + 1) / 2;
constexpr int LX = TX + 1;           // llap level 0: virtual [X0-1, X0+TX)
constexpr int LH = (LX + 1) / 2;
constexpr int BX = TX / 4 + 6;       // hilite coarse level slots
constexpr int NPL = 11;              // NUM_GAMMA curves + grey (llap/config.h:2)

constexpr int RAW_X = MX + 8, RAW_Y = MX;   // TMA box of mosaic codes: [X0-8, X0+TX+8) x [Y0-4, Y0+TY+4)
constexpr uint32_t RAW_BYTES = RAW_X * RAW_Y * sizeof(uint16_t);
struct early_t
{
  float sw[3][CX][CX];         // splat weights, same taps as fw
  float B1[3][BX][BX];         // hilite coarse level (rgb) around the tile
  // the mosaic codes of the tile's window (interior tiles with a tensor map), 128 byte aligned
  // inside this array (the dynamic shared memory base is only known to be 16 byte aligned)
  uint16_t raw[RAW_Y * RAW_X + 64];
};
struct smem_t
{
  float M[MX][2][MB];          // hilite output mosaic, [y][x&1][x>>1]
  float fw[3][CX][CX];         // fix weights of the taps (+-1,0), (0,+-1), (+-1,+-1)
  __half g[GX][2][GH];         // splat output (f16 values), [y][x&1][x>>1]
  float rg[GX][2][GH];         // 1 / (1e-4 + splat output)
  uint32_t hist[257];
  uint64_t bar;                // completion of the mosaic window's TMA copy
  union
  { // the llap level 0 planes are written after the last reads of the others
    early_t e;
    struct
    {
      __half2 p[LLAP_PAIRS][LX][2][LH]; // the curve planes in pairs, [y][x & 1][x >> 1]
      __half g[LX][LX + 1];             // the grey plane, [y][slot] (rows of an even length)
    } L0;
  } u;
};
// without the llap level 0 planes (the kernel ends at filmcurv)
constexpr size_t SMEM_NO_L1 = offsetof(smem_t, u) + sizeof(early_t);

DEV int mirror1(int i, int n)
{ // mirrored repeat for |overshoot| < n, clamped for slots no pixel reads
  if(i < 0) i = -1 - i;
  if(i >= n) i = 2 * n - 1 - i;
  return min(max(i, 0), n - 1);
}

// weight of a 3x3 tap from the per covariance table (h: (+-1,0), v: (0,+-1), d: diagonal)
DEV float tap_weight(float wh, float wv, float wd, int i, int j)
{
  return (i == 0 && j == 0) ? 1.0f : (i == 0 ? wv : (j == 0 ? wh : wd));
}

// demosaic/splat.comp:224-266 taps of one output pixel whose CFA phase is (PX, PY):
// only the greens enter rgb.ggg; taps past the border wrap by the CFA period 6
template<int PX, int PY> DEV void splat_taps(const smem_t &s, int qx, int qy, int W, int H, int X0, int Y0,
    float wh, float wv, float wd, float &rg, float &wg)
{
#pragma unroll
  for(int j = -1; j <= 1; j++)
#pragma unroll
  for(int ii = -1; ii <= 1; ii++)
  {
    if(cfa_bayer(PX + ii, PY + j) != 1) continue;
    int px = qx + ii, py = qy + j;
    if(px < 0) px += 6;
    if(py < 0) py += 6;
    if(px >= W) px -= 6;
    if(py >= H) py -= 6;
    const int mx = px - (X0 - 4), my = py - (Y0 - 4);
    const float col = s.M[my][mx & 1][mx >> 1];
    const float weight = (ii == 0 && j == 0) ? 666.0f : tap_weight(wh, wv, wd, ii, j);
    rg += col * weight;
    wg += weight;
  }
}

// demosaic/fix.comp:99-135 taps of one output pixel whose CFA phase is (PX, PY)
template<int PX, int PY> DEV void fix_taps(const smem_t &s, int px, int py, int gx0, int gy0, int X0, int Y0,
    float gc, float wh, float wv, float wd, float &rr, float &rb, float &wr, float &wb, float &rg, float &wg)
{
#pragma unroll
  for(int j = -1; j <= 1; j++)
#pragma unroll
  for(int ii = -1; ii <= 1; ii++)
  {
    const int c = cfa_bayer(PX + ii, PY + j);
    if(c == 1) { rg = gc; wg = 1.0f; continue; }
    const int gx = gx0 + ii, gy = gy0 + j;
    const float rgh = s.rg[gy][gx & 1][gx >> 1];
    const int mx = px + ii - (X0 - 4), my = py + j - (Y0 - 4);
    const float col = s.M[my][mx & 1][mx >> 1];
    const float weight = tap_weight(wh, wv, wd, ii, j);
    // col * (1e-4 + gc) / (1e-4 + gh) * weight with the reciprocal of the splat stage
    const float v = col * (1e-4f + gc) * rgh * weight;
    if(c == 0) { rr += v; wr += weight; }
    else       { rb += v; wb += weight; }
  }
}

// Interior tiles (the tile and its 4 pixel halo inside the image, no mirrored
// or wrapped position anywhere): the tile origin is even, so a slot's parity
// is its pixel's CFA phase, and every tap is a fixed offset from the slot in
// the split arrays. The same taps, weights and sums in the same order as
// splat_taps / fix_taps, with the slot addresses resolved at compile time.
//
// splat slot (2 bx + PX, 2 by + PY): pixel X0 - 2 + sgx, M slot x = sgx + 2 + ii
template<int PX, int PY> DEV void splat_taps_in(const smem_t &s, int bx, int sgy,
    float wh, float wv, float wd, float &rg, float &wg)
{
#pragma unroll
  for(int j = -1; j <= 1; j++)
#pragma unroll
  for(int ii = -1; ii <= 1; ii++)
  {
    if(cfa_bayer(PX + ii, PY + j) != 1) continue;
    const float col = s.M[sgy + 2 + j][(PX + ii) & 1][bx + ((PX + 2 + ii) >> 1)];
    const float weight = (ii == 0 && j == 0) ? 666.0f : tap_weight(wh, wv, wd, ii, j);
    rg += col * weight;
    wg += weight;
  }
}

// fix slot (2 bx + 1 - PX, sly) of a pixel with CFA phase (PX, PY): pixel
// X0 - 1 + slx, splat slot x = slx + 1 + ii, M slot x = slx + 3 + ii
template<int PX, int PY> DEV void fix_taps_in(const smem_t &s, int bx, int sly,
    float gc, float wh, float wv, float wd, float &rr, float &rb, float &wr, float &wb, float &rg, float &wg)
{
#pragma unroll
  for(int j = -1; j <= 1; j++)
#pragma unroll
  for(int ii = -1; ii <= 1; ii++)
  {
    const int c = cfa_bayer(PX + ii, PY + j);
    if(c == 1) { rg = gc; wg = 1.0f; continue; }
    const float rgh = s.rg[sly + 1 + j][(2 - PX + ii) & 1][bx + ((2 - PX + ii) >> 1)];
    const float col = s.M[sly + 3 + j][(PX + ii) & 1][bx + ((4 - PX + ii) >> 1)];
    const float weight = tap_weight(wh, wv, wd, ii, j);
    const float v = col * (1e-4f + gc) * rgh * weight;
    if(c == 0) { rr += v; wr += weight; }
    else       { rb += v; wb += weight; }
  }
}

// The tiles whose stages see no mirrored or wrapped position (even origin, a 4
// pixel margin to every image edge) form the rectangle of tile indices
// [ix0, ix1] x [iy0, iy1]; the interior kernel runs those, the border kernel the
// ring around them (two specialisations: each keeps only its own tap code).
struct tiles_t { int nx, ny, ix0, ix1, iy0, iy1; };

template<bool INTERIOR> DEV void tile_of(const tiles_t &t, int &bx, int &by)
{
  if(INTERIOR) { bx = t.ix0 + (int)blockIdx.x; by = t.iy0 + (int)blockIdx.y; return; }
  // the ring, one CTA per tile: the rows above and below the interior, then the columns beside it
  int i = blockIdx.x;
  const int top = t.iy0 * t.nx, bot = (t.ny - 1 - t.iy1) * t.nx;
  if(i < top) { bx = i % t.nx; by = i / t.nx; return; }
  i -= top;
  if(i < bot) { bx = i % t.nx; by = t.iy1 + 1 + i / t.nx; return; }
  i -= bot;
  const int left = t.ix0, side = t.ix0 + (t.nx - 1 - t.ix1);
  by = t.iy0 + i / side;
  const int k = i % side;
  bx = k < left ? k : t.ix1 + 1 + (k - left);
}

// bounded wait on an mbarrier's phase 0 (polls; a completed copy takes microseconds, this is seconds)
constexpr int TMA_WAIT_POLLS = 1 << 24;
DEV bool mbar_wait(uint32_t bar, int polls)
{
  uint32_t done = 0;
  for(int i = 0; i < polls && !done; i++)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(bar) : "memory");
  return done != 0;
}

// CTAs per SM the register budget is cut for: 5 with the llap planes (their shared memory allows
// no more), VKDT_DEVELOP_CTAS_NO_L1 without them (shared memory allows 7)
#ifndef VKDT_DEVELOP_CTAS_NO_L1
#define VKDT_DEVELOP_CTAS_NO_L1 6
#endif
template<bool INTERIOR, bool L1> __global__ void __launch_bounds__(NT, L1 ? 5 : VKDT_DEVELOP_CTAS_NO_L1) k_develop(const dev_image_t p, const tiles_t tiles,
    const __grid_constant__ CUtensorMap mmap, int use_map, uint32_t *status)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  smem_t &s = *reinterpret_cast<smem_t *>(smem_raw);
  const int tid = threadIdx.x;
  const int W = p.W, H = p.H, hw = W / 2, hh = H / 2;
  // owned output range and the (possibly shifted) tile origin
  int tbx, tby;
  tile_of<INTERIOR>(tiles, tbx, tby);
  const int OX = tbx * TX, OY = tby * TY;
  const int X0 = W >= TX ? min(OX, W - TX) : 0;
  const int Y0 = H >= TY ? min(OY, H - TY) : 0;
  const int OXe = min(OX + TX, W), OYe = min(OY + TY, H);
  // no position of the tile's stages is mirrored or wrapped (even origin, 4 pixel margin)
  constexpr bool interior = INTERIOR;
  if(p.hist) for(int i = tid; i < 257; i += NT) s.hist[i] = 0;
  // the mosaic window by TMA (interior tiles): [X0-8, X0+TX+8) x [Y0-4, Y0+TY+4) of the codes,
  // the first column 16 byte aligned (the host gives a map only where cx and the pitch allow it)
  const uint32_t raw_addr = ((uint32_t)__cvta_generic_to_shared(s.u.e.raw) + 127u) & ~127u;
  const uint16_t *raw = s.u.e.raw + (raw_addr - (uint32_t)__cvta_generic_to_shared(s.u.e.raw)) / 2;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s.bar);
  const bool tma = interior && use_map;
  if(tma && tid == 0)
  {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(bar), "r"(RAW_BYTES) : "memory");
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
                 :: "r"(raw_addr), "l"(reinterpret_cast<uint64_t>(&mmap)), "r"(X0 - 8 + p.cx), "r"(Y0 - 4 + p.cy), "r"(bar)
                 : "memory");
  }

  // ---- the hilite coarse level around the tile (virtual slots, mirrored)
  const int bx0 = ((X0 / 2 - 2) >> 1) - 2, by0 = ((Y0 / 2 - 2) >> 1) - 2;
  for(int i = tid; i < BX * BX; i += NT)
  {
    const int sx = i % BX, sy = i / BX;
    const int gx = mirror1(bx0 + sx, p.hcw), gy = mirror1(by0 + sy, p.hch);
    float a, b, c, d;
    ld_half4(p.hl_coarse + (size_t)gy * p.hcw + gx, a, b, c, d);
    s.u.e.B1[0][sy][sx] = a; s.u.e.B1[1][sy][sx] = b; s.u.e.B1[2][sy][sx] = c;
  }
  __syncthreads();   // (also orders the barrier's initialisation before the waits below)
  if(tma && !mbar_wait(bar, TMA_WAIT_POLLS))
  { // the copy did not complete: record it, give it a last bounded chance to land, leave
    if(tid == 0) atomicOr(status, 1u);
    mbar_wait(bar, TMA_WAIT_POLLS);
    return;
  }

  // ---- hilite output mosaic on virtual blocks [X0/2-2, X0/2+TX/2+2):
  // denoise/noop (lut), hilite/half, level 0 hilite/assemble, hilite/doub
  {
    const int hx0 = X0 / 2 - 2, hy0 = Y0 / 2 - 2;
    for(int i = tid; i < MB * MB; i += NT)
    {
      const int sbx = i % MB, sby = i / MB;
      const int vbx = hx0 + sbx, vby = hy0 + sby;
      const int rbx = mirror1(vbx, hw), rby = mirror1(vby, hh);
      const bool fx = vbx < 0 || vbx >= hw, fy = vby < 0 || vby >= hh;
      uint32_t r0, r1;
      if(tma)
      { // window column of pixel 2 rbx = X0 - 4 + 2 sbx is 2 sbx + 4, row 2 sby
        r0 = *reinterpret_cast<const uint32_t *>(raw + (2 * sby) * RAW_X + 2 * sbx + 4);
        r1 = *reinterpret_cast<const uint32_t *>(raw + (2 * sby + 1) * RAW_X + 2 * sbx + 4);
      }
      else
      {
        const size_t row = (size_t)(2 * rby + p.cy) * p.pitch + 2 * rbx + p.cx;
        r0 = __ldg(reinterpret_cast<const uint32_t *>(p.mosaic + row));
        r1 = __ldg(reinterpret_cast<const uint32_t *>(p.mosaic + row + p.pitch));
      }
      float m[4];
      m[0] = h2f(__ldg(p.noop_lut + (r0 & 0xffff)));
      m[1] = h2f(__ldg(p.noop_lut + (r0 >> 16)));
      m[2] = h2f(__ldg(p.noop_lut + (r1 & 0xffff)));
      m[3] = h2f(__ldg(p.noop_lut + (r1 >> 16)));
      float o[4] = { m[0], m[1], m[2], m[3] };
      // hilite/doub changes a block only where its largest sample exceeds
      // 0.97 white, and the level 0 assemble feeds nothing else: elsewhere
      // the block is the noop output as it is (f16 values already)
      if(fmaxf(fmaxf(m[2], m[3]), fmaxf(m[1], m[0])) > 0.97f * p.hl_white)
      {
        float h[4];
        hilite_half_bayer(m[0], m[1], m[2], m[3], p.hl_white, h);
        h[3] = 1.0f;
        float up[3];
        hilite_expand_px([&](int ix, int iy, float rgb[3]) {
            const int sx = ix - bx0, sy = iy - by0;
            rgb[0] = s.u.e.B1[0][sy][sx]; rgb[1] = s.u.e.B1[1][sy][sx]; rgb[2] = s.u.e.B1[2][sy][sx];
          }, rbx, rby, up);
        float b0[3];
        hilite_assemble_px(h, up, p.hl_white, p.hl_soft, b0);
        hilite_doub_bayer(m[0], m[1], m[2], m[3], b0, p.hl_white, o);
      }
      // flipped blocks (mirrored at the image border) swap their rows / columns
      const float t0 = fy ? o[2] : o[0], t1 = fy ? o[3] : o[1], t2 = fy ? o[0] : o[2], t3 = fy ? o[1] : o[3];
      s.M[2 * sby][fx ? 1 : 0][sbx] = t0;
      s.M[2 * sby][fx ? 0 : 1][sbx] = t1;
      s.M[2 * sby + 1][fx ? 1 : 0][sbx] = t2;
      s.M[2 * sby + 1][fx ? 0 : 1][sbx] = t3;
      if(p.dbg_denoise && !fx && !fy && 2 * rbx >= OX && 2 * rbx < OXe && 2 * rby >= OY && 2 * rby < OYe)
#pragma unroll
        for(int dy = 0; dy < 2; dy++)
#pragma unroll
        for(int dx = 0; dx < 2; dx++)
        {
          const size_t idx = (size_t)(2 * rby + dy) * W + 2 * rbx + dx;
          p.dbg_denoise[idx] = f2h(m[dy * 2 + dx]);
          p.dbg_hilite[idx] = f2h(o[dy * 2 + dx]);
        }
    }
  }
  __syncthreads();

  // ---- demosaic/gauss.comp:24-75 (bayer) on half positions [X0/2-1, X0/2+TX/2+1),
  // then the splat and fix weight tables of each entry
  for(int i = tid; i < CX * CX; i += NT)
  {
    const int scx = i % CX, scy = i / CX;
    const int cx = X0 / 2 - 1 + scx, cy = Y0 / 2 - 1 + scy;
    float v[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
    if(cx >= 0 && cy >= 0 && cx < hw && cy < hh)
    {
      int dec;
      // green samples at (2c+ii, 2c+j), (ii+j) odd: M slot x = 2scx+2+ii
      float px[8];
      int k = 0;
#pragma unroll
      for(int j = -1; j < 3; j++)
#pragma unroll
      for(int ii = -1; ii < 3; ii++)
      {
        if(((j + ii) & 1) != 1) continue;
        const int xs = 2 * scx + 2 + ii;
        px[k++] = s.M[2 * scy + 2 + j][xs & 1][xs >> 1];
      }
      gauss_exact(px, v, dec, p.neg_zero);
      // debug: the entry's decisions, written by the CTA whose outputs own it
      if(p.dbg_gauss && cx >= OX / 2 && cx < OX / 2 + TX / 2 && cy >= OY / 2 && cy < OY / 2 + TY / 2)
        p.dbg_gauss[(size_t)cy * hw + cx] = (uint8_t)dec;
    }
    // splat.comp:159-163 and fix.comp:21-29 weights of this entry. E (i, j) is
    // (i, j) for evec (1,0), (j, -i) for evec (0,1) and 0 without covariance,
    // so a horizontal tap has dot = 1/e0 resp. 1/e1, a vertical one the other,
    // a diagonal one 1/e0 + 1/e1, and every tap 0 without covariance
    const int ori = v[2] == 1.0f ? 0 : (v[3] == 1.0f ? 1 : 2);
    {
      // (continuous values from here on: fast reciprocal and exp)
      const float r0 = __fdividef(1.0f, gclamp(v[0], 0.01f, 25.0f)), r1 = __fdividef(1.0f, gclamp(v[1], 0.01f, 25.0f));
      const float wa = gclamp(curve_exp(-0.5f * r0), 1e-4f, 1.0f);
      const float wb = gclamp(curve_exp(-0.5f * r1), 1e-4f, 1.0f);
      const float wc = gclamp(curve_exp(-0.5f * (r0 + r1)), 1e-4f, 1.0f);
      s.u.e.sw[0][scy][scx] = ori == 0 ? wa : (ori == 1 ? wb : 1.0f);
      s.u.e.sw[1][scy][scx] = ori == 0 ? wb : (ori == 1 ? wa : 1.0f);
      s.u.e.sw[2][scy][scx] = ori == 2 ? 1.0f : wc;
    }
    {
      const float r0 = __fdividef(1.0f, 2.0f * gclamp(v[0], 1.0f, 49.0f)), r1 = __fdividef(1.0f, 2.0f * gclamp(v[1], 1.0f, 49.0f));
      const float wa = gclamp(curve_exp(-0.5f * r0), 1e-3f, 1.0f);
      const float wb = gclamp(curve_exp(-0.5f * r1), 1e-3f, 1.0f);
      const float wc = gclamp(curve_exp(-0.5f * (r0 + r1)), 1e-3f, 1.0f);
      s.fw[0][scy][scx] = ori == 0 ? wa : (ori == 1 ? wb : 1.0f);
      s.fw[1][scy][scx] = ori == 0 ? wb : (ori == 1 ? wa : 1.0f);
      s.fw[2][scy][scx] = ori == 2 ? 1.0f : wc;
    }
  }
  __syncthreads();

  // ---- demosaic/splat.comp:224-266 (bayer) on virtual [X0-2, X0+TX+1), one CFA phase per warp
  {
    constexpr int NB = GH * GH;
    for(int t = tid; t < 4 * NB; t += NT)
    {
      const int ph = t / NB, b = t % NB;
      const int bx = b % GH, by = b / GH;
      const int sgx = 2 * bx + (ph & 1), sgy = 2 * by + (ph >> 1);
      if(sgx >= GX || sgy >= GX) continue;
      float rg = 0.0f, wg = 0.0f;
      if(interior)
      { // pixel X0 - 2 + sgx: its phase is the slot's, its entry (sgx + 1) / 2
        const int ccx = bx + (ph & 1), ccy = by + (ph >> 1);
        const float wh = s.u.e.sw[0][ccy][ccx], wv = s.u.e.sw[1][ccy][ccx], wd = s.u.e.sw[2][ccy][ccx];
        switch(ph)
        {
          case 0: splat_taps_in<0, 0>(s, bx, sgy, wh, wv, wd, rg, wg); break;
          case 1: splat_taps_in<1, 0>(s, bx, sgy, wh, wv, wd, rg, wg); break;
          case 2: splat_taps_in<0, 1>(s, bx, sgy, wh, wv, wd, rg, wg); break;
          default: splat_taps_in<1, 1>(s, bx, sgy, wh, wv, wd, rg, wg); break;
        }
      }
      else
      {
        const int qx = mirror1(X0 - 2 + sgx, W), qy = mirror1(Y0 - 2 + sgy, H);
        const int ccx = (qx + 1) / 2 - (X0 / 2 - 1), ccy = (qy + 1) / 2 - (Y0 / 2 - 1);
        const float wh = s.u.e.sw[0][ccy][ccx], wv = s.u.e.sw[1][ccy][ccx], wd = s.u.e.sw[2][ccy][ccx];
        switch((qx & 1) | ((qy & 1) << 1))
        { // the CFA phase of the real pixel: uniform in a warp but at mirrored borders
          case 0: splat_taps<0, 0>(s, qx, qy, W, H, X0, Y0, wh, wv, wd, rg, wg); break;
          case 1: splat_taps<1, 0>(s, qx, qy, W, H, X0, Y0, wh, wv, wd, rg, wg); break;
          case 2: splat_taps<0, 1>(s, qx, qy, W, H, X0, Y0, wh, wv, wd, rg, wg); break;
          default: splat_taps<1, 1>(s, qx, qy, W, H, X0, Y0, wh, wv, wd, rg, wg); break;
        }
      }
      const float gv = f16r(rg / fmaxf(1e-8f, wg));
      s.g[sgy][sgx & 1][sgx >> 1] = f2h(gv);    // gv is an f16 value: exact
      s.rg[sgy][sgx & 1][sgx >> 1] = 1.0f / (1e-4f + gv);
    }
  }
  __syncthreads();

  // ---- demosaic/fix -> colour -> hist -> filmcurv -> llap/curve on virtual [X0-1, X0+TX)
  {
    const float sig = p.ll_sigma, shd = p.ll_shadows, hil = p.ll_highlights, cla = p.ll_clarity;
    const float r2s = 1.0f / (2.0f * sig), rden = 1.0f / (2.0f * sig * sig / 3.0f);
    const bool unit_curve = shd == 1.0f && hil == 1.0f;
    constexpr int NB = LH * LH;
    for(int t = tid; t < 4 * NB; t += NT)
    {
      const int ph = t / NB, b = t % NB;
      const int slx = 2 * (b % LH) + (ph & 1), sly = 2 * (b / LH) + (ph >> 1);
      if(slx >= LX || sly >= LX) continue;
      const int vx = X0 - 1 + slx, vy = Y0 - 1 + sly;
      float rr = 0.0f, rb = 0.0f, wr = 0.0f, wb = 0.0f, rg = 0.0f, wg = 0.0f;
      int px, py;
      if(!L1)
      { // only the pixels this tile owns: the halo fed the llap level 0 planes
        const int qx = interior ? vx : mirror1(vx, W), qy = interior ? vy : mirror1(vy, H);
        if(qx != vx || qy != vy || vx < OX || vx >= OXe || vy < OY || vy >= OYe) continue;
      }
      // demosaic/fix.comp:99-135, radius clamp(fixup+1, 1, 2) = 1 for the
      // default fixup 0 (the host rejects other values for this kernel)
      if(interior)
      { // pixel X0 - 1 + slx: phase 1 - the slot's, entry slx / 2 + 1, splat slot slx + 1
        px = vx; py = vy;
        const int bx = b % LH, by = b / LH;
        const int ccx = bx + 1, ccy = by + 1;
        const float wh = s.fw[0][ccy][ccx], wv = s.fw[1][ccy][ccx], wd = s.fw[2][ccy][ccx];
        const float gc = h2f(s.g[sly + 1][1 - (ph & 1)][bx + (ph & 1)]);
        switch(ph)
        {
          case 3: fix_taps_in<0, 0>(s, bx, sly, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          case 2: fix_taps_in<1, 0>(s, bx, sly, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          case 1: fix_taps_in<0, 1>(s, bx, sly, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          default: fix_taps_in<1, 1>(s, bx, sly, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
        }
      }
      else
      {
        px = mirror1(vx, W); py = mirror1(vy, H);
        const int gx0 = px - (X0 - 2), gy0 = py - (Y0 - 2);
        const float gc = h2f(s.g[gy0][gx0 & 1][gx0 >> 1]);
        const int ccx = (px + 1) / 2 - (X0 / 2 - 1), ccy = (py + 1) / 2 - (Y0 / 2 - 1);
        const float wh = s.fw[0][ccy][ccx], wv = s.fw[1][ccy][ccx], wd = s.fw[2][ccy][ccx];
        switch((px & 1) | ((py & 1) << 1))
        {
          case 0: fix_taps<0, 0>(s, px, py, gx0, gy0, X0, Y0, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          case 1: fix_taps<1, 0>(s, px, py, gx0, gy0, X0, Y0, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          case 2: fix_taps<0, 1>(s, px, py, gx0, gy0, X0, Y0, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
          default: fix_taps<1, 1>(s, px, py, gx0, gy0, X0, Y0, gc, wh, wv, wd, rr, rb, wr, wb, rg, wg); break;
        }
      }
      float dm[3];
      dm[0] = f16r(rr / fmaxf(1e-8f, wr));
      dm[1] = f16r(rg / fmaxf(1e-8f, wg));
      dm[2] = f16r(rb / fmaxf(1e-8f, wb));
      float co[3];
      colour_px(p, dm, co);
      const bool own = vx == px && vy == py && px >= OX && px < OXe && py >= OY && py < OYe;
      // the crop window's pixels, at crop coordinates (the whole image without a crop)
      const int ccx = px - p.crop_dx, ccy = py - p.crop_dy;
      const bool keep = own && ccx >= 0 && ccy >= 0 && ccx < p.crop_w && ccy < p.crop_h;
      const size_t co_at = (size_t)ccy * p.crop_w + ccx;
      if(own && p.dbg_colour) p.dbg_demosaic[(size_t)py * W + px] = mk_half4(dm[0], dm[1], dm[2], 1.0f);
      if(keep && p.dbg_colour) p.dbg_colour[co_at] = mk_half4(co[0], co[1], co[2], 1.0f);
      if(keep && p.hist)
      {
        const uint32_t bin = hist_bin(co[0], co[1], co[2]);
        if(bin > 0) { atomicAdd(&s.hist[bin], 1u); atomicAdd(&s.hist[256], 1u); }
      }
      float fc[3];
      filmcurv_px(p, co, fc);
      if(keep) p.rgbf[co_at] = mk_half4(fc[0], fc[1], fc[2], 1.0f);
      if(!L1) continue;
      const float yv = lum2020(gclamp(fc[0], -1000.0f, 1000.0f), gclamp(fc[1], -1000.0f, 1000.0f), gclamp(fc[2], -1000.0f, 1000.0f));
      if(unit_curve)
      {
        const float2 X = make_float2(yv, yv), nr = make_float2(-rden, -rden), cl = make_float2(cla, cla);
#pragma unroll
        for(int j = 0; j < LLAP_PAIRS; j++) s.u.L0.p[j][sly][slx & 1][slx >> 1] = llap_curve_unit2(X, j, nr, cl);
      }
      else
      {
#pragma unroll
        for(int j = 0; j < LLAP_PAIRS; j++)
          s.u.L0.p[j][sly][slx & 1][slx >> 1] = __floats2half2_rn(
              llap_curve_rcp(yv, kLlapGamma[2 * j], sig, r2s, rden, shd, hil, cla),
              llap_curve_rcp(yv, kLlapGamma[2 * j + 1], sig, r2s, rden, shd, hil, cla));
      }
      s.u.L0.g[sly][slx] = f2h(yv);
    }
  }
  __syncthreads();

  // ---- llap/reduce.comp (sample_semisoft) for level 1 outputs [X0/2, X0/2+TX/2) (llap_reduce_px2/_px).
  // A warp takes 16 outputs of row ly and 16 of row ly + 4: its two halves read level 0 rows 8
  // apart, 16 banks apart in the pair arrays
  if(L1)
  {
    const int w = tid >> 5, lx = tid & 15;
    const int ly = (w & 3) + 8 * (w >> 2) + 4 * ((tid >> 4) & 1);
    const int ox = X0 / 2 + lx, oy = Y0 / 2 + ly;
    const bool own = ox >= OX / 2 && ox < min(OX / 2 + TX / 2, p.l1w) && oy >= OY / 2 && oy < min(OY / 2 + TY / 2, p.l1h);
    if(own)
    {
      // level 0 slot of virtual x = 2ox + a - 1 is 2lx + a: pair words [.][0][lx], [.][1][lx], [.][0][lx + 1]
      const size_t o = (size_t)oy * p.l1pitch + ox;
#pragma unroll
      for(int j = 0; j < LLAP_PAIRS; j++)
      {
        const __half2 *a[3], *b[3], *c[3];
#pragma unroll
        for(int r = 0; r < 3; r++)
        {
          a[r] = &s.u.L0.p[j][2 * ly + r][0][lx];
          b[r] = &s.u.L0.p[j][2 * ly + r][1][lx];
          c[r] = &s.u.L0.p[j][2 * ly + r][0][lx + 1];
        }
        const float2 v = llap_reduce_px2(a, b, c);
        p.l1[(2 * j) * p.l1plane + o] = f2h(v.x);
        p.l1[(2 * j + 1) * p.l1plane + o] = f2h(v.y);
      }
      const __half *const row[3] = { &s.u.L0.g[2 * ly][2 * lx], &s.u.L0.g[2 * ly + 1][2 * lx], &s.u.L0.g[2 * ly + 2][2 * lx] };
      p.l1[(NPL - 1) * p.l1plane + o] = f2h(llap_reduce_px(row));
    }
  }
  if(p.hist)
  {
    __syncthreads();
    for(int i = tid; i < 257; i += NT) if(s.hist[i]) atomicAdd(p.hist + i, s.hist[i]);
  }
}

} // namespace

cudaError_t init_develop()
{
  cudaError_t e = cudaSuccess;
  const void *fs[4] = { (const void *)k_develop<true, true>, (const void *)k_develop<false, true>,
                        (const void *)k_develop<true, false>, (const void *)k_develop<false, false> };
  for(int i = 0; i < 4; i++)
  {
    const int bytes = i < 2 ? (int)sizeof(smem_t) : (int)SMEM_NO_L1;
    if(e == cudaSuccess) e = cudaFuncSetAttribute(fs[i], cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    // the whole unified L1 as shared memory: 5 CTAs of 43.5 KB per SM (with the llap planes)
    if(e == cudaSuccess) e = cudaFuncSetAttribute(fs[i], cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  }
  if(e == cudaSuccess) e = init_llap();
  if(e == cudaSuccess) e = init_hilite();
  return e;
}

template<bool L1> static void launch_tiles(const dev_image_t &p, const tiles_t &t, int nin, const CUtensorMap *map,
    uint32_t *status, cudaStream_t s)
{
  const size_t bytes = L1 ? sizeof(smem_t) : SMEM_NO_L1;
  CUtensorMap none;
  memset(&none, 0, sizeof(none));
  if(nin > 0) k_develop<true, L1><<<dim3(t.ix1 - t.ix0 + 1, t.iy1 - t.iy0 + 1), NT, bytes, s>>>(p, t, map ? *map : none, map ? 1 : 0, status);
  k_develop<false, L1><<<t.nx * t.ny - nin, NT, bytes, s>>>(p, t, none, 0, status);
}

// the 2D tensor map over a mosaic of u16 codes (or the f16 bits of the denoised mosaic) that
// interior tiles stage their window through: base 16 byte aligned, pitch a multiple of 8 codes
cudaError_t develop_tensor_map(const void *mosaic, int wd, int ht, int pitch, CUtensorMap *map)
{
  if(((uintptr_t)mosaic & 15) || (pitch & 7)) return cudaErrorInvalidValue;
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if(!encode) return cudaErrorNotSupported;
  const cuuint64_t dim[2] = { (cuuint64_t)wd, (cuuint64_t)ht };
  const cuuint64_t stride[1] = { (cuuint64_t)pitch * sizeof(uint16_t) };
  const cuuint32_t box[2] = { (cuuint32_t)RAW_X, (cuuint32_t)RAW_Y };
  const cuuint32_t estride[2] = { 1, 1 };
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(mosaic), dim, stride, box, estride,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_develop(const dev_image_t &p, const CUtensorMap *map, uint32_t *status, cudaStream_t s)
{
  tiles_t t;
  t.nx = (p.W + TX - 1) / TX; t.ny = (p.H + TY - 1) / TY;
  // interior tile bx: origin 32 bx >= 4 and 32 bx + TX + 4 <= W (then it is not the shifted last tile)
  t.ix0 = 1; t.ix1 = (p.W - TX - 4) / TX;
  t.iy0 = 1; t.iy1 = (p.H - TY - 4) / TY;
  if(p.W < 2 * TX + 4 || p.H < 2 * TY + 4 || t.ix1 < t.ix0 || t.iy1 < t.iy0)
  { // no interior: every tile is a border tile (the ring is the whole grid)
    t.ix0 = t.nx; t.ix1 = t.nx - 1; t.iy0 = t.ny; t.iy1 = t.ny - 1;
  }
  const int nin = t.ix1 < t.ix0 ? 0 : (t.ix1 - t.ix0 + 1) * (t.iy1 - t.iy0 + 1);
  // p.l1 null: end at filmcurv (a crop follows demosaic; the llap level 1 is made from rgbf)
  if(p.l1) launch_tiles<true>(p, t, nin, map, status, s);
  else launch_tiles<false>(p, t, nin, map, status, s);
  return cudaGetLastError();
}
