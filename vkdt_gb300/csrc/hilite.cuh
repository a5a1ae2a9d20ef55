// Per pixel bodies of denoise/noop and the hilite module shaders, shared by
// the hilite pyramid kernels and the fused develop kernel.
#pragma once
#include "common.cuh"
#include "kernels.h"

DEV int mirror_full(int i, int n)
{ // mirrored repeat for any i (periodic with 2n)
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  t = t < n ? t : m - 1 - t;
  return t < 0 ? 0 : (t >= n ? n - 1 : t);
}

// denoise/noop.comp:36-57: normalised mosaic value at a position of the
// denoise output (crop offset applied), stored as f16
DEV float noop_val(const uint16_t *__restrict__ mosaic, int pitch, int cx, int cy, int W, int H,
    int x, int y, float black, float white)
{
  x = min(max(x, 0), W - 1);
  y = min(max(y, 0), H - 1);
  const float v = (float)__ldg(mosaic + (size_t)(y + cy) * pitch + (x + cx)) / 65535.0f;
  return f16r(fmaxf(0.0f, (v - black) / (white - black)));
}

// denoise/noop.comp:36-57 per u16 code: max(0, (v/65535 - black)/(white - black))
// stored as f16, the IEEE operations of the code table (k_static.cu), with the
// two quotients by Markstein's correction on reciprocals made once (div_ry).
// For kernels whose shared memory leaves the 128 KB table no room in L1: a
// lookup there is a random L2 sector read, evaluating the code a few
// instructions. Identity codes are f16 bits.
struct noop_eval_t { float black, wmb, ywb, y65535; bool wok, identity; };

DEV noop_eval_t noop_prep(const dev_codes_t &c)
{
  noop_eval_t n;
  n.black = c.black;
  n.wmb = __fsub_rn(c.white, c.black);
  n.ywb = __frcp_rn(n.wmb);
  n.wok = div_ok(n.wmb);
  n.y65535 = __frcp_rn(65535.0f);
  n.identity = c.identity != 0;
  return n;
}

DEV float noop_code(const noop_eval_t &n, uint32_t v)
{
  if(n.identity) return __half2float(__ushort_as_half((unsigned short)v));
  // zero numerators are +0 here (v = 0; x equal to black) and give +0
  const float x = v ? div_ry((float)v, 65535.0f, n.y65535, true) : 0.0f;
  const float a = __fsub_rn(x, n.black);
  const float q = a == 0.0f ? 0.0f : div_ry(a, n.wmb, n.ywb, n.wok);
  return __half2float(__float2half_rn(fmaxf(0.0f, q)));
}

// hilite/half.comp:157-165 (bayer): textureGather order x=(0,1) y=(1,1) z=(1,0) w=(0,0)
DEV void hilite_half_bayer(float m00, float m10, float m01, float m11, float white, float h[3])
{
  float cx = m01, cy = m11, cz = m10, cw = m00;
  if(cx >= white) cx = cz;
  if(cz >= white) cz = cx;
  h[0] = f16r(cw);
  h[1] = f16r((cx + cz) * 0.5f); // exactly the shader's /2
  h[2] = f16r(cy);
}

// hilite/half.comp:124-156 (x-trans). c[3*i+j] = texel (3x+i, 3y+j)
DEV void hilite_half_xtrans(float c[9], int x, int y, float white, float h[3])
{
  if(c[1] >= white) c[1] = c[7];
  if(c[7] >= white) c[7] = c[1];
  if(c[3] >= white) c[3] = c[5];
  if(c[5] >= white) c[5] = c[3];
  const float maxg = fmaxf(fmaxf(fmaxf(c[0], c[2]), c[4]), fmaxf(c[6], c[8]));
  if(maxg >= white) c[0] = c[2] = c[4] = c[6] = c[8] = 1.0f;
  const float c0 = (c[1] + c[7]) * 0.5f, c1 = (c[3] + c[5]) * 0.5f;
  float r, b;
  if(((x + y) & 1) > 0) { r = c0; b = c1; }
  else                  { b = c0; r = c1; }
  h[0] = f16r(r);
  h[1] = f16r(__fdiv_rn(c[0] + c[2] + c[4] + c[6] + c[8], 5.0f));
  h[2] = f16r(b);
}

// hilite/reduce.comp:21-61 in two parts. The terms a tap takes from its
// texel (the luminance, and for an unclipped texel the colour desaturated
// towards its grey) depend on the texel alone, so the kernels make them once
// per texel of a tile (hilite_reduce_texel); an output then sums them over its
// 5x5 taps (hilite_reduce_sum) in the shader's order.
struct hl_reduce_t { float white, iwhite, d5, wb[3], hwb[3]; };

DEV hl_reduce_t hilite_reduce_args(float white_p, float desat, const float wbp[3])
{
  hl_reduce_t a;
  a.white = white_p;
  if(!(a.white > 0.0f)) a.white = 1.0f;
  for(int k = 0; k < 3; k++) a.wb[k] = wbp[k];
  if(!(a.wb[0] * a.wb[0] + a.wb[1] * a.wb[1] + a.wb[2] * a.wb[2] > 1e-3f)) a.wb[0] = a.wb[1] = a.wb[2] = 1.0f;
  const float ds = desat * desat;
  a.d5 = 5.0f * ds * ds;
  // the divisions by loop invariants as products (continuous values only:
  // the clip test compares the texels themselves)
  a.iwhite = 1.0f / a.white;
  for(int k = 0; k < 3; k++) a.hwb[k] = 0.5f / a.wb[k];
  return a;
}

// t[0]: luminance; t[1..3]: the desaturated colour of an unclipped texel, t[4] = 1
// (a clipped texel: t[1..4] = 0, it takes no weight)
DEV void hilite_reduce_texel(const hl_reduce_t &a, const float rgb[3], float t[5])
{
  t[0] = lum2020(rgb[0], rgb[1], rgb[2]);
  t[1] = t[2] = t[3] = t[4] = 0.0f;
  if(rgb[0] < a.white && rgb[1] < a.white && rgb[2] < a.white)
  {
    const float rw = rgb[0] * a.wb[0], gw = rgb[1] * a.wb[1], bw = rgb[2] * a.wb[2];
    const float cmax = fmaxf(rw, fmaxf(gw, bw));
    const float cmin = fminf(rw, fminf(gw, bw));
    const float sat = __fdividef(cmax - cmin, fmaxf(1e-3f, cmax));
    // smoothstep(0.2, 1, max / white) and smoothstep(0.15, 0.9, sat)
    float s = gclamp((fmaxf(rgb[0], fmaxf(rgb[1], rgb[2])) * a.iwhite - 0.2f) * 1.25f, 0.0f, 1.0f);
    s = s * s * (3.0f - 2.0f * s);
    float t2 = gclamp((sat - 0.15f) * (1.0f / 0.75f), 0.0f, 1.0f);
    t2 = t2 * t2 * (3.0f - 2.0f * t2);
    t2 = gclamp(a.d5 * s * t2, 0.0f, 1.0f);
#pragma unroll
    for(int k = 0; k < 3; k++) t[1 + k] = gmix(rgb[k], (cmax + cmin) * a.hwb[k], t2);
    t[4] = 1.0f;
  }
}

// fetch(ii, jj, t) returns the terms of the texel at (2o+ii, 2o+jj)
template<class F> DEV void hilite_reduce_sum(F fetch, float o[4])
{
  const float w[5] = { 1.0f / 16.0f, 4.0f / 16.0f, 6.0f / 16.0f, 4.0f / 16.0f, 1.0f / 16.0f };
  const float sw[5] = { 1.0f, 2.0f, 0.0f, -2.0f, -1.0f };
  float e0 = 0.0f, e1 = 0.0f, col[3] = { 0.0f, 0.0f, 0.0f }, wgt = 0.0f;
#pragma unroll
  for(int jj = -2; jj <= 2; jj++)
#pragma unroll
  for(int ii = -2; ii <= 2; ii++)
  {
    float t[5];
    fetch(ii, jj, t);
    e0 += w[jj + 2] * sw[ii + 2] * t[0];
    e1 += w[ii + 2] * sw[jj + 2] * t[0];
    const float u = w[ii + 2] * w[jj + 2];
    if(t[4] != 0.0f)
    {
#pragma unroll
      for(int k = 0; k < 3; k++) col[k] += t[1 + k] * u;
      wgt += u;
    }
  }
  if(wgt == 0.0f) { o[0] = o[1] = o[2] = 1.0f; }
  else for(int k = 0; k < 3; k++) o[k] = col[k] / wgt;
  o[3] = sqrtf(e0 * e0 + e1 * e1);
}

// hilite/assemble.comp:23-81 gauss_expand. fetch(ix, iy, rgb) reads the
// coarse texel (ix, iy) (caller applies the mirrored repeat)
DEV float binom5(int k)
{ // (1 4 6 4 1) / 16 at k = 0..4, without an indexed table (kept in registers)
  return k == 2 ? 6.0f / 16.0f : ((k == 1 || k == 3) ? 4.0f / 16.0f : 1.0f / 16.0f);
}
template<class F> DEV void hilite_expand_px(F fetch, int ox, int oy, float c[3])
{
  c[0] = c[1] = c[2] = 0.0f;
  float wgt = 0.0f;
  const int ix = ox / 2, iy = oy / 2;
  const int dx = ox & 1, dy = oy & 1;
  const int i0 = dx ? 0 : -1, j0 = dy ? 0 : -1;
  for(int ii = i0; ii <= 1; ii++) for(int jj = j0; jj <= 1; jj++)
  {
    const float wy = dy ? binom5(2 * jj + 1) : binom5(2 * jj + 2);
    const float wx = dx ? binom5(2 * ii + 1) : binom5(2 * ii + 2);
    float rgb[3];
    fetch(ix + ii, iy + jj, rgb);
    for(int k = 0; k < 3; k++) c[k] += rgb[k] * wy * wx;
    wgt += wy * wx;
  }
  if(wgt == 0.0f) { c[0] = 0.0f; c[1] = 1.0f; c[2] = 1.0f; return; }
  for(int k = 0; k < 3; k++) c[k] /= wgt;
}

// the same expand for an output of known parity (DX, DY): the taps unrolled,
// their weights constants, the sums in the same order (bit-identical)
template<int DX, int DY, class F> DEV void hilite_expand_px_t(F fetch, int ox, int oy, float c[3])
{
  c[0] = c[1] = c[2] = 0.0f;
  float wgt = 0.0f;
  const int ix = ox / 2, iy = oy / 2;
  constexpr int i0 = DX ? 0 : -1, j0 = DY ? 0 : -1;
#pragma unroll
  for(int ii = i0; ii <= 1; ii++)
#pragma unroll
  for(int jj = j0; jj <= 1; jj++)
  {
    const float wy = DY ? binom5(2 * jj + 1) : binom5(2 * jj + 2);
    const float wx = DX ? binom5(2 * ii + 1) : binom5(2 * ii + 2);
    float rgb[3];
    fetch(ix + ii, iy + jj, rgb);
    for(int k = 0; k < 3; k++) c[k] += rgb[k] * wy * wx;
    wgt += wy * wx;
  }
  if(wgt == 0.0f) { c[0] = 0.0f; c[1] = 1.0f; c[2] = 1.0f; return; }
  for(int k = 0; k < 3; k++) c[k] /= wgt;
}

// hilite/assemble.comp:88-118 (f: fine rgba, up: expanded coarse rgb)
DEV void hilite_assemble_px(float f[4], const float up[3], float white, float soft, float o[3])
{
  const float sr = f[0] / fmaxf(0.001f, up[0]);
  const float sg = f[1] / fmaxf(0.001f, up[1]);
  const float sb = f[2] / fmaxf(0.001f, up[2]);
  const float wr = expf(up[0] - fmaxf(up[1], up[2]));
  const float wg = expf(up[1] - fmaxf(up[0], up[2]));
  const float wbb = expf(up[2] - fmaxf(up[0], up[1]));
  const float scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
  float rec[3];
  for(int k = 0; k < 3; k++) rec[k] = gclamp(up[k] * scale, -65535.0f, 65535.0f);
  float t = soft;
  if(f[0] >= white || f[1] >= white || f[2] >= white) t = 1.0f;
  if(isnan(f[3])) f[3] = 0.0f;
  t = gclamp(gmix(t, 1.0f, sqrtf(fmaxf(0.0f, f[3]))), 0.0f, 1.0f);
  for(int k = 0; k < 3; k++) o[k] = f16r(gmix(f[k], rec[k], t));
}

// hilite/doub.comp:213-240 (bayer). in: noop'd block m00 m10 m01 m11, up: coarse rgb.
// out: the four f16 mosaic values in the order (0,0) (1,0) (0,1) (1,1)
DEV void hilite_doub_bayer(float m00, float m10, float m01, float m11, const float up[3], float white, float out[4])
{
  float cx = m01, cy = m11, cz = m10, cw = m00;
  const float ming = fminf(cx, cz);
  const float sr = cw / fmaxf(0.001f, up[0]);
  const float sg = ming / fmaxf(0.001f, up[1]);
  const float sb = cy / fmaxf(0.001f, up[2]);
  const float wr = expf(up[0] - fmaxf(up[1], up[2]));
  const float wg = expf(up[1] - fmaxf(up[0], up[2]));
  const float wbb = expf(up[2] - fmaxf(up[0], up[1]));
  const float scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
  const float softw = 0.97f * white;
  const float maxrgb = fmaxf(fmaxf(cx, cy), fmaxf(cz, cw));
  if(maxrgb > softw)
  {
    const float t = smoothstep(softw, white, maxrgb);
    cx = gmix(cx, scale * up[1], t);
    cy = gmix(cy, scale * up[2], t);
    cz = gmix(cz, scale * up[1], t);
    cw = gmix(cw, scale * up[0], t);
  }
  out[0] = f16r(cw); out[1] = f16r(cz); out[2] = f16r(cx); out[3] = f16r(cy);
}
