// Per pixel bodies of denoise/noop and the hilite module shaders, shared by
// the hilite pyramid kernels and the fused develop kernel.
#pragma once
#include "common.cuh"

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

// hilite/reduce.comp:21-61. fetch(ii, jj, rgb) returns the texel at (2o+ii, 2o+jj)
template<class F> DEV void hilite_reduce_px(F fetch, float white_p, float desat, const float wbp[3], float o[4])
{
  float white = white_p;
  if(!(white > 0.0f)) white = 1.0f;
  const float w[5] = { 1.0f / 16.0f, 4.0f / 16.0f, 6.0f / 16.0f, 4.0f / 16.0f, 1.0f / 16.0f };
  const float sw[5] = { 1.0f, 2.0f, 0.0f, -2.0f, -1.0f };
  float wb[3] = { wbp[0], wbp[1], wbp[2] };
  if(!(wb[0] * wb[0] + wb[1] * wb[1] + wb[2] * wb[2] > 1e-3f)) wb[0] = wb[1] = wb[2] = 1.0f;
  float e0 = 0.0f, e1 = 0.0f, col[3] = { 0.0f, 0.0f, 0.0f }, wgt = 0.0f;
  const float ds = desat * desat, d5 = 5.0f * ds * ds;
  // the divisions by loop invariants as products (continuous values only:
  // the clip test below compares the texels themselves)
  const float iwhite = 1.0f / white;
  const float hwb[3] = { 0.5f / wb[0], 0.5f / wb[1], 0.5f / wb[2] };
#pragma unroll
  for(int jj = -2; jj <= 2; jj++)
#pragma unroll
  for(int ii = -2; ii <= 2; ii++)
  {
    float rgb[3];
    fetch(ii, jj, rgb);
    const float l = lum2020(rgb[0], rgb[1], rgb[2]);
    e0 += w[jj + 2] * sw[ii + 2] * l;
    e1 += w[ii + 2] * sw[jj + 2] * l;
    const float u = w[ii + 2] * w[jj + 2];
    if(rgb[0] < white && rgb[1] < white && rgb[2] < white)
    {
      const float rw = rgb[0] * wb[0], gw = rgb[1] * wb[1], bw = rgb[2] * wb[2];
      const float cmax = fmaxf(rw, fmaxf(gw, bw));
      const float cmin = fminf(rw, fminf(gw, bw));
      const float sat = __fdividef(cmax - cmin, fmaxf(1e-3f, cmax));
      // smoothstep(0.2, 1, max / white) and smoothstep(0.15, 0.9, sat)
      float s = gclamp((fmaxf(rgb[0], fmaxf(rgb[1], rgb[2])) * iwhite - 0.2f) * 1.25f, 0.0f, 1.0f);
      s = s * s * (3.0f - 2.0f * s);
      float t = gclamp((sat - 0.15f) * (1.0f / 0.75f), 0.0f, 1.0f);
      t = t * t * (3.0f - 2.0f * t);
      t = gclamp(d5 * s * t, 0.0f, 1.0f);
#pragma unroll
      for(int k = 0; k < 3; k++)
      {
        const float v = gmix(rgb[k], (cmax + cmin) * hwb[k], t);
        col[k] += v * u;
      }
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
