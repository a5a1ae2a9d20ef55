// texture() on rgba f16 images as the reference's samplers evaluate it
// (LINEAR filter, MIRRORED_REPEAT, normalised coordinates; src/qvk/qvk.c:596-611):
// the sample position is rounded to 8 sub-texel bits, then the four texels
// are blended in FP32.
#pragma once
#include "common.cuh"

DEV void ld4(const half4 *img, int w, int x, int y, float v[4]) { ld_half4(img + (size_t)y * w + x, v[0], v[1], v[2], v[3]); }

// position of a texture() read in texel space, rounded to the sampler's 8 sub-texel bits
DEV float subtexel(float v) { return __fmul_rn(floorf(__fadd_rn(__fmul_rn(v, 256.0f), 0.5f)), 0.00390625f); }

// the blend of texture() once its position is resolved: texel (x0, y0) and fractions (ax, ay)
DEV void bilinear_at(const half4 *img, int w, int h, int x0, int y0, float ax, float ay, float out[4])
{
  const int X0 = mirror(x0, w), X1 = mirror(x0 + 1, w), Y0 = mirror(y0, h), Y1 = mirror(y0 + 1, h);
  float t00[4], t10[4], t01[4], t11[4];
  ld4(img, w, X0, Y0, t00); ld4(img, w, X1, Y0, t10); ld4(img, w, X0, Y1, t01); ld4(img, w, X1, Y1, t11);
#pragma unroll
  for(int k = 0; k < 4; k++)
    out[k] = (t00[k] * (1.0f - ax) + t10[k] * ax) * (1.0f - ay) + (t01[k] * (1.0f - ax) + t11[k] * ax) * ay;
}

// MIRRORED_REPEAT for any texel index (the period 2n), every index in [0, n)
DEV int mirror_any(int i, int n)
{
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  return t < n ? t : m - 1 - t;
}

// texture() with LINEAR + MIRRORED_REPEAT at texel-space position (x, y). ANY:
// positions anywhere (a NaN or a position past +-1e9 texels read as +-1e9 before
// the conversion, every index wrapped by mirror_any), else within one image size
// of the image (mirror)
template<bool ANY = false> DEV void bilinear(const half4 *img, int w, int h, float x, float y, float out[4])
{
  const float xs = subtexel(__fsub_rn(x, 0.5f)), ys = subtexel(__fsub_rn(y, 0.5f));
  const float fx = floorf(xs), fy = floorf(ys);
  const int x0 = ANY ? (int)fminf(fmaxf(fx, -1e9f), 1e9f) : (int)fx, y0 = ANY ? (int)fminf(fmaxf(fy, -1e9f), 1e9f) : (int)fy;
  const float ax = xs - fx, ay = ys - fy;
  const int X0 = ANY ? mirror_any(x0, w) : mirror(x0, w), X1 = ANY ? mirror_any(x0 + 1, w) : mirror(x0 + 1, w);
  const int Y0 = ANY ? mirror_any(y0, h) : mirror(y0, h), Y1 = ANY ? mirror_any(y0 + 1, h) : mirror(y0 + 1, h);
  float t00[4], t10[4], t01[4], t11[4];
  ld4(img, w, X0, Y0, t00); ld4(img, w, X1, Y0, t10); ld4(img, w, X0, Y1, t01); ld4(img, w, X1, Y1, t11);
#pragma unroll
  for(int k = 0; k < 4; k++)
    out[k] = (t00[k] * (1.0f - ax) + t10[k] * ax) * (1.0f - ay) + (t01[k] * (1.0f - ax) + t11[k] * ax) * ay;
}

// shared.glsl:47-96 sample_catmull_rom at normalised uv on a w x h image: nine
// texture() taps. The tap positions decide the texels read, so they are
// formed with IEEE operations in the shader's order (including its division
// back to normalised coordinates, which texture() scales again).
template<bool ANY = false> DEV void catmull_rom_uv(const half4 *img, int w, int h, float u, float v, float res[4])
{
  const float ts[2] = { (float)w, (float)h }, uv[2] = { u, v };
  float t[2][3], wt[2][3];
#pragma unroll
  for(int k = 0; k < 2; k++)
  {
    const float sp = __fmul_rn(uv[k], ts[k]);
    const float tp1 = __fadd_rn(floorf(__fsub_rn(sp, 0.5f)), 0.5f);
    const float f = __fsub_rn(sp, tp1);
    const float w1 = __fadd_rn(1.0f, __fmul_rn(__fmul_rn(f, f), __fadd_rn(-2.5f, __fmul_rn(1.5f, f))));
    const float w2 = __fmul_rn(f, __fadd_rn(0.5f, __fmul_rn(f, __fsub_rn(2.0f, __fmul_rn(1.5f, f)))));
    const float w12 = __fadd_rn(w1, w2);
    t[k][0] = __fmul_rn(__fdiv_rn(__fsub_rn(tp1, 1.0f), ts[k]), ts[k]);
    t[k][1] = __fmul_rn(__fdiv_rn(__fadd_rn(tp1, __fdiv_rn(w2, w12)), ts[k]), ts[k]);
    t[k][2] = __fmul_rn(__fdiv_rn(__fadd_rn(tp1, 2.0f), ts[k]), ts[k]);
    wt[k][0] = f * (-0.5f + f * (1.0f - 0.5f * f));
    wt[k][1] = w12;
    wt[k][2] = f * f * (-0.5f + 0.5f * f);
  }
#pragma unroll
  for(int c = 0; c < 4; c++) res[c] = 0.0f;
#pragma unroll
  for(int j = 0; j < 3; j++)
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
      float q[4];
      bilinear<ANY>(img, w, h, t[0][i], t[1][j], q);
#pragma unroll
      for(int c = 0; c < 4; c++) res[c] += q[c] * wt[0][i] * wt[1][j];
    }
}
