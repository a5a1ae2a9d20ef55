// Per pixel bodies shared across kernel files: the llap tone curve and the
// histogram bin index.
#pragma once
#include "common.cuh"

// exp of the tone curves (llap/curve.comp, filmcurv): the accurate expf, or
// the hardware ex2 approximation when built with VKDT_FAST_EXP
#ifdef VKDT_FAST_EXP
#define curve_exp __expf
#else
#define curve_exp expf
#endif

// llap/llap.glsl:3-14 (i / (NUM_GAMMA - 1), correctly rounded: it decides the plane selection)
DEV float llap_gamma(int i) { return __fdiv_rn((float)i, 10.0f - 1.0f); }
// the same values as compile-time constants (for loops unrolled over the planes);
// the initialisers are constant expressions, divided in IEEE round to nearest
__device__ constexpr float kLlapGamma[10] = { 0.0f / 9.0f, 1.0f / 9.0f, 2.0f / 9.0f, 3.0f / 9.0f, 4.0f / 9.0f,
                                              5.0f / 9.0f, 6.0f / 9.0f, 7.0f / 9.0f, 8.0f / 9.0f, 9.0f / 9.0f };

// llap/curve.comp:39-63 (shared with the final llap kernel)
DEV float llap_curve_fn(float x, float g, float sigma, float shadows, float highlights, float clarity)
{
  const float c = x - g;
  float val;
  const float ssigma = c > 0.0f ? sigma : -sigma;
  const float shadhi = c > 0.0f ? shadows : highlights;
  if(fabsf(c) > 2.0f * sigma) val = g + ssigma + shadhi * (c - ssigma);
  else
  {
    const float t = gclamp(c / (2.0f * ssigma), 0.0f, 1.0f);
    const float t2 = t * t;
    const float mt = 1.0f - t;
    val = g + ssigma * 2.0f * mt * t + t2 * (ssigma + ssigma * shadhi);
  }
  val += clarity * c * expf(-c * c / (2.0f * sigma * sigma / 3.0f));
  return val;
}

// the same curve with the two divisions by loop invariants replaced by
// products with their reciprocals, r2s = 1/(2 sigma), rden = 1/(2 sigma^2/3)
// (differs from llap_curve_fn by at most a few ulp before the f16 store)
DEV float llap_curve_rcp(float x, float g, float sigma, float r2s, float rden, float shadows, float highlights, float clarity)
{
  const float c = x - g;
  float val;
  const float ssigma = c > 0.0f ? sigma : -sigma;
  const float shadhi = c > 0.0f ? shadows : highlights;
  if(fabsf(c) > 2.0f * sigma) val = g + ssigma + shadhi * (c - ssigma);
  else
  {
    const float t = gclamp(c * (c > 0.0f ? r2s : -r2s), 0.0f, 1.0f);
    const float t2 = t * t;
    const float mt = 1.0f - t;
    val = g + ssigma * 2.0f * mt * t + t2 * (ssigma + ssigma * shadhi);
  }
  val += clarity * c * curve_exp(-c * c * rden);
  return val;
}

// the curve for shadows = highlights = 1 (the darkroom values): the linear
// part g + s + (c - s) and the quadratic bezier g + 2 s t, t = c / (2 s), are
// both x itself, which leaves x + clarity c exp(-c^2 / (2 sigma^2 / 3)); equal
// to llap_curve_fn up to the rounding of the operations it leaves out
DEV float llap_curve_unit(float x, float g, float rden, float clarity)
{
  const float c = x - g;
  return x + clarity * c * curve_exp(-c * c * rden);
}

// llap/reduce.comp (sample_semisoft) of one level 1 output from a level 0 plane
// staged in slot order: row[r] points at the slot of virtual x = 2 ox - 1 in the
// row of virtual y = 2 oy - 1 + r (4 byte aligned). The four bilinear taps at
// half texel offsets are ((t00/2 + t10/2)/2 + (t01/2 + t11/2)/2 ...)/4; halving is
// exact, so with the pair sums P = t0 + t1 the shader's value is
// ((((P00 + P10)/4 + (P01 + P11)/4) + (P10 + P20)/4) + (P11 + P21)/4)/4, and as
// scaling by a power of two commutes with rounding (no subnormal sums here) that
// is the same chain of sums scaled once by 1/16.
DEV float llap_reduce_px(const __half *const row[3])
{
  float P[3][2];
#pragma unroll
  for(int r = 0; r < 3; r++)
  {
    const __half2 a = *reinterpret_cast<const __half2 *>(row[r]);
    const float t0 = __low2float(a), t1 = __high2float(a), t2 = h2f(row[r][2]);
    P[r][0] = t0 + t1;
    P[r][1] = t1 + t2;
  }
  return (((((P[0][0] + P[1][0]) + (P[0][1] + P[1][1])) + (P[1][0] + P[2][0])) + (P[1][1] + P[2][1]))) * 0.0625f;
}

// The 10 curve planes of llap level 0 kept as five pairs (2j, 2j+1) of f16 in
// one 32 bit word: the curves of a pair and the level 1 reduce of a pair run
// as paired FP32 operations (add/mul/fma.f32x2, one instruction for both
// planes, each component rounded as the scalar operation rounds it).
constexpr int LLAP_PAIRS = 5;

// llap_curve_unit for planes 2j and 2j+1 of value x, rounded to f16
DEV __half2 llap_curve_unit2(float2 X, int j, float2 nrden, float2 cla)
{
  const float2 c = __fadd2_rn(X, make_float2(-kLlapGamma[2 * j], -kLlapGamma[2 * j + 1]));
  const float2 a = __fmul2_rn(__fmul2_rn(c, c), nrden);               // -c c rden
  const float2 e = make_float2(curve_exp(a.x), curve_exp(a.y));
  const float2 v = __ffma2_rn(__fmul2_rn(cla, c), e, X);             // x + clarity c e
  return __floats2half2_rn(v.x, v.y);
}

// llap_reduce_px for a pair of planes: r[k] points at the pair word of row k
// (virtual y = 2 oy - 1 + k) at virtual x = 2 ox - 1, r1[k] at 2 ox and r0[k]
// at 2 ox + 1 (the three taps of the row); the same sums in the same order
DEV float2 llap_reduce_px2(const __half2 *const a[3], const __half2 *const b[3], const __half2 *const c[3])
{
  float2 P[3][2];
#pragma unroll
  for(int r = 0; r < 3; r++)
  {
    const float2 t0 = __half22float2(*a[r]), t1 = __half22float2(*b[r]), t2 = __half22float2(*c[r]);
    P[r][0] = __fadd2_rn(t0, t1);
    P[r][1] = __fadd2_rn(t1, t2);
  }
  const float2 s = __fadd2_rn(__fadd2_rn(__fadd2_rn(__fadd2_rn(P[0][0], P[1][0]), __fadd2_rn(P[0][1], P[1][1])),
                                          __fadd2_rn(P[1][0], P[2][0])), __fadd2_rn(P[1][1], P[2][1]));
  return __fmul2_rn(s, make_float2(0.0625f, 0.0625f));
}

// histogram bin, bit exact with the oracle (see hist_log there for the method)
DEV float hist_log(float x)
{
  if(!(x > 0.0f)) return x == 0.0f ? -INFINITY : __int_as_float(0x7fc00000);
  if(x == INFINITY) return INFINITY;
  uint32_t u = __float_as_uint(x);
  int e = (int)((u >> 23) & 0xff);
  if(e == 0) { x = __fmul_rn(x, 8388608.0f); u = __float_as_uint(x); e = (int)((u >> 23) & 0xff) - 23; }
  e -= 127;
  u = (u & 0x007fffffu) | 0x3f800000u;
  float m = __uint_as_float(u);
  if(m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float s2 = __fmul_rn(s, s);
  float poly = 1.0f / 13.0f;
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f / 11.0f);
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f / 9.0f);
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f / 7.0f);
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f / 5.0f);
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f / 3.0f);
  poly = __fadd_rn(__fmul_rn(poly, s2), 1.0f);
  const float lm = __fmul_rn(__fmul_rn(2.0f, s), poly);
  const float fe = (float)e;
  const float hi = __fmul_rn(fe, 0.693145752f);
  const float lo = __fmul_rn(fe, 1.42860677e-06f);
  return __fadd_rn(hi, __fadd_rn(lo, lm));
}

// OpenDRT/hist.comp:15-20 get_bin
DEV uint32_t hist_bin(float r, float g, float b)
{
  const float v = lum2020(r, g, b);
  float l;
  if(v < 0.0f) l = __fadd_rn(__fmul_rn(v, 16.184376489665897f), 0.075f);
  else l = __fadd_rn(__fmul_rn(hist_log(__fadd_rn(v, 0.0057048244042473785f)), 0.09232902596577353f), 0.5520126568606655f);
  const float fb = __fadd_rn(__fmul_rn(256.0f, l), 0.5f);
  uint32_t bin;
  if(!(fb > 0.0f)) bin = 0;
  else if(fb >= 4294967295.0f) bin = 0xffffffffu;
  else bin = (uint32_t)fb;
  return bin > 255u ? 255u : bin;
}

