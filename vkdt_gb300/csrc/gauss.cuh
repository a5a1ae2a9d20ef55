// demosaic/gauss.comp (bayer) for one covariance entry, shared by the fused
// develop kernel and the per-node bayer gauss kernel.
#pragma once
#include "common.cuh"
#include "kernels.h"

// x / b for both components of a pair as div_ry does each (one reciprocal per
// component shared by its quotients; IEEE division outside div_ok's range)
DEV float2 div2_ry(float2 a, float2 b, float2 y, bool okx, bool oky)
{
  if(okx && oky && div_ok(a.x) && div_ok(a.y))
  {
    const float2 q = __fmul2_rn(a, y);
    return __ffma2_rn(__ffma2_rn(make_float2(-q.x, -q.y), b, a), y, q);
  }
  return make_float2(div_ry(a.x, b.x, y.x, okx), div_ry(a.y, b.y, y.y, oky));
}

// demosaic/gauss.comp:24-75 (bayer) for one entry, px the 8 greens around it
// in the shader's loop order: the covariance sums in the shader's order, each
// rounded on its own. They decide the form and the snapped direction, and on
// flat input the direction is a near tie: the sample positions alone have the
// covariance (1.25 -0.25; -0.25 1.25), eigenvectors at 45 degrees, so the snap
// there follows the last bits of the sums and is evaluated exactly. The two
// structure tensors (Sw of the greens, Sb of their reciprocals) are built side
// by side as pairs (w, b) where a paired FP32 instruction (add/mul/fma.f32x2)
// rounds each component as the scalar IEEE operation does: the weighted sums of
// the means (exact products), the differences to the means, the products, the
// sums and the quotients. A paired product that a paired sum consumes may be
// contracted into one fma by the code generator, so the products the sums take
// are paired fmas with an addend of -0 the compiler cannot see (nz, a kernel
// parameter; x + -0 = x for every x), which leave it nothing to contract; the
// determinant is scalar. The greens are f16
// values (the hilite output), so their reciprocals and those of their squares
// come from rcp_f16v; the quotients by the four sums share one correctly
// rounded reciprocal each (div_ry): the same IEEE results.
DEV void gauss_exact(const float px[8], float v[4], int &dec, float nz)
{
  const float2 z = make_float2(nz, nz);
  // sample values with their reciprocals: (px, 1/px)
  float2 pv[8];
#pragma unroll
  for(int k = 0; k < 8; k++) pv[k] = make_float2(px[k], rcp_f16v(px[k]));
  int k;
  // (mw0, mb0), (mw1, mb1), (smw, smb): i*px and i/px for i in {-1,0,1,2} are exact,
  // so the fused steps round only the sums
  float2 m0 = make_float2(0.0f, 0.0f), m1 = m0, sm = m0;
  k = 0;
#pragma unroll
  for(int j = -1; j < 3; j++)
#pragma unroll
  for(int ii = -1; ii < 3; ii++)
  {
    if(((j + ii) & 1) != 1) continue;
    m0 = __ffma2_rn(make_float2((float)ii, (float)ii), pv[k], m0);
    m1 = __ffma2_rn(make_float2((float)j, (float)j), pv[k], m1);
    sm = __fadd2_rn(sm, pv[k]);
    k++;
  }
  {
    const float2 y = make_float2(__frcp_rn(sm.x), __frcp_rn(sm.y));
    const bool okw = div_ok(sm.x), okb = div_ok(sm.y);
    m0 = div2_ry(m0, sm, y, okw, okb);
    m1 = div2_ry(m1, sm, y, okw, okb);
  }
  const float2 n0 = make_float2(-m0.x, -m0.y), n1 = make_float2(-m1.x, -m1.y);   // i - m as i + (-m): exact
  float2 S00 = make_float2(0.0f, 0.0f), S01 = S00, S10 = S00, S11 = S00, ss = S00;
  k = 0;
#pragma unroll
  for(int j = -1; j < 3; j++)
#pragma unroll
  for(int ii = -1; ii < 3; ii++)
  {
    if(((j + ii) & 1) != 1) continue;
    const float p2 = __fmul_rn(px[k], px[k]);
    const float2 P = make_float2(p2, rcp_f16v(p2));                  // (p2, 1/p2)
    const float2 q0 = __fadd2_rn(make_float2((float)ii, (float)ii), n0);
    const float2 q1 = __fadd2_rn(make_float2((float)j, (float)j), n1);
    const float2 a = __fmul2_rn(P, q0), b = __fmul2_rn(P, q1);
    S00 = __fadd2_rn(S00, __ffma2_rn(a, q0, z));
    S01 = __fadd2_rn(S01, __ffma2_rn(a, q1, z));
    S10 = __fadd2_rn(S10, __ffma2_rn(b, q0, z));
    S11 = __fadd2_rn(S11, __ffma2_rn(b, q1, z));
    ss = __fadd2_rn(ss, P);
    k++;
  }
  {
    const float2 y = make_float2(__frcp_rn(ss.x), __frcp_rn(ss.y));
    const bool okw = div_ok(ss.x), okb = div_ok(ss.y);
    S00 = div2_ry(S00, ss, y, okw, okb); S01 = div2_ry(S01, ss, y, okw, okb);
    S10 = div2_ry(S10, ss, y, okw, okb); S11 = div2_ry(S11, ss, y, okw, okb);
  }
  // (detw, detb) = S00 S11 - S10 S01 (scalar: a difference of products)
  const float2 det = make_float2(__fsub_rn(__fmul_rn(S00.x, S11.x), __fmul_rn(S10.x, S01.x)),
                                 __fsub_rn(__fmul_rn(S00.y, S11.y), __fmul_rn(S10.y, S01.y)));
  float eval[2], evec0[2], evec1[2];
  const bool usew = det.x < det.y;
  if(usew) evd2x2(eval, evec0, evec1, S00.x, S10.x, S11.x);
  else     evd2x2(eval, evec0, evec1, S00.y, S10.y, S11.y);
  eval[0] = __fmul_rn(eval[0], 0.2f); eval[1] = __fmul_rn(eval[1], 0.2f);
  const bool horiz = fabsf(evec0[0]) > fabsf(evec0[1]);
  if(horiz) { evec0[0] = 1.0f; evec0[1] = 0.0f; }
  else      { evec0[0] = 0.0f; evec0[1] = 1.0f; }
  v[0] = f16r(eval[0]); v[1] = f16r(eval[1]); v[2] = f16r(evec0[0]); v[3] = f16r(evec0[1]);
  dec = (usew ? GAUSS_DEC_USEW : 0) | ((horiz ? 0 : 1) << GAUSS_DEC_SNAP_SHIFT);
}
