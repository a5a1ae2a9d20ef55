// demosaic/gauss.comp (bayer) for one covariance entry, shared by the fused
// develop kernel and the per-node bayer gauss kernel.
#pragma once
#include "common.cuh"
#include "kernels.h"

// demosaic/gauss.comp:24-75 (bayer) for one entry, px the 8 greens around it
// in the shader's loop order: the covariance sums in the shader's order
// without contraction. They decide the form and the snapped direction, and
// on flat input the direction is a near tie: the sample positions alone have
// the covariance (1.25 -0.25; -0.25 1.25), eigenvectors at 45 degrees, so the
// snap there follows the last bits of the sums and is evaluated exactly.
// The greens are f16 values (the hilite output), so their reciprocals and
// those of their squares come from rcp_f16v; the quotients by the four sums
// share one correctly rounded reciprocal each (div_ry): the same IEEE results.
DEV void gauss_exact(const float px[8], float v[4], int &dec)
{
  float inv[8];
#pragma unroll
  for(int k = 0; k < 8; k++) inv[k] = rcp_f16v(px[k]);
  int k;
  // i/px for i in {-1,0,1,2} is i*(1/px) exactly (scaling by +-1, 2 is exact)
  float mw0 = 0, mw1 = 0, mb0 = 0, mb1 = 0, smw = 0, smb = 0;
  k = 0;
#pragma unroll
  for(int j = -1; j < 3; j++)
#pragma unroll
  for(int ii = -1; ii < 3; ii++)
  {
    if(((j + ii) & 1) != 1) continue;
    mw0 += (float)ii * px[k]; mw1 += (float)j * px[k];
    smw += px[k];
    mb0 += (float)ii * inv[k]; mb1 += (float)j * inv[k];
    smb += inv[k];
    k++;
  }
  // (the products above are exact, so contraction cannot change them;
  // the covariance sums below decide the snapped direction and are
  // evaluated without contraction, in the shader's order)
  {
    const float yw = __frcp_rn(smw), yb = __frcp_rn(smb);
    const bool okw = div_ok(smw), okb = div_ok(smb);
    mw0 = div_ry(mw0, smw, yw, okw); mw1 = div_ry(mw1, smw, yw, okw);
    mb0 = div_ry(mb0, smb, yb, okb); mb1 = div_ry(mb1, smb, yb, okb);
  }
  float Sw00 = 0, Sw01 = 0, Sw10 = 0, Sw11 = 0, Sb00 = 0, Sb01 = 0, Sb10 = 0, Sb11 = 0, sw = 0, sb = 0;
  k = 0;
#pragma unroll
  for(int j = -1; j < 3; j++)
#pragma unroll
  for(int ii = -1; ii < 3; ii++)
  {
    if(((j + ii) & 1) != 1) continue;
    float p2 = __fmul_rn(px[k], px[k]);
    float q0 = __fsub_rn((float)ii, mw0), q1 = __fsub_rn((float)j, mw1);
    Sw00 = __fadd_rn(Sw00, __fmul_rn(__fmul_rn(p2, q0), q0));
    Sw01 = __fadd_rn(Sw01, __fmul_rn(__fmul_rn(p2, q0), q1));
    Sw10 = __fadd_rn(Sw10, __fmul_rn(__fmul_rn(p2, q1), q0));
    Sw11 = __fadd_rn(Sw11, __fmul_rn(__fmul_rn(p2, q1), q1));
    sw = __fadd_rn(sw, p2);
    q0 = __fsub_rn((float)ii, mb0); q1 = __fsub_rn((float)j, mb1);
    p2 = rcp_f16v(p2);
    Sb00 = __fadd_rn(Sb00, __fmul_rn(__fmul_rn(p2, q0), q0));
    Sb01 = __fadd_rn(Sb01, __fmul_rn(__fmul_rn(p2, q0), q1));
    Sb10 = __fadd_rn(Sb10, __fmul_rn(__fmul_rn(p2, q1), q0));
    Sb11 = __fadd_rn(Sb11, __fmul_rn(__fmul_rn(p2, q1), q1));
    sb = __fadd_rn(sb, p2);
    k++;
  }
  {
    const float yw = __frcp_rn(sw), yb = __frcp_rn(sb);
    const bool okw = div_ok(sw), okb = div_ok(sb);
    Sw00 = div_ry(Sw00, sw, yw, okw); Sw01 = div_ry(Sw01, sw, yw, okw);
    Sw10 = div_ry(Sw10, sw, yw, okw); Sw11 = div_ry(Sw11, sw, yw, okw);
    Sb00 = div_ry(Sb00, sb, yb, okb); Sb01 = div_ry(Sb01, sb, yb, okb);
    Sb10 = div_ry(Sb10, sb, yb, okb); Sb11 = div_ry(Sb11, sb, yb, okb);
  }
  const float detw = __fsub_rn(__fmul_rn(Sw00, Sw11), __fmul_rn(Sw10, Sw01));
  const float detb = __fsub_rn(__fmul_rn(Sb00, Sb11), __fmul_rn(Sb10, Sb01));
  float eval[2], evec0[2], evec1[2];
  const bool usew = detw < detb;
  if(usew) evd2x2(eval, evec0, evec1, Sw00, Sw10, Sw11);
  else     evd2x2(eval, evec0, evec1, Sb00, Sb10, Sb11);
  eval[0] = __fmul_rn(eval[0], 0.2f); eval[1] = __fmul_rn(eval[1], 0.2f);
  const bool horiz = fabsf(evec0[0]) > fabsf(evec0[1]);
  if(horiz) { evec0[0] = 1.0f; evec0[1] = 0.0f; }
  else      { evec0[0] = 0.0f; evec0[1] = 1.0f; }
  v[0] = f16r(eval[0]); v[1] = f16r(eval[1]); v[2] = f16r(evec0[0]); v[3] = f16r(evec0[1]);
  dec = (usew ? GAUSS_DEC_USEW : 0) | ((horiz ? 0 : 1) << GAUSS_DEC_SNAP_SHIFT);
}

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

// The same entry with the two structure tensors (Sw of the greens, Sb of their
// reciprocals) built side by side as pairs (w, b), each pair operation one
// paired FP32 instruction (add/mul/fma.f32x2) whose components round as the
// scalar IEEE operations of the shader's order do. Only for greens that are
// all positive and finite: a zero green gives an infinite reciprocal, whose
// product with a zero weight must stay NaN as in the shader, and the paired
// form is not relied on for that (gauss_exact takes those entries).
DEV void gauss_exact_paired(const float px[8], float v[4], int &dec)
{
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
    S00 = __fadd2_rn(S00, __fmul2_rn(a, q0));
    S01 = __fadd2_rn(S01, __fmul2_rn(a, q1));
    S10 = __fadd2_rn(S10, __fmul2_rn(b, q0));
    S11 = __fadd2_rn(S11, __fmul2_rn(b, q1));
    ss = __fadd2_rn(ss, P);
    k++;
  }
  {
    const float2 y = make_float2(__frcp_rn(ss.x), __frcp_rn(ss.y));
    const bool okw = div_ok(ss.x), okb = div_ok(ss.y);
    S00 = div2_ry(S00, ss, y, okw, okb); S01 = div2_ry(S01, ss, y, okw, okb);
    S10 = div2_ry(S10, ss, y, okw, okb); S11 = div2_ry(S11, ss, y, okw, okb);
  }
  // (detw, detb) = S00 S11 - S10 S01, the difference as a sum with the negated product
  const float2 d1 = __fmul2_rn(S00, S11), d2 = __fmul2_rn(S10, S01);
  const float2 det = __fadd2_rn(d1, make_float2(-d2.x, -d2.y));
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

// the entry by the paired form where its greens allow it (positive, finite: the
// usual case), else by the scalar form
DEV void gauss_entry(const float px[8], float v[4], int &dec)
{
  bool ok = true;
#pragma unroll
  for(int k = 0; k < 8; k++) ok = ok && px[k] > 0.0f && px[k] < INFINITY;
  if(ok) gauss_exact_paired(px, v, dec);
  else   gauss_exact(px, v, dec);
}
