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
