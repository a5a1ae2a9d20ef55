// Per pixel bodies of colour/main and filmcurv/main, shared by the fused
// develop kernel and the per-node kernels.
#pragma once
#include "common.cuh"
#include "kernels.h"
#include "pixel.cuh"

// colour/main-impl.glsl:200-341 on the matrix path (no clut/pick/rbf, sat 1):
// camera matrix, CAT16 in, cone scale, CAT16 out and exposure, linear in the
// pixel, applied as their product cmat (made by the host per image)
DEV void colour_px(const dev_image_t &p, const float in[3], float o[3])
{
  for(int i = 0; i < 3; i++)
    o[i] = f16r(gclamp(p.cmat[3 * i + 0] * in[0] + p.cmat[3 * i + 1] * in[1] + p.cmat[3 * i + 2] * in[2],
                       -65535.0f, 65535.0f));
}

// filmcurv/main.comp:106-205, colour modes 1 and 3 (adjust_colour_dng,
// shared.glsl:371-387). pow as GPUs evaluate GLSL pow: exp2(k log2 x), on the
// special function unit (the result is stored as f16)
DEV void filmcurv_px(const dev_image_t &p, const float in[3], float o[3])
{
  float c0[3], c1[3];
  for(int k = 0; k < 3; k++) c0[k] = in[k] + p.fc_bias;
  for(int k = 0; k < 3; k++) c1[k] = 1.0f - curve_exp(-__powf(fmaxf(c0[k], 1e-7f) * p.fc_il, p.fc_k));
  if(p.fc_mode == 3)
  {
    bool fx = false, fy = false, fz = false;
    float t;
    if(c0[2] > c0[1]) { t = c0[2]; c0[2] = c0[1]; c0[1] = t; t = c1[2]; c1[2] = c1[1]; c1[1] = t; fx = true; }
    if(c0[1] > c0[0]) { t = c0[0]; c0[0] = c0[1]; c0[1] = t; t = c1[0]; c1[0] = c1[1]; c1[1] = t; fy = true; }
    if(c0[2] > c0[1]) { t = c0[2]; c0[2] = c0[1]; c0[1] = t; t = c1[2]; c1[2] = c1[1]; c1[1] = t; fz = true; }
    c1[1] = gmix(c1[2], c1[0], (c0[1] - c0[2] + 1e-6f) / (c0[0] - c0[2] + 1e-6f));
    if(fz) { t = c1[2]; c1[2] = c1[1]; c1[1] = t; }
    if(fy) { t = c1[0]; c1[0] = c1[1]; c1[1] = t; }
    if(fx) { t = c1[2]; c1[2] = c1[1]; c1[1] = t; }
  }
  for(int k = 0; k < 3; k++) o[k] = f16r(c1[k]);
}
