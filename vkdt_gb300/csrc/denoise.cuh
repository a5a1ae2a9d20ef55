// exact helpers of the wavelet denoise kernels (k_denoise.cu)
#pragma once
#include "common.cuh"

// v / 65535 correctly rounded for a u16 code v (an R16_UNORM read): the
// quotient correction of div_ry from y = RN(1/65535) without its guard, as
// every code and every quotient is zero or normal. Equal to
// __fdiv_rn((float)v, 65535.0f) on all 65536 codes (checked on the device).
DEV float unorm16_exact(uint32_t v)
{
  constexpr float y = 1.0f / 65535.0f;
  const float a = (float)v, q = __fmul_rn(a, y);
  return __fmaf_rn(__fmaf_rn(-q, 65535.0f, a), y, q);
}
