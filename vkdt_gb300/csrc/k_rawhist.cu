// rawhist/collect.comp:22-66: noise statistics of a raw mosaic. Per CFA block
// the cross of greens (bayer: (1,0) and (0,1); x-trans: the 5 greens of the
// 3x3 block) gives a mean and a second moment of the black/white normalised
// values; the log2 of the mean picks one of `bins` bins, which count the
// blocks and sum their means and second moments.
//
// The reference adds floats atomically (an order dependent rounding). Here
// the sums are 64-bit fixed point (value * 2^36, values in [0, 1]): integer
// additions are associative, so every block's contribution is exact and the
// result does not depend on the order the blocks are added in. Each CTA
// accumulates in shared memory and adds its nonzero bins to the global sums;
// a last small kernel converts them to FP64. The bin index uses the
// project's correctly ordered natural log (pixel.cuh hist_log), so the oracle
// reproduces every count.
#include "common.cuh"
#include "kernels.h"
#include "pixel.cuh"

namespace {

constexpr int RH_MAXBINS = 1024;
constexpr double RH_SCALE = 68719476736.0;   // 2^36

DEV float rh_val(const dev_rawhist_t &p, int x, int y)
{ // texelFetch of the R16_UNORM mosaic (0 outside), normalised and clamped like collect.comp
  const float v = (x < p.wd && y < p.ht) ? __fdiv_rn((float)__ldg(p.mosaic + (size_t)y * p.pitch + x), 65535.0f) : 0.0f;
  return gclamp(__fdiv_rn(__fsub_rn(v, p.black), __fsub_rn(p.white, p.black)), 0.0f, 1.0f);
}

__global__ void __launch_bounds__(256) k_rawhist(const dev_rawhist_t p)
{
  __shared__ uint32_t cnt[RH_MAXBINS];
  __shared__ unsigned long long smean[RH_MAXBINS], smom[RH_MAXBINS];
  for(int i = threadIdx.x; i < p.bins; i += blockDim.x) { cnt[i] = 0; smean[i] = 0; smom[i] = 0; }
  __syncthreads();
  const int bx = blockIdx.x * 16 + threadIdx.x % 16, by = blockIdx.y * 16 + threadIdx.x / 16;
  if(bx < p.bw && by < p.bh)
  {
    float mean, mom2;
    if(p.filters == 9u)
    {
      const int x = 3 * bx, y = 3 * by;
      const float v0 = rh_val(p, x, y), v1 = rh_val(p, x + 2, y), v2 = rh_val(p, x + 1, y + 1);
      const float v3 = rh_val(p, x, y + 2), v4 = rh_val(p, x + 2, y + 2);
      mean = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v0, v1), v2), v3), v4), 5.0f);
      mom2 = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v0, v0), __fmul_rn(v1, v1)),
                 __fmul_rn(v2, v2)), __fmul_rn(v3, v3)), __fmul_rn(v4, v4)), 5.0f);
    }
    else
    {
      const int x = 2 * bx, y = 2 * by;
      const float v0 = rh_val(p, x + 1, y), v1 = rh_val(p, x, y + 1);
      mean = __fmul_rn(__fadd_rn(v0, v1), 0.5f);
      mom2 = __fmul_rn(__fadd_rn(__fmul_rn(v0, v0), __fmul_rn(v1, v1)), 0.5f);
    }
    // the bin: bins * log2(mean + 1), truncated like ivec2(x, 0); log2 as the
    // natural log of the histogram bins (the same operations in the oracle) / ln 2
    const float xb = __fmul_rn((float)p.bins, __fmul_rn(hist_log(__fadd_rn(mean, 1.0f)), 1.44269504f));
    const int bin = (int)xb;
    if(bin >= 0 && bin < p.bins)
    {
      atomicAdd(&cnt[bin], 1u);
      atomicAdd(&smean[bin], __double2ull_rn((double)mean * RH_SCALE));
      atomicAdd(&smom[bin], __double2ull_rn((double)mom2 * RH_SCALE));
    }
  }
  __syncthreads();
  for(int i = threadIdx.x; i < p.bins; i += blockDim.x)
    if(cnt[i])
    {
      atomicAdd(p.acc + i, (unsigned long long)cnt[i]);
      atomicAdd(p.acc + RH_MAXBINS + i, smean[i]);
      atomicAdd(p.acc + 2 * RH_MAXBINS + i, smom[i]);
    }
}

// the FP64 combine: counts and sums per bin
__global__ void k_rawhist_final(const unsigned long long *__restrict__ acc, int bins, double *__restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= bins) return;
  out[i] = (double)acc[i];
  out[bins + i] = (double)acc[RH_MAXBINS + i] / RH_SCALE;
  out[2 * bins + i] = (double)acc[2 * RH_MAXBINS + i] / RH_SCALE;
}

} // namespace

size_t rawhist_scratch_bytes() { return 3 * RH_MAXBINS * sizeof(unsigned long long) + 3 * RH_MAXBINS * sizeof(double); }
int rawhist_max_bins() { return RH_MAXBINS; }

cudaError_t launch_rawhist(const dev_rawhist_t &p, double *d_out, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(p.acc, 0, 3 * RH_MAXBINS * sizeof(unsigned long long), s);
  if(e != cudaSuccess) return e;
  k_rawhist<<<dim3((p.bw + 15) / 16, (p.bh + 15) / 16), 256, 0, s>>>(p);
  k_rawhist_final<<<(p.bins + 255) / 256, 256, 0, s>>>(p.acc, p.bins, d_out);
  return cudaGetLastError();
}
