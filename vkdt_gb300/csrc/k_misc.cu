// Synthetic scene generation and the standalone histogram (OpenDRT/hist.comp).
#include "common.cuh"
#include "kernels.h"
#include "scene.h"
#include "pixel.cuh"

namespace {

__global__ void __launch_bounds__(256) k_scene(const scene_layout_t *__restrict__ s, uint16_t *__restrict__ out)
{
  __shared__ scene_layout_t sl;
  for(int i = threadIdx.x; i < (int)(sizeof(scene_layout_t) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t *>(&sl)[i] = reinterpret_cast<const uint32_t *>(s)[i];
  __syncthreads();
  const int x = blockIdx.x * 64 + threadIdx.x % 64, y = blockIdx.y * 4 + threadIdx.x / 64;
  if(x >= sl.wd || y >= sl.ht) return;
  out[(size_t)y * sl.wd + x] = scene_pixel(&sl, x, y);
}

// OpenDRT/hist.comp:22-45: 256 bins of T-Log luminance, bin 0 skipped, count in [256]
__global__ void __launch_bounds__(256) k_hist(const half4 *__restrict__ in, int W, int H, uint32_t *__restrict__ hist)
{
  __shared__ uint32_t lh[257];
  for(int i = threadIdx.x; i < 257; i += blockDim.x) lh[i] = 0;
  __syncthreads();
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x < W && y < H)
  {
    float r, g, b, a;
    ld_half4(in + (size_t)y * W + x, r, g, b, a);
    const uint32_t bin = hist_bin(r, g, b);
    if(bin > 0) { atomicAdd(&lh[bin], 1u); atomicAdd(&lh[256], 1u); }
  }
  __syncthreads();
  for(int i = threadIdx.x; i < 257; i += blockDim.x) if(lh[i]) atomicAdd(hist + i, lh[i]);
}

} // namespace

cudaError_t launch_scene(const scene_layout_t *d_layout, int wd, int ht, uint16_t *out, cudaStream_t s)
{
  dim3 grid((wd + 63) / 64, (ht + 3) / 4);
  k_scene<<<grid, 256, 0, s>>>(d_layout, out);
  return cudaGetLastError();
}

cudaError_t launch_hist_rgba(const half4 *in, int W, int H, uint32_t *hist, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(hist, 0, 257 * sizeof(uint32_t), s);
  if(e != cudaSuccess) return e;
  dim3 grid((W + 15) / 16, (H + 15) / 16);
  k_hist<<<grid, 256, 0, s>>>(in, W, H, hist);
  return cudaGetLastError();
}
