// Synthetic scene generation, the standalone histogram (OpenDRT/hist.comp) and
// the rgb waveform (hist/collect.comp).
#include "common.cuh"
#include "kernels.h"
#include "scene.h"
#include "pixel.cuh"

#include <algorithm>

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

// hist/collect.comp:13-26: the rgb waveform. Input column x lands in output
// column int(scale x) (scale = output width / input width), each channel at
// row (1 - value) * height + 0.5 converted to an unsigned integer (negative
// and NaN to 0, as the GPU conversion saturates) and clamped to the last row;
// red adds 1, green 1024, blue 1048576 (three 10-bit counters per u32).
// A CTA owns a strip of input columns and a band of rows; its output columns
// (c0 .. c0 + ncols - 1) are counted in shared memory, then added to the
// image. Integer sums: the counts are exact whatever the order.
DEV uint32_t wf_row(float v, int ho)
{
  const float t = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, v), (float)ho), 0.5f);
  const uint32_t u = t >= 4294967296.0f ? 0xffffffffu : (t > 0.0f ? (uint32_t)t : 0u);
  return min(u, (uint32_t)(ho - 1));
}
DEV int wf_col(float scale, int x, int wo)
{
  return min(max((int)__fmul_rn(scale, (float)x), 0), wo - 1);
}

__global__ void __launch_bounds__(256) k_waveform(const half4 *__restrict__ in, int W, int H, uint32_t *__restrict__ out,
    int wo, int ho, float scale, int tx, int ty, int ncols)
{
  extern __shared__ uint32_t wh[];   // ncols x ho, or none (ncols 0: straight to the image)
  const int x0 = blockIdx.x * tx, y0 = blockIdx.y * ty;
  const int c0 = wf_col(scale, x0, wo);
  for(int i = threadIdx.x; i < ncols * ho; i += blockDim.x) wh[i] = 0;
  __syncthreads();
  const int xe = min(x0 + tx, W), ye = min(y0 + ty, H);
  const int n = (xe - x0) * (ye - y0);
  for(int i = threadIdx.x; i < n; i += blockDim.x)
  {
    const int x = x0 + i % (xe - x0), y = y0 + i / (xe - x0);
    float r, g, b, a;
    ld_half4(in + (size_t)y * W + x, r, g, b, a);
    const int c = wf_col(scale, x, wo);
    const uint32_t yr = wf_row(r, ho), yg = wf_row(g, ho), yb = wf_row(b, ho);
    const int lc = c - c0;
    if(ncols && lc >= 0 && lc < ncols)
    {
      atomicAdd(&wh[yr * ncols + lc], 1u);
      atomicAdd(&wh[yg * ncols + lc], 1024u);
      atomicAdd(&wh[yb * ncols + lc], 1048576u);
    }
    else
    {
      atomicAdd(out + (size_t)yr * wo + c, 1u);
      atomicAdd(out + (size_t)yg * wo + c, 1024u);
      atomicAdd(out + (size_t)yb * wo + c, 1048576u);
    }
  }
  if(!ncols) return;
  __syncthreads();
  for(int i = threadIdx.x; i < ncols * ho; i += blockDim.x)
  {
    const int lc = i % ncols, row = i / ncols;
    if(wh[i] && c0 + lc < wo) atomicAdd(out + (size_t)row * wo + c0 + lc, wh[i]);
  }
}

} // namespace

cudaError_t launch_waveform(const half4 *in, int W, int H, uint32_t *out, int wo, int ho, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)wo * ho * sizeof(uint32_t), s);  // s_conn_clear
  if(e != cudaSuccess) return e;
  const float scale = (float)wo / (float)W;
  // strips of input columns whose output columns fit 48 KB of counters (at most 64 columns);
  // the widest strip is counted exactly with the kernel's own column map
  int tx = 0, ncols = 0;
  const int budget = (int)(48 * 1024 / (4 * ho));
  if(budget >= 2)
  {
    tx = 256;
    for(;;)
    {
      ncols = 0;
      for(int x0 = 0; x0 < W; x0 += tx)
      {
        const int xl = std::min(x0 + tx, W) - 1;
        const int c0 = std::min(std::max((int)(scale * (float)x0), 0), wo - 1);
        const int c1 = std::min(std::max((int)(scale * (float)xl), 0), wo - 1);
        ncols = std::max(ncols, c1 - c0 + 1);
      }
      if(ncols <= std::min(budget, 64) || tx == 1) break;
      tx /= 2;
    }
    if(ncols > std::min(budget, 64)) { tx = 256; ncols = 0; }
  }
  else tx = 256;
  const int ty = 256;
  dim3 grid((W + tx - 1) / tx, (H + ty - 1) / ty);
  k_waveform<<<grid, 256, (size_t)ncols * ho * 4, s>>>(in, W, H, out, wo, ho, scale, tx, ty, ncols);
  return cudaGetLastError();
}

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
