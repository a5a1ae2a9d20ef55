// Fixed device scratch of vkdt_cuda_graph_develop_static, and the kernel that
// fills the denoise/noop code table inside it.
//
// Some callers cannot allocate device memory at the moment they want a
// develop: a display or video callback that runs while other streams are busy
// (cudaMalloc and cudaFree may synchronise the device and stall them), code
// that runs under a memory budget it does not own, or an embedding that has
// handed every allocation to its own pool. For them the intermediate buffers
// of a small develop (previews, thumbnails) live in one array that the CUDA
// module reserves when it loads, so the call itself allocates nothing.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "vkdt_cuda.h"
#include "kernels.h"

namespace {

// one per device, reserved when the module loads; every call shares it
static __device__ __align__(256) unsigned char g_static_scratch[VKDT_CUDA_STATIC_SCRATCH_BYTES];

// denoise/noop.comp:36-57 for every u16 code: max(0, (v/65535 - black)/(white - black)) as f16,
// in IEEE single precision as the host builds the same table for allocated graphs
__global__ void __launch_bounds__(256) k_noop_lut(__half *__restrict__ lut, float black, float white)
{
  const int v = blockIdx.x * 256 + threadIdx.x;
  const float x = __fdiv_rn((float)v, 65535.0f);
  lut[v] = __float2half_rn(fmaxf(0.0f, __fdiv_rn(__fsub_rn(x, black), __fsub_rn(white, black))));
}

} // namespace

cudaError_t static_scratch_address(void **ptr)
{
  return cudaGetSymbolAddress(ptr, g_static_scratch);
}

cudaError_t launch_noop_lut(__half *lut, float black, float white, cudaStream_t s)
{
  k_noop_lut<<<65536 / 256, 256, 0, s>>>(lut, black, white);
  return cudaGetLastError();
}
