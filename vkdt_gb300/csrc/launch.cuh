// kernel launches with programmatic dependent launch (PDL): the next kernel of
// a stream may be scheduled while the previous one drains, so its CTAs are
// resident when that one completes. Every kernel launched this way calls
// pdl_begin() (common.cuh) as its first statement: it waits there until the
// previous kernel of the stream has completed and its writes are visible, so
// the ordering of the stream is kept for every memory access.
#pragma once
#include <cuda_runtime.h>
#include <utility>

template<typename... K, typename... A>
inline cudaError_t launch_pdl(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A &&... args)
{
  cudaLaunchAttribute at;
  at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at.val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = &at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}
