// Ingestion of packed raw video on the device: the uncompressed magic lantern
// frame of i-mlv (video_mlv.c:254-274, which the reference unpacks on the
// host before the upload). The frame travels to the device packed (10, 12 or
// 14 bits per sample) and is unpacked here into the graph's u16 source.
//
// Pixel i is the 32-bit little-endian word made of the 16-bit words
// (i*bpp)/16 and (i*bpp)/16 + 1, rotated right by 16 + (32 - bpp) - (i*bpp)%16
// (a rotate: the amount counts modulo 32) and masked to bpp bits. A word past
// the frame reads 0; its bits are never selected.
#include <cstdint>
#include "kernels.h"

namespace {

constexpr int UP_PX = 8;   // pixels per thread: one 16-byte store

__global__ void __launch_bounds__(256) k_unpack_mlv(const uint16_t *__restrict__ words, size_t nwords, int bpp,
    size_t npix, uint16_t *__restrict__ out, int vec_store)
{
  const size_t i0 = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * UP_PX;
  if(i0 >= npix) return;
  const uint32_t mask = bpp >= 16 ? 0xffffu : (1u << bpp) - 1u;
  uint16_t v[UP_PX];
#pragma unroll
  for(int k = 0; k < UP_PX; k++)
  {
    const size_t i = i0 + k;
    const uint64_t off = (uint64_t)i * (uint64_t)bpp;
    const size_t a = (size_t)(off >> 4);
    const uint32_t r = (uint32_t)(48 - bpp - (int)(off & 15)) & 31u;
    const uint32_t w0 = a < nwords ? __ldg(words + a) : 0u;
    const uint32_t w1 = a + 1 < nwords ? __ldg(words + a + 1) : 0u;
    const uint32_t u = w0 | (w1 << 16);
    v[k] = (uint16_t)(__funnelshift_r(u, u, r) & mask);
  }
  if(vec_store && i0 + UP_PX <= npix)
  {
    uint4 q;
    q.x = v[0] | ((uint32_t)v[1] << 16); q.y = v[2] | ((uint32_t)v[3] << 16);
    q.z = v[4] | ((uint32_t)v[5] << 16); q.w = v[6] | ((uint32_t)v[7] << 16);
    *reinterpret_cast<uint4 *>(out + i0) = q;
  }
  else
  {
#pragma unroll
    for(int k = 0; k < UP_PX; k++) if(i0 + k < npix) out[i0 + k] = v[k];
  }
}

} // namespace

cudaError_t launch_unpack_mlv(const void *packed, size_t bytes, int bpp, size_t npix, uint16_t *out, cudaStream_t s)
{
  const int vec = ((uintptr_t)out & 15) == 0;
  const size_t threads = (npix + UP_PX - 1) / UP_PX;
  k_unpack_mlv<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(reinterpret_cast<const uint16_t *>(packed), bytes / 2,
                                                                 bpp, npix, out, vec);
  return cudaGetLastError();
}
