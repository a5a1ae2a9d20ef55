// Ingestion of motioncam raw video on the device (i-mcraw/prefix.comp and
// i-mcraw/decode.comp): a frame is a sequence of blocks of 64 samples, each
// a 4-bit bit count (two per byte), a u16 reference value and 0..128 bytes
// of deltas. Four consecutive blocks cover 64 x 4 pixels, one CFA phase each
// in steps of two pixels.
//
// k_mc_sizes: the bytes of every chunk of MC_CHUNK blocks; k_mc_scan (one
// CTA) turns them into the chunks' byte offsets.
// k_mc_decode: one CTA per chunk; the blocks' offsets are an exclusive scan in
// the CTA (integers: any order of addition gives the reference's offsets).
// The chunk's data is staged in shared memory with 8-byte loads, then a warp
// decodes a block, lane si the two deltas the shader's invocation si
// extracts; the samples are stored as the reference's R16_UNORM store of
// (reference + delta) / 65536 leaves them.
#include <cstdint>
#include "kernels.h"

namespace {

constexpr int MC_CHUNK = 256;           // blocks per CTA, one per thread (a 4096x2160 frame: 540 CTAs)
constexpr int MC_NT = 256;
constexpr int MC_STAGE = MC_CHUNK * 128; // the chunk's data: at most 128 bytes a block

__device__ __forceinline__ uint32_t mc_bytes(uint32_t cnt)
{ // i-mcraw/prefix.comp:46-63
  return cnt == 0 ? 0u : cnt <= 6 ? 8u * cnt : cnt <= 8 ? 64u : cnt <= 10 ? 80u : 128u;
}
__device__ __forceinline__ uint32_t mc_cnt(const uint8_t *__restrict__ bitcnt, uint32_t idx)
{
  uint32_t c = __ldg(bitcnt + idx / 2);
  if(idx & 1) c >>= 4;
  return c & 0xfu;
}
__device__ __forceinline__ uint32_t mc_bits(uint32_t v, int off, int n) { return (v >> off) & ((1u << n) - 1u); }

// the bytes of this chunk's blocks
__global__ void __launch_bounds__(MC_NT) k_mc_sizes(const uint8_t *__restrict__ bitcnt, uint32_t blocks,
    unsigned long long *__restrict__ chunk_bytes)
{
  __shared__ unsigned long long red[MC_NT / 32];
  const uint32_t b0 = blockIdx.x * MC_CHUNK;
  unsigned long long s = 0;
  for(uint32_t i = threadIdx.x; i < MC_CHUNK; i += MC_NT)
    if(b0 + i < blocks) s += mc_bytes(mc_cnt(bitcnt, b0 + i));
  for(int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if(threadIdx.x == 0)
  {
    unsigned long long t = 0;
    for(int w = 0; w < MC_NT / 32; w++) t += red[w];
    chunk_bytes[blockIdx.x] = t;
  }
}

// i-mcraw/decode.comp:31-282: the two deltas of invocation si of a block whose
// bytes start at d (n valid bytes; the rest read 0)
__device__ __forceinline__ void mc_pair(uint32_t cnt, const uint8_t *d, uint32_t n, int si, uint32_t r[2])
{
  auto byte = [&](int i) -> uint32_t { return (uint32_t)i < n ? (uint32_t)d[i] : 0u; };
  uint32_t p0, p1;
  auto pr = [&](int reg) { p0 = byte(reg); p1 = byte(reg + 1); };
  switch(cnt)
  {
    case 0: r[0] = r[1] = 0; return;
    case 1: pr(2 * (si % 4)); r[0] = mc_bits(p0, si / 4, 1); r[1] = mc_bits(p1, si / 4, 1); return;
    case 2: pr(2 * (si % 8)); r[0] = mc_bits(p0, 2 * (si / 8), 2); r[1] = mc_bits(p1, 2 * (si / 8), 2); return;
    case 3:
    {
      const int g = si / 4, k = si % 4;                       // groups of four invocations
      const int reg = (g / 3) * 8 + k * 2, off = (g % 3) * 3;   // g: 0..7 -> regs 0, 8, 16 and offsets 0, 3, 6
      pr(reg);
      r[0] = mc_bits(p0, off, 3); r[1] = mc_bits(p1, off, 3);
      if(g == 2 || g == 5)
      { // the third bit from regs 16..23, bit 6 (g 2) or 7 (g 5)
        pr(16 + k * 2);
        r[0] |= mc_bits(p0, g == 2 ? 6 : 7, 1) << 2; r[1] |= mc_bits(p1, g == 2 ? 6 : 7, 1) << 2;
      }
      return;
    }
    case 4:
    {
      pr((2 * si / 16) * 8 + (2 * si) % 8);
      const int off = ((2 * si / 8) & 1) == 0 ? 0 : 4;
      r[0] = mc_bits(p0, off, 4); r[1] = mc_bits(p1, off, 4);
      return;
    }
    case 5:
      if(si < 20) { pr(2 * si); r[0] = mc_bits(p0, 0, 5); r[1] = mc_bits(p1, 0, 5); return; }
      if(si < 28)
      {
        pr(si < 24 ? (si - 20) * 2 : 8 + (si - 24) * 2);
        const uint32_t l0 = p0, l1 = p1;
        pr(si < 24 ? 24 + (si - 20) * 2 : 32 + (si - 24) * 2);
        r[0] = mc_bits(l0, 5, 3) | (mc_bits(p0, 5, 2) << 3); r[1] = mc_bits(l1, 5, 3) | (mc_bits(p1, 5, 2) << 3);
        return;
      }
      {
        pr(16 + (si - 28) * 2); const uint32_t l0 = p0, l1 = p1;
        pr(24 + (si - 28) * 2); const uint32_t m0 = p0, m1 = p1;
        pr(32 + (si - 28) * 2);
        r[0] = mc_bits(l0, 5, 3) | (mc_bits(m0, 7, 1) << 3) | (mc_bits(p0, 7, 1) << 4);
        r[1] = mc_bits(l1, 5, 3) | (mc_bits(m1, 7, 1) << 3) | (mc_bits(p1, 7, 1) << 4);
      }
      return;
    case 6:
      if(si < 24) { pr(2 * si); r[0] = mc_bits(p0, 0, 6); r[1] = mc_bits(p1, 0, 6); return; }
      {
        const int b = si < 28 ? 0 : 24, k = si < 28 ? si - 24 : si - 28;
        pr(b + k * 2); const uint32_t l0 = p0, l1 = p1;
        pr(b + 8 + k * 2); const uint32_t m0 = p0, m1 = p1;
        pr(b + 16 + k * 2);
        r[0] = mc_bits(l0, 6, 2) | (mc_bits(m0, 6, 2) << 2) | (mc_bits(p0, 6, 2) << 4);
        r[1] = mc_bits(l1, 6, 2) | (mc_bits(m1, 6, 2) << 2) | (mc_bits(p1, 6, 2) << 4);
      }
      return;
    case 7: case 8: r[0] = byte(2 * si); r[1] = byte(2 * si + 1); return;
    case 9: case 10:
    {
      pr(si < 16 ? 2 * si : 40 + (si - 16) * 2);
      const uint32_t l0 = p0, l1 = p1;
      pr(si < 16 ? 32 + (si % 4) * 2 : 72 + (si % 4) * 2);
      const int off = 2 * ((si & 15) / 4);
      r[0] = l0 | (mc_bits(p0, off, 2) << 8); r[1] = l1 | (mc_bits(p1, off, 2) << 8);
      return;
    }
    default:
      r[0] = byte(4 * si) | (byte(4 * si + 1) << 8);
      r[1] = byte(4 * si + 2) | (byte(4 * si + 3) << 8);
      return;
  }
}

// the chunks' sizes into their exclusive offsets, in place (one CTA of 1024 threads)
__global__ void __launch_bounds__(1024) k_mc_scan(unsigned long long *__restrict__ cb, unsigned chunks)
{
  __shared__ unsigned long long wsum[32];
  __shared__ unsigned long long carry_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if(tid == 0) carry_s = 0;
  __syncthreads();
  for(unsigned b = 0; b < chunks; b += 1024)
  {
    const unsigned i = b + tid;
    const unsigned long long v = i < chunks ? cb[i] : 0ull;
    unsigned long long incl = v;
    for(int o = 1; o < 32; o <<= 1)
    {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
      if(lane >= o) incl += t;
    }
    if(lane == 31) wsum[warp] = incl;
    __syncthreads();
    unsigned long long before = carry_s;
    for(int w = 0; w < warp; w++) before += wsum[w];
    if(i < chunks) cb[i] = before + incl - v;
    __syncthreads();
    if(tid == 1023) carry_s = before + incl;
    __syncthreads();
  }
}

template<bool ALIGNED> __global__ void __launch_bounds__(MC_NT) k_mc_decode(const uint8_t *__restrict__ bitcnt,
    const uint16_t *__restrict__ refval, const uint8_t *__restrict__ data, size_t data_bytes, int rwd, int ht, int ox,
    int oy, int W, int H, const unsigned long long *__restrict__ chunk_off, uint16_t *__restrict__ out)
{
  __shared__ unsigned long long boff[MC_CHUNK];   // byte offset of each block of the chunk
  __shared__ unsigned long long red[MC_NT / 32];
  __shared__ __align__(16) uint8_t sd[MC_STAGE];
  __shared__ uint32_t scr[MC_CHUNK];              // bit count | reference << 8 of each block
  const uint32_t blocks = (uint32_t)rwd * (uint32_t)ht / 64;
  const uint32_t b0 = blockIdx.x * MC_CHUNK;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned long long base = chunk_off[blockIdx.x];
  // exclusive scan of the block sizes, one block per thread
  const uint32_t cnt0 = b0 + tid < blocks ? mc_cnt(bitcnt, b0 + tid) : 0u;
  const uint32_t sz = mc_bytes(cnt0);
  scr[tid] = cnt0 | (b0 + tid < blocks ? (uint32_t)__ldg(refval + b0 + tid) << 8 : 0u);
  unsigned long long incl = sz;
  for(int o = 1; o < 32; o <<= 1)
  {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if(lane >= o) incl += t;
  }
  if(lane == 31) red[warp] = incl;
  __syncthreads();
  unsigned long long wbase = 0;
  for(int w = 0; w < warp; w++) wbase += red[w];
  boff[tid] = base + wbase + incl - sz;
  unsigned long long total = 0;
  for(int w = 0; w < MC_NT / 32; w++) total += red[w];
  // stage the chunk's bytes (past data_bytes: 0), 8 at a time (block sizes are multiples of 8)
  for(unsigned long long w = tid; 8 * w < total; w += MC_NT)
  {
    const unsigned long long g = base + 8 * w;
    uint2 q = make_uint2(0u, 0u);
    if(ALIGNED && g + 8 <= data_bytes) q = __ldg(reinterpret_cast<const uint2 *>(data + g));
    else
    {
      uint32_t b[8];
#pragma unroll
      for(int k = 0; k < 8; k++) b[k] = g + k < data_bytes ? (uint32_t)__ldg(data + g + k) : 0u;
      q.x = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24);
      q.y = b[4] | (b[5] << 8) | (b[6] << 16) | (b[7] << 24);
    }
    *reinterpret_cast<uint2 *>(sd + 8 * w) = q;
  }
  __syncthreads();
  // decode: a warp per block
  const int bpr = rwd / 64;
  for(int j = warp; j < MC_CHUNK; j += MC_NT / 32)
  {
    const uint32_t idx = b0 + j;
    if(idx >= blocks) break;
    const uint32_t cr = scr[j], cnt = cr & 0xffu;
    const uint32_t o = (uint32_t)(boff[j] - base);
    uint32_t r[2];
    mc_pair(cnt, sd + o, (uint32_t)min((unsigned long long)128, total - o), lane, r);
    const uint32_t ref = cr >> 8;
    const uint32_t k = idx / 4;
    int x = 64 * (int)(k % bpr), y = 4 * (int)(k / bpr);
    if(lane >= 16) { x -= 64; y += 2; }
    x += (idx & 1) + 4 * lane - ox;
    y += ((idx >> 1) & 1) - oy;
#pragma unroll
    for(int c = 0; c < 2; c++)
    {
      const int px = x + 2 * c;
      if(px >= 0 && y >= 0 && px < W && y < H)
      { // R16_UNORM store of (ref + delta) / 65536
        const float v = fminf(fmaxf(__fdiv_rn((float)(r[c] + ref), 65536.0f), 0.0f), 1.0f);
        out[(size_t)y * W + px] = (uint16_t)__float2uint_rn(__fmul_rn(v, 65535.0f));
      }
    }
  }
}

} // namespace

size_t mcraw_scratch_bytes(int rwd, int ht)
{
  const size_t blocks = (size_t)rwd * ht / 64;
  return ((blocks + MC_CHUNK - 1) / MC_CHUNK) * sizeof(unsigned long long);
}

cudaError_t launch_mcraw_decode(const void *bitcnt, const void *refval, const void *data, size_t data_bytes, int rwd,
    int ht, int ox, int oy, int W, int H, void *scratch, uint16_t *out, cudaStream_t s)
{
  const uint32_t blocks = (uint32_t)((size_t)rwd * ht / 64);
  const unsigned chunks = (blocks + MC_CHUNK - 1) / MC_CHUNK;
  if(!chunks) return cudaSuccess;
  unsigned long long *cb = reinterpret_cast<unsigned long long *>(scratch);
  k_mc_sizes<<<chunks, MC_NT, 0, s>>>(reinterpret_cast<const uint8_t *>(bitcnt), blocks, cb);
  k_mc_scan<<<1, 1024, 0, s>>>(cb, chunks);
  if(((uintptr_t)data & 7) == 0)
    k_mc_decode<true><<<chunks, MC_NT, 0, s>>>(reinterpret_cast<const uint8_t *>(bitcnt), reinterpret_cast<const uint16_t *>(refval),
        reinterpret_cast<const uint8_t *>(data), data_bytes, rwd, ht, ox, oy, W, H, cb, out);
  else
    k_mc_decode<false><<<chunks, MC_NT, 0, s>>>(reinterpret_cast<const uint8_t *>(bitcnt), reinterpret_cast<const uint16_t *>(refval),
        reinterpret_cast<const uint8_t *>(data), data_bytes, rwd, ht, ox, oy, W, H, cb, out);
  return cudaGetLastError();
}
