// Device check of the exact reciprocal and quotient helpers of common.cuh
// against the IEEE intrinsics: rcp_f16v on every f16 encoding and on the
// squares of all of them (every input it is used on), div_ry on random
// operands across the exponent range and on zeros, infinities, NaN and
// subnormals, noop_code against the code table's IEEE formula on every u16
// code for several black and white levels, and unorm16_exact (denoise.cuh)
// against the IEEE quotient on every u16 code. Prints the counts and exits
// non-zero on any difference.
#include "common.cuh"
#include "hilite.cuh"
#include "denoise.cuh"
#include <cstdio>

__device__ bool same(float a, float b) { return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b); }

__global__ void k_rcp(unsigned *bad)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= 65536) return;
  __half_raw hr;
  hr.x = (unsigned short)i;
  const float b = __half2float(__half(hr)), b2 = __fmul_rn(b, b);
  if(!same(rcp_f16v(b), __frcp_rn(b))) atomicAdd(bad, 1u);
  if(!same(rcp_f16v(b2), __frcp_rn(b2))) atomicAdd(bad + 1, 1u);
}

__device__ uint32_t mix(uint32_t x) { x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16; return x; }

__device__ float special(uint32_t h)
{
  const float s[8] = { 0.0f, -0.0f, INFINITY, -INFINITY, __int_as_float(0x7fc00000), 1e-40f, -3e-39f, 0x1p-61f };
  return s[h % 8];
}

__global__ void k_div(unsigned long long *cnt, int iters)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long fast = 0, bad = 0;
  for(int i = 0; i < iters; i++)
  {
    const uint32_t h1 = mix(t * 2654435761u + (uint32_t)i * 40503u), h2 = mix(h1 ^ 0x9e3779b9u), h3 = mix(h2 + 7u);
    const int ea = (int)(h3 % 161) - 80, eb = (int)((h3 >> 8) % 161) - 80;
    float a = __uint_as_float(((uint32_t)(ea + 127) << 23) | (h1 & 0x807fffffu));
    float b = __uint_as_float(((uint32_t)(eb + 127) << 23) | (h2 & 0x807fffffu));
    if(((h3 >> 20) & 31) == 0) a = special(h1 >> 7);
    if(((h3 >> 25) & 31) == 0) b = special(h2 >> 7);
    const bool ok = div_ok(b);
    const float q = div_ry(a, b, __frcp_rn(b), ok);
    if(ok && div_ok(a)) fast++;
    if(!same(q, __fdiv_rn(a, b))) bad++;
  }
  atomicAdd(cnt, fast);
  atomicAdd(cnt + 1, bad);
}

// every u16 code for 6 black / white pairs (DN): the table's formula (k_static.cu) against noop_code
__global__ void k_noop(unsigned *bad)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= 65536 * 6) return;
  const float bw[6][2] = { { 512, 16383 }, { 0, 65535 }, { 2048, 15000 }, { 64, 1023 }, { 600, 65535 }, { 1, 4095 } };
  const int v = i % 65536, c = i / 65536;
  dev_codes_t codes;
  codes.black = __fdiv_rn(bw[c][0], 65535.0f);
  codes.white = __fdiv_rn(bw[c][1], 65535.0f);
  codes.identity = 0;
  const float x = __fdiv_rn((float)v, 65535.0f);
  const __half want = __float2half_rn(fmaxf(0.0f, __fdiv_rn(__fsub_rn(x, codes.black), __fsub_rn(codes.white, codes.black))));
  const __half got = __float2half_rn(noop_code(noop_prep(codes), (uint32_t)v));
  if(__half_as_ushort(want) != __half_as_ushort(got)) atomicAdd(bad, 1u);
}

// every u16 code: unorm16_exact against the IEEE quotient of an R16_UNORM read
__global__ void k_unorm(unsigned *bad)
{
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if(v >= 65536) return;
  if(!same(unorm16_exact((uint32_t)v), __fdiv_rn((float)v, 65535.0f))) atomicAdd(bad, 1u);
}

int main()
{
  unsigned *d_bad;
  unsigned long long *d_cnt;
  if(cudaMalloc(&d_bad, 4 * sizeof(unsigned)) || cudaMalloc(&d_cnt, 2 * sizeof(unsigned long long))) return 2;
  cudaMemset(d_bad, 0, 4 * sizeof(unsigned));
  cudaMemset(d_cnt, 0, 2 * sizeof(unsigned long long));
  k_rcp<<<256, 256>>>(d_bad);
  k_div<<<152 * 4, 256>>>(d_cnt, 2048);
  k_noop<<<65536 * 6 / 256, 256>>>(d_bad + 2);
  k_unorm<<<256, 256>>>(d_bad + 3);
  unsigned bad[4];
  unsigned long long cnt[2];
  cudaMemcpy(bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost);
  cudaMemcpy(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  printf("rcp_f16v: %u of 65536 f16 values differ, %u of their squares\n", bad[0], bad[1]);
  printf("div_ry: %llu quotients on the corrected path, %llu differ from __fdiv_rn\n", cnt[0], cnt[1]);
  printf("noop_code: %u of 6 x 65536 codes differ from the code table\n", bad[2]);
  printf("unorm16_exact: %u of 65536 codes differ\n", bad[3]);
  printf("cuda: %s\n", cudaGetErrorString(e));
  return (e != cudaSuccess || bad[0] || bad[1] || bad[2] || bad[3] || cnt[1] || cnt[0] == 0) ? 1 : 0;
}
