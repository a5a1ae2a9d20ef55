// Device check of the paired FP32 intrinsics (add/mul/fma.f32x2 through
// __fadd2_rn, __fmul2_rn, __ffma2_rn) against the scalar IEEE intrinsics, per
// component, on random operands across the exponent range, on subnormal
// results and inputs, and on zeros, infinities and NaN. The kernels use the
// paired forms where a value only feeds continuous arithmetic; this records
// whether they may also stand where a result decides a branch. Prints the
// counts per operation and class of operand.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>

__device__ bool same(float a, float b) { return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b); }
__device__ uint32_t mix(uint32_t x) { x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16; return x; }

// an operand: class 0 normal in 2^-60..2^60, 1 near the subnormal range, 2 subnormal, 3 special
__device__ float operand(uint32_t h, int cls)
{
  if(cls == 3)
  {
    const float s[6] = { 0.0f, -0.0f, INFINITY, -INFINITY, __int_as_float(0x7fc00000), 1.0f };
    return s[h % 6];
  }
  const int e = cls == 0 ? (int)((h >> 23) % 121) - 60 : cls == 1 ? -126 + (int)((h >> 23) % 8) : -127;
  return __uint_as_float(((uint32_t)(e + 127) << 23) | (h & 0x807fffffu));
}

// cnt[3 * cls + op]: differing components of add (0), mul (1), fma (2)
__global__ void k_paired(unsigned long long *cnt, int iters)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  for(int i = 0; i < iters; i++)
  {
    const int cls = i & 3;
    uint32_t h = mix(t * 2654435761u + (uint32_t)i * 40503u);
    float v[6];
    for(int k = 0; k < 6; k++) { v[k] = operand(h, (k == 0 || cls == 0) ? cls : 0); h = mix(h + 0x9e3779b9u); }
    const float2 a = make_float2(v[0], v[1]), b = make_float2(v[2], v[3]), c = make_float2(v[4], v[5]);
    const float2 s = __fadd2_rn(a, b), m = __fmul2_rn(a, b), f = __ffma2_rn(a, b, c);
    unsigned long long d0 = !same(s.x, __fadd_rn(a.x, b.x)) + !same(s.y, __fadd_rn(a.y, b.y));
    unsigned long long d1 = !same(m.x, __fmul_rn(a.x, b.x)) + !same(m.y, __fmul_rn(a.y, b.y));
    unsigned long long d2 = !same(f.x, __fmaf_rn(a.x, b.x, c.x)) + !same(f.y, __fmaf_rn(a.y, b.y, c.y));
    if(d0) atomicAdd(cnt + 3 * cls + 0, d0);
    if(d1) atomicAdd(cnt + 3 * cls + 1, d1);
    if(d2) atomicAdd(cnt + 3 * cls + 2, d2);
  }
}

// the exact remainder of a correctly rounded quotient, r = a - q b (Markstein): fused it is exact
__global__ void k_remainder(unsigned long long *cnt, int iters)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  for(int i = 0; i < iters; i++)
  {
    uint32_t h = mix(t * 747796405u + (uint32_t)i * 2891336453u);
    const float a = operand(h, 0), b = operand(mix(h + 1u), 0), a2 = operand(mix(h + 2u), 0), b2 = operand(mix(h + 3u), 0);
    const float q = __fdiv_rn(a, b), q2 = __fdiv_rn(a2, b2);
    const float2 r = __ffma2_rn(make_float2(-q, -q2), make_float2(b, b2), make_float2(a, a2));
    const unsigned long long d = !same(r.x, __fmaf_rn(-q, b, a)) + !same(r.y, __fmaf_rn(-q2, b2, a2));
    if(d) atomicAdd(cnt, d);
  }
}

int main()
{
  unsigned long long *d, h[13] = { 0 };
  cudaMalloc(&d, sizeof(h));
  cudaMemset(d, 0, sizeof(h));
  const int blocks = 152 * 4, threads = 256, iters = 256;
  k_paired<<<blocks, threads>>>(d, iters);
  k_remainder<<<blocks, threads>>>(d + 12, iters);
  if(cudaDeviceSynchronize() != cudaSuccess) { printf("device error\n"); return 2; }
  cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  const unsigned long long n = (unsigned long long)blocks * threads * iters / 4 * 2;   // components per class
  const char *cls[4] = { "normal", "near subnormal", "subnormal", "special" };
  for(int c = 0; c < 4; c++)
    printf("%-15s of %llu components: add %llu, mul %llu, fma %llu differ\n", cls[c], n, h[3 * c], h[3 * c + 1], h[3 * c + 2]);
  printf("quotient remainders: %llu of %llu differ\n", h[12], (unsigned long long)blocks * threads * iters * 2);
  return 0;
}
