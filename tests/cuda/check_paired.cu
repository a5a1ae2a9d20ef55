// Device check of the paired FP32 intrinsics (add/mul/fma.f32x2 through
// __fadd2_rn, __fmul2_rn, __ffma2_rn) against the scalar IEEE intrinsics.
// The operands live in memory as float2 (one 8 byte load per operand, so the
// paired form has its register pairs); the scalar results come from a kernel
// that handles one component per thread (nothing to pair). The host compares
// them bit for bit per operation and class of operand: normal operands across
// the exponent range, operands near the subnormal range, subnormal operands,
// and zeros, infinities and NaN; and the Markstein remainder a - q b of a
// correctly rounded quotient, which is exact only when the fma is fused. Two
// more lines compare a product followed by a sum, a b + c: as two paired
// operations, which the code generator contracts into one paired fma (one
// rounding instead of two), and as the demosaic covariance writes it, the
// paired product followed by scalar IEEE adds, which are never contracted;
// and the denoise structure tensor's form: the product as a paired fma whose
// addend is a -0 the compiler cannot see (exact: x + -0 = x), then a paired
// add, which has no product to contract with.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

static uint32_t mix(uint32_t x) { x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16; return x; }
static float operand(uint32_t h, int cls)
{
  if(cls == 3)
  {
    const float s[6] = { 0.0f, -0.0f, INFINITY, -INFINITY, NAN, 1.0f };
    return s[h % 6];
  }
  const int e = cls == 0 ? (int)((h >> 23) % 121) - 60 : cls == 1 ? -126 + (int)((h >> 23) % 8) : -127;
  const uint32_t u = ((uint32_t)(e + 127) << 23) | (h & 0x807fffffu);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

__global__ void k_pair(const float2 *a, const float2 *b, const float2 *c, float2 *o, int n, int op, float nz)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  const float2 x = a[i], y = b[i], z = c[i];
  o[i] = op == 0 ? __fadd2_rn(x, y) : op == 1 ? __fmul2_rn(x, y) : op == 2 ? __ffma2_rn(x, y, z)
       : op == 3 ? __fadd2_rn(__fmul2_rn(x, y), z)
       : op == 4 ? [&] { const float2 t = __fmul2_rn(x, y); return make_float2(__fadd_rn(t.x, z.x), __fadd_rn(t.y, z.y)); }()
       // the product as a paired fma with an addend of -0 the compiler cannot see (x + -0 = x for every x)
       : __fadd2_rn(__ffma2_rn(x, y, make_float2(nz, nz)), z);
}
__global__ void k_scalar(const float *a, const float *b, const float *c, float *o, int n, int op)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  o[i] = op == 0 ? __fadd_rn(a[i], b[i]) : op == 1 ? __fmul_rn(a[i], b[i]) : op == 2 ? __fmaf_rn(a[i], b[i], c[i])
       : __fadd_rn(__fmul_rn(a[i], b[i]), c[i]);
}

static bool same(float x, float y)
{
  uint32_t a, b;
  memcpy(&a, &x, 4); memcpy(&b, &y, 4);
  return a == b || (x != x && y != y);
}

int main()
{
  const int n = 1 << 22;   // pairs per class
  std::vector<float> ha(2 * n), hb(2 * n), hc(2 * n), hp(2 * n), hs(2 * n);
  float *da, *db, *dc, *dp, *ds;
  const size_t bytes = sizeof(float) * 2 * n;
  if(cudaMalloc(&da, bytes) || cudaMalloc(&db, bytes) || cudaMalloc(&dc, bytes) || cudaMalloc(&dp, bytes) || cudaMalloc(&ds, bytes))
  { printf("device allocation failed\n"); return 2; }
  const char *cls[5] = { "normal", "near subnormal", "subnormal", "special", "remainder" };
  const char *ops[6] = { "add", "mul", "fma", "paired mul+add", "paired mul, scalar add", "paired fma -0, paired add" };
  for(int c = 0; c < 5; c++)
  {
    uint32_t h = 12345u + 977u * c;
    for(int i = 0; i < 2 * n; i++)
    {
      h = mix(h + 0x9e3779b9u); const uint32_t h1 = h; h = mix(h + 0x9e3779b9u); const uint32_t h2 = h; h = mix(h + 0x9e3779b9u);
      if(c < 4)
      { // one operand of the class, the others normal (all of the class for class 0)
        ha[i] = operand(h1, c); hb[i] = operand(h2, c == 3 ? 0 : c); hc[i] = operand(h, 0);
      }
      else
      { // a, b normal, q = a / b rounded, fma(-q, b, a): the remainder
        const float a = operand(h1, 0), b = operand(h2, 0);
        ha[i] = -(a / b); hb[i] = b; hc[i] = a;
      }
    }
    cudaMemcpy(da, ha.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(db, hb.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dc, hc.data(), bytes, cudaMemcpyHostToDevice);
    printf("%-15s of %d components:", cls[c], 2 * n);
    for(int op = (c < 4 ? 0 : 2); op < (c == 0 ? 6 : 3); op++)
    {
      k_pair<<<(n + 255) / 256, 256>>>((const float2 *)da, (const float2 *)db, (const float2 *)dc, (float2 *)dp, n, op, -0.0f);
      k_scalar<<<(2 * n + 255) / 256, 256>>>(da, db, dc, ds, 2 * n, op > 4 ? 3 : op);
      if(cudaDeviceSynchronize() != cudaSuccess) { printf(" device error\n"); return 2; }
      cudaMemcpy(hp.data(), dp, bytes, cudaMemcpyDeviceToHost);
      cudaMemcpy(hs.data(), ds, bytes, cudaMemcpyDeviceToHost);
      long bad = 0;
      for(int i = 0; i < 2 * n; i++) bad += !same(hp[i], hs[i]);
      printf(" %s %ld", ops[op], bad);
    }
    printf(" differ\n");
  }
  cudaFree(da); cudaFree(db); cudaFree(dc); cudaFree(dp); cudaFree(ds);
  return 0;
}
