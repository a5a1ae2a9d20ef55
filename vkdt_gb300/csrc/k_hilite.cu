// hilite module kernels (src/pipe/modules/hilite): the level 1 reduce fused
// with denoise/noop and hilite/half, and the pyramid reduce/assemble levels.
#include "common.cuh"
#include "hilite.cuh"
#include "kernels.h"

namespace {

constexpr int K1_T = 16;              // r1 outputs per tile side
constexpr int K1_N = 2 * K1_T + 3;    // h0 slots per side (5 tap support)

// denoise/noop.comp + hilite/half.comp + hilite/reduce.comp for one r1 tile.
// h0 (the half size image) lives only in shared memory.
DEV int mirror1c(int i, int n)
{ // mirrored repeat for |overshoot| < n, clamped beyond
  if(i < 0) i = -1 - i;
  if(i >= n) i = 2 * n - 1 - i;
  return min(max(i, 0), n - 1);
}

__global__ void __launch_bounds__(256) k_hilite_k1(const dev_hilite_k1_t p)
{
  // the reduce terms of every h0 texel of the tile (hilite_reduce_texel)
  __shared__ float st[5][K1_N][K1_N + 1];
  const int OX0 = blockIdx.x * K1_T, OY0 = blockIdx.y * K1_T;
  const int bx0 = 2 * OX0 - 2, by0 = 2 * OY0 - 2;
  const hl_reduce_t ra = hilite_reduce_args(p.hl_white, p.hl_desat, p.wb);
  const noop_eval_t nc = noop_prep(p.codes);
  for(int i = threadIdx.x; i < K1_N * K1_N; i += blockDim.x)
  {
    const int sx = i % K1_N, sy = i / K1_N;
    // outputs read h0 within 2 of the image: mirror1 is exact there; the
    // clamp keeps the slots past it (images narrower than a tile) in bounds
    const int hx = mirror1c(bx0 + sx, p.hw), hy = mirror1c(by0 + sy, p.hh);
    float h[3];
    const size_t row = (size_t)(2 * hy + p.cy) * p.pitch + 2 * hx + p.cx;
    const uint32_t r0 = __ldg(reinterpret_cast<const uint32_t *>(p.mosaic + row));
    const uint32_t r1 = __ldg(reinterpret_cast<const uint32_t *>(p.mosaic + row + p.pitch));
    const float m00 = noop_code(nc, r0 & 0xffff), m10 = noop_code(nc, r0 >> 16);
    const float m01 = noop_code(nc, r1 & 0xffff), m11 = noop_code(nc, r1 >> 16);
    hilite_half_bayer(m00, m10, m01, m11, p.hl_white, h);
    float t[5];
    hilite_reduce_texel(ra, h, t);
#pragma unroll
    for(int k = 0; k < 5; k++) st[k][sy][sx] = t[k];
  }
  __syncthreads();
  const int tx = threadIdx.x % K1_T, ty = threadIdx.x / K1_T;
  const int ox = OX0 + tx, oy = OY0 + ty;
  if(ox >= p.s1w || oy >= p.s1h) return;
  float o[4];
  hilite_reduce_sum([&](int ii, int jj, float t[5]) {
      const int sx = 2 * tx + 2 + ii, sy = 2 * ty + 2 + jj;
#pragma unroll
      for(int k = 0; k < 5; k++) t[k] = st[k][sy][sx];
    }, o);
  p.r1[(size_t)oy * p.s1w + ox] = mk_half4(o[0], o[1], o[2], o[3]);
}

struct reduce_args_t { float white, desat, wb[3]; };

// hilite/reduce.comp:21-61 on a stored level: 16x16 outputs per CTA, the
// reduce terms of the 35x35 input texels they read made once each
__global__ void __launch_bounds__(256) k_hilite_reduce(const half4 *__restrict__ in, int iw, int ih,
    half4 *__restrict__ out, int ow, int oh, const reduce_args_t a)
{
  __shared__ float st[5][K1_N][K1_N + 1];
  const int OX0 = blockIdx.x * K1_T, OY0 = blockIdx.y * K1_T;
  const int bx0 = 2 * OX0 - 2, by0 = 2 * OY0 - 2;
  const hl_reduce_t ra = hilite_reduce_args(a.white, a.desat, a.wb);
  // taps overshoot the level by at most 2: the cheap mirror is exact unless it is tiny
  const bool tiny = iw < 3 || ih < 3;
  for(int i = threadIdx.x; i < K1_N * K1_N; i += blockDim.x)
  {
    const int sx = i % K1_N, sy = i / K1_N;
    const int x = tiny ? mirror_full(bx0 + sx, iw) : mirror1c(bx0 + sx, iw);
    const int y = tiny ? mirror_full(by0 + sy, ih) : mirror1c(by0 + sy, ih);
    float rgb[3], w;
    ld_half4(in + (size_t)y * iw + x, rgb[0], rgb[1], rgb[2], w);
    float t[5];
    hilite_reduce_texel(ra, rgb, t);
#pragma unroll
    for(int k = 0; k < 5; k++) st[k][sy][sx] = t[k];
  }
  __syncthreads();
  const int tx = threadIdx.x % K1_T, ty = threadIdx.x / K1_T;
  const int x = OX0 + tx, y = OY0 + ty;
  if(x >= ow || y >= oh) return;
  float o[4];
  hilite_reduce_sum([&](int ii, int jj, float t[5]) {
      const int sx = 2 * tx + 2 + ii, sy = 2 * ty + 2 + jj;
#pragma unroll
      for(int k = 0; k < 5; k++) t[k] = st[k][sy][sx];
    }, o);
  out[(size_t)y * ow + x] = mk_half4(o[0], o[1], o[2], o[3]);
}

// hilite/assemble.comp:83-119 on stored levels
__global__ void __launch_bounds__(256) k_hilite_assemble(const half4 *__restrict__ fine, int fw, int fh,
    const half4 *__restrict__ coarse, int cw, int ch, half4 *__restrict__ out, float white, float soft)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= fw || y >= fh) return;
  float up[3];
  const bool tiny = cw < 2 || ch < 2;     // expand taps overshoot the coarse level by at most 1
  hilite_expand_px([&](int ix, int iy, float rgb[3]) {
      const int sx = tiny ? mirror_full(ix, cw) : mirror1c(ix, cw), sy = tiny ? mirror_full(iy, ch) : mirror1c(iy, ch);
      float w;
      ld_half4(coarse + (size_t)sy * cw + sx, rgb[0], rgb[1], rgb[2], w);
    }, x, y, up);
  float f[4];
  ld_half4(fine + (size_t)y * fw + x, f[0], f[1], f[2], f[3]);
  float o[3];
  hilite_assemble_px(f, up, white, soft, o);
  out[(size_t)y * fw + x] = mk_half4(o[0], o[1], o[2], 1.0f);
}

} // namespace

cudaError_t launch_hilite_k1(const dev_hilite_k1_t &p, cudaStream_t s)
{
  dim3 grid((p.s1w + K1_T - 1) / K1_T, (p.s1h + K1_T - 1) / K1_T);
  k_hilite_k1<<<grid, 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_hilite_reduce(const half4 *in, int iw, int ih, half4 *out, int ow, int oh,
    float white, float desat, const float wb[3], cudaStream_t s)
{
  reduce_args_t a = { white, desat, { wb[0], wb[1], wb[2] } };
  dim3 grid((ow + K1_T - 1) / K1_T, (oh + K1_T - 1) / K1_T);
  k_hilite_reduce<<<grid, 256, 0, s>>>(in, iw, ih, out, ow, oh, a);
  return cudaGetLastError();
}

cudaError_t launch_hilite_assemble(const half4 *fine, int fw, int fh, const half4 *coarse, int cw, int ch,
    half4 *out, float white, float soft, cudaStream_t s)
{
  dim3 grid((fw + 15) / 16, (fh + 15) / 16);
  k_hilite_assemble<<<grid, 256, 0, s>>>(fine, fw, fh, coarse, cw, ch, out, white, soft);
  return cudaGetLastError();
}
