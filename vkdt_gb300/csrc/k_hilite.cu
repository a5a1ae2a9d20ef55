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
  __shared__ float sh[3][K1_N][K1_N + 1];
  const int OX0 = blockIdx.x * K1_T, OY0 = blockIdx.y * K1_T;
  const int bx0 = 2 * OX0 - 2, by0 = 2 * OY0 - 2;
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
    const float m00 = h2f(__ldg(p.noop_lut + (r0 & 0xffff))), m10 = h2f(__ldg(p.noop_lut + (r0 >> 16)));
    const float m01 = h2f(__ldg(p.noop_lut + (r1 & 0xffff))), m11 = h2f(__ldg(p.noop_lut + (r1 >> 16)));
    hilite_half_bayer(m00, m10, m01, m11, p.hl_white, h);
    sh[0][sy][sx] = h[0]; sh[1][sy][sx] = h[1]; sh[2][sy][sx] = h[2];
  }
  __syncthreads();
  const int tx = threadIdx.x % K1_T, ty = threadIdx.x / K1_T;
  const int ox = OX0 + tx, oy = OY0 + ty;
  if(ox >= p.s1w || oy >= p.s1h) return;
  float o[4];
  hilite_reduce_px([&](int ii, int jj, float rgb[3]) {
      const int sx = 2 * tx + 2 + ii, sy = 2 * ty + 2 + jj;
      rgb[0] = sh[0][sy][sx]; rgb[1] = sh[1][sy][sx]; rgb[2] = sh[2][sy][sx];
    }, p.hl_white, p.hl_desat, p.wb, o);
  p.r1[(size_t)oy * p.s1w + ox] = mk_half4(o[0], o[1], o[2], o[3]);
}

struct reduce_args_t { float white, desat, wb[3]; };

// hilite/reduce.comp:21-61 on a stored level
__global__ void __launch_bounds__(256) k_hilite_reduce(const half4 *__restrict__ in, int iw, int ih,
    half4 *__restrict__ out, int ow, int oh, const reduce_args_t a)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= ow || y >= oh) return;
  float o[4];
  // taps overshoot the level by at most 2: the cheap mirror is exact unless it is tiny
  const bool tiny = iw < 3 || ih < 3;
  hilite_reduce_px([&](int ii, int jj, float rgb[3]) {
      const int sx = tiny ? mirror_full(2 * x + ii, iw) : mirror1c(2 * x + ii, iw);
      const int sy = tiny ? mirror_full(2 * y + jj, ih) : mirror1c(2 * y + jj, ih);
      float w;
      ld_half4(in + (size_t)sy * iw + sx, rgb[0], rgb[1], rgb[2], w);
    }, a.white, a.desat, a.wb, o);
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
  dim3 grid((ow + 15) / 16, (oh + 15) / 16);
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
