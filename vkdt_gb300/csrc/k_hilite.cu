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

// hilite/assemble.comp:83-119 on stored levels: 16x16 outputs per CTA, a
// warp takes outputs of one (x, y) parity, so its expand taps and weights
// are fixed (hilite_expand_px_t)
template<int DX, int DY> DEV void assemble_one(const half4 *__restrict__ fine, int fw, const half4 *__restrict__ coarse,
    int cw, int ch, bool tiny, int x, int y, half4 *__restrict__ out, float white, float soft)
{
  float up[3];
  hilite_expand_px_t<DX, DY>([&](int ix, int iy, float rgb[3]) {
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

__global__ void __launch_bounds__(256) k_hilite_assemble(const half4 *__restrict__ fine, int fw, int fh,
    const half4 *__restrict__ coarse, int cw, int ch, half4 *__restrict__ out, float white, float soft)
{
  const int ph = threadIdx.x >> 6, b = threadIdx.x & 63;      // parity class, position in it
  const int x = blockIdx.x * 16 + 2 * (b & 7) + (ph & 1), y = blockIdx.y * 16 + 2 * (b >> 3) + (ph >> 1);
  if(x >= fw || y >= fh) return;
  const bool tiny = cw < 2 || ch < 2;     // expand taps overshoot the coarse level by at most 1
  switch(ph)
  {
    case 0: assemble_one<0, 0>(fine, fw, coarse, cw, ch, tiny, x, y, out, white, soft); break;
    case 1: assemble_one<1, 0>(fine, fw, coarse, cw, ch, tiny, x, y, out, white, soft); break;
    case 2: assemble_one<0, 1>(fine, fw, coarse, cw, ch, tiny, x, y, out, white, soft); break;
    default: assemble_one<1, 1>(fine, fw, coarse, cw, ch, tiny, x, y, out, white, soft); break;
  }
}

// The small end of the pyramid (levels of a few thousand texels and less) in
// one CTA of 1024 threads: per-level launches there cost more than their work.
// The same device functions as k_hilite_reduce and k_hilite_assemble on the
// same f16 values, so the levels are bit identical; they live in shared
// memory: the reduce terms of the current input level, the reduce outputs
// R[t..L-1] and the assembled B[t..L-2] (rgba f16 each).
constexpr int HT_NT = 1024;

// rgba f16 from shared memory (ld_half4 reads through the read-only global path)
DEV void lds_half4(const half4 *p, float &a, float &b, float &c, float &d)
{
  const uint2 u = *reinterpret_cast<const uint2 *>(p);
  const __half2 lo = *reinterpret_cast<const __half2 *>(&u.x), hi = *reinterpret_cast<const __half2 *>(&u.y);
  a = __low2float(lo); b = __high2float(lo); c = __low2float(hi); d = __high2float(hi);
}

__global__ void __launch_bounds__(HT_NT) k_hilite_tail(const dev_hilite_tail_t p)
{
  extern __shared__ __align__(16) unsigned char tail_raw[];
  const int nr = p.nr;
  const int n0 = p.lw[0] * p.lh[0];
  float *terms = reinterpret_cast<float *>(tail_raw);          // 5 planes of n0
  half4 *R[HL_TAIL_MAX], *B[HL_TAIL_MAX];
  {
    half4 *q = reinterpret_cast<half4 *>(terms + 5 * ((n0 + 3) & ~3));
    for(int l = 1; l <= nr; l++) { R[l] = q; q += p.lw[l] * p.lh[l]; }      // R[l]: level t-1+l
    for(int l = 1; l < nr; l++) { B[l] = q; q += p.lw[l] * p.lh[l]; }       // B[l]: assembled level t-1+l
  }
  const hl_reduce_t ra = hilite_reduce_args(p.white, p.desat, p.wb);
  // terms of the input level
  for(int i = threadIdx.x; i < n0; i += HT_NT)
  {
    float rgb[3], w, t[5];
    ld_half4(p.in + i, rgb[0], rgb[1], rgb[2], w);
    hilite_reduce_texel(ra, rgb, t);
#pragma unroll
    for(int k = 0; k < 5; k++) terms[k * n0 + i] = t[k];
  }
  __syncthreads();
  for(int l = 1; l <= nr; l++)
  { // reduce level l - 1 (terms) into R[l]
    const int iw = p.lw[l - 1], ih = p.lh[l - 1], ow = p.lw[l], oh = p.lh[l], ni = iw * ih;
    const bool tiny = iw < 3 || ih < 3;
    for(int o = threadIdx.x; o < ow * oh; o += HT_NT)
    {
      const int x = o % ow, y = o / ow;
      float r[4];
      hilite_reduce_sum([&](int ii, int jj, float t[5]) {
          const int sx = tiny ? mirror_full(2 * x + ii, iw) : mirror1c(2 * x + ii, iw);
          const int sy = tiny ? mirror_full(2 * y + jj, ih) : mirror1c(2 * y + jj, ih);
#pragma unroll
          for(int k = 0; k < 5; k++) t[k] = terms[k * ni + sy * iw + sx];
        }, r);
      R[l][o] = mk_half4(r[0], r[1], r[2], r[3]);
    }
    __syncthreads();
    if(l < nr)
    { // the terms of R[l], the next input
      const int n = ow * oh;
      for(int i = threadIdx.x; i < n; i += HT_NT)
      {
        float rgb[3], w, t[5];
        lds_half4(R[l] + i, rgb[0], rgb[1], rgb[2], w);
        hilite_reduce_texel(ra, rgb, t);
#pragma unroll
        for(int k = 0; k < 5; k++) terms[k * n + i] = t[k];
      }
      __syncthreads();
    }
  }
  for(int l = nr - 1; l >= 1; l--)
  { // assemble B[l] from the fine R[l] and the coarse B[l + 1] (R[nr] for the coarsest)
    const half4 *coarse = l + 1 < nr ? B[l + 1] : R[nr];
    const int fw = p.lw[l], fh = p.lh[l], cw = p.lw[l + 1], ch = p.lh[l + 1];
    const bool tiny = cw < 2 || ch < 2;
    half4 *dst = l == 1 ? p.out : B[l];
    for(int o = threadIdx.x; o < fw * fh; o += HT_NT)
    {
      const int x = o % fw, y = o / fw;
      float up[3];
      hilite_expand_px([&](int ix, int iy, float rgb[3]) {
          const int sx = tiny ? mirror_full(ix, cw) : mirror1c(ix, cw), sy = tiny ? mirror_full(iy, ch) : mirror1c(iy, ch);
          float w;
          lds_half4(coarse + sy * cw + sx, rgb[0], rgb[1], rgb[2], w);
        }, x, y, up);
      float f[4];
      lds_half4(R[l] + o, f[0], f[1], f[2], f[3]);
      float ov[3];
      hilite_assemble_px(f, up, p.white, p.soft, ov);
      dst[o] = mk_half4(ov[0], ov[1], ov[2], 1.0f);
    }
    __syncthreads();
  }
}

} // namespace

size_t hilite_tail_smem_bytes(const int *lw, const int *lh, int nr)
{
  size_t b = 5 * sizeof(float) * (size_t)((lw[0] * lh[0] + 3) & ~3);
  for(int l = 1; l <= nr; l++) b += 8 * (size_t)lw[l] * lh[l];
  for(int l = 1; l < nr; l++) b += 8 * (size_t)lw[l] * lh[l];
  return b;
}

cudaError_t init_hilite()
{
  return cudaFuncSetAttribute(k_hilite_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HL_TAIL_SMEM);
}

cudaError_t launch_hilite_tail(const dev_hilite_tail_t &p, cudaStream_t s)
{
  if(p.nr < 2 || p.nr >= HL_TAIL_MAX) return cudaErrorInvalidValue;
  const size_t smem = hilite_tail_smem_bytes(p.lw, p.lh, p.nr);
  if(smem > HL_TAIL_SMEM) return cudaErrorInvalidValue;
  k_hilite_tail<<<1, HT_NT, smem, s>>>(p);
  return cudaGetLastError();
}

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
