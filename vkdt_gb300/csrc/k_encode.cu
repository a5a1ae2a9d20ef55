// Output encode after the path: colenc/main.comp (the output primaries and
// transfer curve of an rgba f16 image, as f16 or as the rgba u8 an 8-bit
// sink reads) and o-bc1's BC1 compression of an rgba u8 image (its vendored
// stb_dxt encoder restated; the reference runs it on the host in write_sink).
//
// k_bc1: one thread per 4x4 block, the encoder's integer steps as they are
// and its float/double steps in IEEE operations of the same order, so every
// block equals the reference encoder's bit for bit.
#include <cstdint>
#include <cstring>
#include "common.cuh"
#include "kernels.h"

namespace {

__constant__ uint8_t c_om5[256][2], c_om6[256][2];   // optimal endpoint pairs of a constant 5/6 bit channel

DEV int e5(int i) { return (i << 3) | (i >> 2); }
DEV int e6(int i) { return (i << 2) | (i >> 4); }
DEV int mul8(int a, int b) { const int t = a * b + 128; return (t + (t >> 8)) >> 8; }
DEV int lerp13(int a, int b) { return (2 * a + b) / 3; }
DEV uint16_t to565(int r, int g, int b) { return (uint16_t)((mul8(r, 31) << 11) + (mul8(g, 63) << 5) + mul8(b, 31)); }

DEV void palette(uint16_t c0, uint16_t c1, int col[4][3])
{
  col[0][0] = e5(c0 >> 11); col[0][1] = e6((c0 >> 5) & 63); col[0][2] = e5(c0 & 31);
  col[1][0] = e5(c1 >> 11); col[1][1] = e6((c1 >> 5) & 63); col[1][2] = e5(c1 & 31);
#pragma unroll
  for(int k = 0; k < 3; k++) { col[2][k] = lerp13(col[0][k], col[1][k]); col[3][k] = lerp13(col[1][k], col[0][k]); }
}

DEV uint32_t match(const uint8_t px[16][4], const int col[4][3])
{
  const int dr = col[0][0] - col[1][0], dg = col[0][1] - col[1][1], db = col[0][2] - col[1][2];
  int st[4];
#pragma unroll
  for(int k = 0; k < 4; k++) st[k] = col[k][0] * dr + col[k][1] * dg + col[k][2] * db;
  const int c0p = (st[1] + st[3]) >> 1, half = (st[3] + st[2]) >> 1, c3p = (st[2] + st[0]) >> 1;
  uint32_t mask = 0;
#pragma unroll
  for(int i = 15; i >= 0; i--)
  {
    const int dot = px[i][0] * dr + px[i][1] * dg + px[i][2] * db;
    mask <<= 2;
    if(dot < half) mask |= dot < c0p ? 1u : 3u;
    else           mask |= dot < c3p ? 2u : 0u;
  }
  return mask;
}

DEV void pca(const uint8_t px[16][4], uint16_t &mx16, uint16_t &mn16)
{
  int mu[3], lo[3], hi[3];
#pragma unroll
  for(int c = 0; c < 3; c++)
  {
    int sum = px[0][c];
    lo[c] = hi[c] = px[0][c];
#pragma unroll
    for(int i = 1; i < 16; i++) { const int v = px[i][c]; sum += v; lo[c] = min(lo[c], v); hi[c] = max(hi[c], v); }
    mu[c] = (sum + 8) >> 4;
  }
  int cov[6] = { 0, 0, 0, 0, 0, 0 };
#pragma unroll
  for(int i = 0; i < 16; i++)
  {
    const int r = px[i][0] - mu[0], g = px[i][1] - mu[1], b = px[i][2] - mu[2];
    cov[0] += r * r; cov[1] += r * g; cov[2] += r * b; cov[3] += g * g; cov[4] += g * b; cov[5] += b * b;
  }
  float cf[6];
#pragma unroll
  for(int i = 0; i < 6; i++) cf[i] = __fdiv_rn((float)cov[i], 255.0f);
  float vr = (float)(hi[0] - lo[0]), vg = (float)(hi[1] - lo[1]), vb = (float)(hi[2] - lo[2]);
#pragma unroll
  for(int it = 0; it < 4; it++)
  { // power iteration: each product rounded, summed left to right
    const float r = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[0]), __fmul_rn(vg, cf[1])), __fmul_rn(vb, cf[2]));
    const float g = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[1]), __fmul_rn(vg, cf[3])), __fmul_rn(vb, cf[4]));
    const float b = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[2]), __fmul_rn(vg, cf[4])), __fmul_rn(vb, cf[5]));
    vr = r; vg = g; vb = b;
  }
  double magn = fabs((double)vr);
  if(fabs((double)vg) > magn) magn = fabs((double)vg);
  if(fabs((double)vb) > magn) magn = fabs((double)vb);
  int wr, wg, wb;
  if(magn < 4.0) { wr = 299; wg = 587; wb = 114; }
  else
  {
    magn = __ddiv_rn(512.0, magn);
    wr = __double2int_rz(__dmul_rn((double)vr, magn));
    wg = __double2int_rz(__dmul_rn((double)vg, magn));
    wb = __double2int_rz(__dmul_rn((double)vb, magn));
  }
  int mind = 0x7fffffff, maxd = -0x7fffffff;
  uint16_t lo16 = 0, hi16 = 0;   // the colours of the first pixels with the smallest / largest projection
#pragma unroll
  for(int i = 0; i < 16; i++)
  {
    const int dot = px[i][0] * wr + px[i][1] * wg + px[i][2] * wb;
    if(dot < mind) { mind = dot; lo16 = to565(px[i][0], px[i][1], px[i][2]); }
    if(dot > maxd) { maxd = dot; hi16 = to565(px[i][0], px[i][1], px[i][2]); }
  }
  mx16 = hi16;
  mn16 = lo16;
}

DEV int sclamp(float y, int lo, int hi) { const int x = __float2int_rz(y); return x < lo ? lo : (x > hi ? hi : x); }

DEV bool refine(const uint8_t px[16][4], uint16_t &mx16, uint16_t &mn16, uint32_t mask)
{
  const uint16_t omn = mn16, omx = mx16;
  uint16_t a16, b16;
  if((mask ^ (mask << 2)) < 4)
  {
    int r = 8, g = 8, b = 8;
#pragma unroll
    for(int i = 0; i < 16; i++) { r += px[i][0]; g += px[i][1]; b += px[i][2]; }
    r >>= 4; g >>= 4; b >>= 4;
    a16 = (uint16_t)((c_om5[r][0] << 11) | (c_om6[g][0] << 5) | c_om5[b][0]);
    b16 = (uint16_t)((c_om5[r][1] << 11) | (c_om6[g][1] << 5) | c_om5[b][1]);
  }
  else
  {
    int xx = 0, yy = 0, xy = 0, a1[3] = { 0, 0, 0 }, a2[3] = { 0, 0, 0 };
    uint32_t cm = mask;
#pragma unroll
    for(int i = 0; i < 16; i++, cm >>= 2)
    {
      const uint32_t st = cm & 3;
      const int w = st == 0 ? 3 : st == 1 ? 0 : st == 2 ? 2 : 1;
      xx += w * w; yy += (3 - w) * (3 - w); xy += w * (3 - w);
#pragma unroll
      for(int c = 0; c < 3; c++) { a1[c] += w * px[i][c]; a2[c] += px[i][c]; }
    }
#pragma unroll
    for(int c = 0; c < 3; c++) a2[c] = 3 * a2[c] - a1[c];
    const float frb = __fdiv_rn(__fdiv_rn(93.0f, 255.0f), (float)(xx * yy - xy * xy));   // 3 * 31 / 255 / det
    const float fg = __fdiv_rn(__fmul_rn(frb, 63.0f), 31.0f);
    auto q = [&](int num, float f, int hi) { return sclamp(__fadd_rn(__fmul_rn((float)num, f), 0.5f), 0, hi); };
    a16 = (uint16_t)((q(a1[0] * yy - a2[0] * xy, frb, 31) << 11) | (q(a1[1] * yy - a2[1] * xy, fg, 63) << 5)
                     | q(a1[2] * yy - a2[2] * xy, frb, 31));
    b16 = (uint16_t)((q(a2[0] * xx - a1[0] * xy, frb, 31) << 11) | (q(a2[1] * xx - a1[1] * xy, fg, 63) << 5)
                     | q(a2[2] * xx - a1[2] * xy, frb, 31));
  }
  mn16 = b16; mx16 = a16;
  return omn != mn16 || omx != mx16;
}

// o-bc1/main.c:30-47 + stb_dxt's stb_compress_dxt_block (no alpha, normal mode): one thread per block
template<bool VEC> __global__ void __launch_bounds__(128) k_bc1(const uint8_t *__restrict__ rgba, int wd, int ht, uint8_t *__restrict__ out)
{
  const int bx = wd / 4, by = ht / 4;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if(i >= bx || j >= by) return;
  uint8_t px[16][4];
  bool constant = true;
  uint32_t w0 = 0;
#pragma unroll
  for(int jj = 0; jj < 4; jj++)
  {
    const uint8_t *rp = rgba + 4 * ((size_t)wd * (4 * j + jj) + 4 * i);
    uint32_t w[4];
    if(VEC)
    { // 16-byte rows (width a multiple of 4, aligned image)
      const uint4 row = __ldg(reinterpret_cast<const uint4 *>(rp));
      w[0] = row.x; w[1] = row.y; w[2] = row.z; w[3] = row.w;
    }
    else
#pragma unroll
      for(int ii = 0; ii < 4; ii++) w[ii] = __ldg(reinterpret_cast<const uint32_t *>(rp) + ii);
#pragma unroll
    for(int ii = 0; ii < 4; ii++)
    {
      if(jj == 0 && ii == 0) w0 = w[0];
      constant = constant && w[ii] == w0;
#pragma unroll
      for(int c = 0; c < 4; c++) px[4 * jj + ii][c] = (uint8_t)(w[ii] >> (8 * c));
    }
  }
  uint32_t mask;
  uint16_t mx16, mn16;
  if(constant)
  {
    const int r = px[0][0], g = px[0][1], b = px[0][2];
    mask = 0xaaaaaaaau;
    mx16 = (uint16_t)((c_om5[r][0] << 11) | (c_om6[g][0] << 5) | c_om5[b][0]);
    mn16 = (uint16_t)((c_om5[r][1] << 11) | (c_om6[g][1] << 5) | c_om5[b][1]);
  }
  else
  {
    int col[4][3];
    pca(px, mx16, mn16);
    if(mx16 != mn16) { palette(mx16, mn16, col); mask = match(px, col); }
    else mask = 0;
    if(refine(px, mx16, mn16, mask))
    {
      if(mx16 != mn16) { palette(mx16, mn16, col); mask = match(px, col); }
      else mask = 0;
    }
  }
  if(mx16 < mn16) { const uint16_t t = mn16; mn16 = mx16; mx16 = t; mask ^= 0x55555555u; }
  uint2 o;
  o.x = (uint32_t)mx16 | ((uint32_t)mn16 << 16);
  o.y = mask;
  *reinterpret_cast<uint2 *>(out + 8 * ((size_t)bx * j + i)) = o;
}

// colenc/main.comp:15-80
struct colenc_t { float M[9]; int mat, trc; };
__global__ void __launch_bounds__(256) k_colenc(const half4 *__restrict__ in, int wd, int ht, colenc_t c,
    half4 *__restrict__ out16, uint32_t *__restrict__ out8)
{
  const int x = blockIdx.x * 64 + threadIdx.x % 64, y = blockIdx.y * 4 + threadIdx.x / 64;
  if(x >= wd || y >= ht) return;
  float rgb[3], a;
  ld_half4(in + (size_t)y * wd + x, rgb[0], rgb[1], rgb[2], a);
  if(c.mat)
  {
    float o[3];
#pragma unroll
    for(int i = 0; i < 3; i++)   // the shader's order, each product rounded: tiny results cancel
      o[i] = __fadd_rn(__fadd_rn(__fmul_rn(c.M[3 * i], rgb[0]), __fmul_rn(c.M[3 * i + 1], rgb[1])), __fmul_rn(c.M[3 * i + 2], rgb[2]));
#pragma unroll
    for(int i = 0; i < 3; i++) rgb[i] = o[i];
  }
#pragma unroll
  for(int k = 0; k < 3; k++)
  {
    float v = rgb[k];
    switch(c.trc)
    {
      case 1: v = v > 0.018053968510807f ? powf(v, 1.0f / 2.2f) * 1.09929682680944f - (1.09929682680944f - 1.0f) : v * 4.5f; break;
      case 2: v = v > 0.0031308f ? powf(v, 1.0f / 2.4f) * 1.055f - 0.055f : v * 12.92f; break;
      case 3:
      { // PQ oetf
        const float c3 = 2392.0f / 128.0f, c2 = 2413.0f / 128.0f, c1 = c3 - c2 + 1.0f, m1 = 1305.0f / 8192.0f, m2 = 2523.0f / 32.0f;
        const float p = powf(fmaxf(0.0f, v), m1);
        v = powf(1.0f + ((c1 - 1.0f) + (c2 - c3) * p) / (1.0f + c3 * p), m2);
        break;
      }
      case 4: v = powf(v, 1.0f / 2.6f); break;
      case 5:
      { // HLG
        const float aa = 0.17883277f, bb = 1.0f - 4.0f * aa, cc = 0.5f - aa * logf(4.0f * aa);
        v = v > 1.0f / 12.0f ? aa * logf(12.0f * v - bb) + cc : sqrtf(3.0f * v);
        break;
      }
      case 6: v = powf(v, 1.0f / 2.2f); break;
      default: break;
    }
    rgb[k] = v;
  }
  const size_t o = (size_t)y * wd + x;
  if(out16) out16[o] = mk_half4(rgb[0], rgb[1], rgb[2], 1.0f);
  if(out8)
  { // R8G8B8A8_UNORM stores: clamp, scale, round to nearest
    uint32_t w = 255u << 24;
#pragma unroll
    for(int k = 0; k < 3; k++) w |= (uint32_t)__float2uint_rn(fminf(fmaxf(rgb[k], 0.0f), 1.0f) * 255.0f) << (8 * k);
    out8[o] = w;
  }
}

bool g_bc1_tables = false;

} // namespace

cudaError_t launch_bc1(const void *rgba, int wd, int ht, void *out, cudaStream_t s)
{
  if(!g_bc1_tables)
  { // stb_dxt's single colour tables (PrepareOptTable): the endpoints whose 1/3 point reproduces each value best
    uint8_t om5[256][2], om6[256][2];
    for(int t = 0; t < 2; t++)
    {
      const int size = t ? 64 : 32;
      uint8_t (*tab)[2] = t ? om6 : om5;
      for(int i = 0; i < 256; i++)
      {
        int best = 256;
        for(int mn = 0; mn < size; mn++) for(int mx = 0; mx < size; mx++)
        {
          const int emx = t ? ((mx << 2) | (mx >> 4)) : ((mx << 3) | (mx >> 2));
          const int emn = t ? ((mn << 2) | (mn >> 4)) : ((mn << 3) | (mn >> 2));
          const int err = abs((2 * emx + emn) / 3 - i) + abs(emx - emn) * 3 / 100;
          if(err < best) { tab[i][0] = (uint8_t)mx; tab[i][1] = (uint8_t)mn; best = err; }
        }
      }
    }
    cudaError_t e = cudaMemcpyToSymbol(c_om5, om5, sizeof(om5));
    if(e == cudaSuccess) e = cudaMemcpyToSymbol(c_om6, om6, sizeof(om6));
    if(e != cudaSuccess) return e;
    g_bc1_tables = true;
  }
  const int bx = wd / 4, by = ht / 4;
  if(bx == 0 || by == 0) return cudaSuccess;
  const dim3 grid((bx + 127) / 128, by);
  if(((uintptr_t)rgba & 15) == 0 && (wd & 3) == 0)
    k_bc1<true><<<grid, 128, 0, s>>>(reinterpret_cast<const uint8_t *>(rgba), wd, ht, reinterpret_cast<uint8_t *>(out));
  else
    k_bc1<false><<<grid, 128, 0, s>>>(reinterpret_cast<const uint8_t *>(rgba), wd, ht, reinterpret_cast<uint8_t *>(out));
  return cudaGetLastError();
}

cudaError_t launch_colenc(const void *rgba16, int wd, int ht, const float *M, int trc, void *out16, void *out8, cudaStream_t s)
{
  colenc_t c;
  memset(&c, 0, sizeof(c));
  c.mat = M != nullptr;
  if(M) memcpy(c.M, M, sizeof(c.M));
  c.trc = trc;
  k_colenc<<<dim3((wd + 63) / 64, (ht + 3) / 4), 256, 0, s>>>(reinterpret_cast<const half4 *>(rgba16), wd, ht, c,
      reinterpret_cast<half4 *>(out16), reinterpret_cast<uint32_t *>(out8));
  return cudaGetLastError();
}
