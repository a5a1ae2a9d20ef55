// The per-node chain of the path for what the fused develop kernel does not
// cover: x-trans mosaics, and reduced output sizes (demosaic/halfsize +
// shared/resample, the thumbnail path) for both mosaics. One kernel per
// reference node, intermediates in HBM as f16 images like the reference:
//   [denoise/noop] -> hilite/half -> (hilite reduce/assemble pyramid, k_hilite.cu)
//   -> hilite/doub -> demosaic (gauss, splat, fix | halfsize [-> resample])
//   -> colour -> [histogram] -> filmcurv -> llap/curve -> first llap/reduce (k_post)
//   -> (llap pyramid, k_llap.cu)
// The arithmetic restates the shaders in their order; computations that
// decide a branch (the green structure tensor and its snapping, the clip
// tests) use explicit IEEE operations, as the oracle evaluates them.
#include "common.cuh"
#include "develop_px.cuh"
#include "gauss.cuh"
#include "hilite.cuh"
#include "kernels.h"
#include "lens.h"
#include "pixel.cuh"
#include "sampler.cuh"

namespace {

DEV float dn_m(const dev_nodes_t &p, const __half *img, int x, int y)
{ // texture() at a texel centre of a W x H one channel image: the mirrored texel
  return h2f(img[(size_t)mirror(y, p.H) * p.W + mirror(x, p.W)]);
}
DEV float dn_z(const dev_nodes_t &p, const __half *img, int x, int y)
{ // texelFetch: out of range reads 0
  if(x < 0 || y < 0 || x >= p.W || y >= p.H) return 0.0f;
  return h2f(img[(size_t)y * p.W + x]);
}

// denoise/noop.comp:36-57 through the code table: the normalised mosaic as f16
__global__ void __launch_bounds__(256) k_nd_noop(const dev_nodes_t p)
{
  const int x = blockIdx.x * 64 + threadIdx.x % 64, y = blockIdx.y * 4 + threadIdx.x / 64;
  if(x >= p.W || y >= p.H) return;
  p.dn[(size_t)y * p.W + x] = __ldg(p.noop_lut + __ldg(p.mosaic + (size_t)(y + p.cy) * p.pitch + x + p.cx));
}

// hilite/half.comp:21-72
template<bool XT> __global__ void __launch_bounds__(256) k_nd_hl_half(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  float h[3];
  if(XT)
  {
    float c[9];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++) c[3 * i + j] = dn_z(p, p.dn, 3 * x + i, 3 * y + j);
    hilite_half_xtrans(c, x, y, p.hl_white, h);
  }
  else
    hilite_half_bayer(dn_m(p, p.dn, 2 * x, 2 * y), dn_m(p, p.dn, 2 * x + 1, 2 * y),
                      dn_m(p, p.dn, 2 * x, 2 * y + 1), dn_m(p, p.dn, 2 * x + 1, 2 * y + 1), p.hl_white, h);
  p.h0[(size_t)y * p.hw + x] = mk_half4(h[0], h[1], h[2], 1.0f);
}

// hilite/doub.comp:141-241: re-mosaic, blending clipped samples towards the
// scaled coarse colour. Mosaic positions no block covers are not written.
template<bool XT> __global__ void __launch_bounds__(256) k_nd_hl_doub(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  float up[3], a;
  ld_half4(p.b0 + (size_t)y * p.hw + x, up[0], up[1], up[2], a);
  const float white = p.hl_white;
  if(XT)
  {
    if(((x + y) & 1) == 0) { const float t = up[0]; up[0] = up[2]; up[2] = t; }
    float c[9];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++) c[3 * i + j] = dn_z(p, p.dn, 3 * x + i, 3 * y + j);
    const float minr = fminf(c[1], c[7]), minb = fminf(c[3], c[5]);
    const float ming = fminf(fminf(fminf(c[0], c[2]), c[4]), fminf(c[6], c[8]));
    const float sr = minr / fmaxf(0.001f, up[0]);
    const float sg = ming / fmaxf(0.001f, up[1]);
    const float sb = minb / fmaxf(0.001f, up[2]);
    const float wr = expf(up[0] - fmaxf(up[1], up[2]));
    const float wg = expf(up[1] - fmaxf(up[0], up[2]));
    const float wbb = expf(up[2] - fmaxf(up[0], up[1]));
    const float scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
    const float maxr = fmaxf(c[1], c[7]), maxb = fmaxf(c[3], c[5]);
    const float maxg = fmaxf(fmaxf(fmaxf(c[0], c[2]), c[4]), fmaxf(c[6], c[8]));
    const float softw = __fmul_rn(0.97f, white);
    const float maxrgb = fmaxf(maxr, fmaxf(maxg, maxb));
    if(maxrgb > softw)
    {
      float t = smoothstep(softw, white, maxrgb);
      c[1] = gmix(c[1], up[0] * scale, t);
      c[7] = gmix(c[7], up[0] * scale, t);
      c[3] = gmix(c[3], up[2] * scale, t);
      c[5] = gmix(c[5], up[2] * scale, t);
      t = smoothstep(softw, white, ming);
      c[0] = gmix(c[0], up[1] * scale, t);
      c[2] = gmix(c[2], up[1] * scale, t);
      c[4] = gmix(c[4], up[1] * scale, t);
      c[6] = gmix(c[6], up[1] * scale, t);
      c[8] = gmix(c[8], up[1] * scale, t);
    }
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++)
      {
        const int X = 3 * x + i, Y = 3 * y + j;
        if(X < p.W && Y < p.H) p.hl[(size_t)Y * p.W + X] = f2h(c[3 * i + j]);
      }
  }
  else
  {
    float o[4];
    hilite_doub_bayer(dn_m(p, p.dn, 2 * x, 2 * y), dn_m(p, p.dn, 2 * x + 1, 2 * y),
                      dn_m(p, p.dn, 2 * x, 2 * y + 1), dn_m(p, p.dn, 2 * x + 1, 2 * y + 1), up, white, o);
    const int X = 2 * x, Y = 2 * y;
    if(X < p.W && Y < p.H) p.hl[(size_t)Y * p.W + X] = f2h(o[0]);
    if(X + 1 < p.W && Y < p.H) p.hl[(size_t)Y * p.W + X + 1] = f2h(o[1]);
    if(X < p.W && Y + 1 < p.H) p.hl[(size_t)(Y + 1) * p.W + X] = f2h(o[2]);
    if(X + 1 < p.W && Y + 1 < p.H) p.hl[(size_t)(Y + 1) * p.W + X + 1] = f2h(o[3]);
  }
}

// denoise/noop, hilite/half, the level 0 hilite/assemble and hilite/doub of a
// bayer block at once, from the mosaic through the code table and the
// assembled level 1 of the hilite pyramid: the first stage of the fused
// develop kernel, for the demosaic methods that run node by node after it.
// doub changes a block only where its largest sample exceeds 0.97 white;
// elsewhere the block is the noop output as it is.
__global__ void __launch_bounds__(256) k_nd_hl_bayer(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  // the pairs of a block row as one 32 bit word (bayer: even pitch, crop offset and size)
  const uint16_t *row = p.mosaic + (size_t)(2 * y + p.cy) * p.pitch + 2 * x + p.cx;
  const uint32_t r0 = __ldg(reinterpret_cast<const uint32_t *>(row));
  const uint32_t r1 = __ldg(reinterpret_cast<const uint32_t *>(row + p.pitch));
  float m[4];
  m[0] = h2f(__ldg(p.noop_lut + (r0 & 0xffff)));
  m[1] = h2f(__ldg(p.noop_lut + (r0 >> 16)));
  m[2] = h2f(__ldg(p.noop_lut + (r1 & 0xffff)));
  m[3] = h2f(__ldg(p.noop_lut + (r1 >> 16)));
  float o[4] = { m[0], m[1], m[2], m[3] };
  const float white = p.hl_white;
  if(fmaxf(fmaxf(m[2], m[3]), fmaxf(m[1], m[0])) > 0.97f * white)
  {
    float h[4];
    hilite_half_bayer(m[0], m[1], m[2], m[3], white, h);
    h[3] = 1.0f;
    float up[3];
    hilite_expand_px([&](int ix, int iy, float rgb[3]) {
        float a;
        ld_half4(p.coarse + (size_t)mirror(iy, p.cch) * p.ccw + mirror(ix, p.ccw), rgb[0], rgb[1], rgb[2], a);
      }, x, y, up);
    float b0[3];
    hilite_assemble_px(h, up, white, p.hl_soft, b0);
    hilite_doub_bayer(m[0], m[1], m[2], m[3], b0, white, o);
  }
  const size_t o0 = (size_t)(2 * y) * p.W + 2 * x;
  *reinterpret_cast<__half2 *>(p.hl + o0) = __halves2half2(f2h(o[0]), f2h(o[1]));
  *reinterpret_cast<__half2 *>(p.hl + o0 + p.W) = __halves2half2(f2h(o[2]), f2h(o[3]));
  if(p.dn)
  {
    p.dn[o0] = f2h(m[0]); p.dn[o0 + 1] = f2h(m[1]);
    p.dn[o0 + p.W] = f2h(m[2]); p.dn[o0 + p.W + 1] = f2h(m[3]);
  }
}

// demosaic/gauss.comp:19-126 (x-trans): structure tensor of the 5 greens of
// each 3x3 block, the form with the smaller determinant decomposed; the
// eigenvector snapped to an axis when it is within a factor 2 of it, else an
// isotropic 0.1
__global__ void __launch_bounds__(256) k_nd_gauss_xt(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  // greens (i + j even) of the block, i the x offset
  const int gi[5] = { 0, 2, 1, 0, 2 }, gj[5] = { 0, 0, 1, 2, 2 };
  float px[5];
  float mw0 = 0.0f, mw1 = 0.0f, mb0 = 0.0f, mb1 = 0.0f, smw = 0.0f, smb = 0.0f;
#pragma unroll
  for(int k = 0; k < 5; k++)
  { // the shader's loop order is j outer, i inner: (0,0) (2,0) (1,1) (0,2) (2,2)
    px[k] = dn_m(p, p.hl, 3 * x + gi[k], 3 * y + gj[k]);
    const float fi = (float)gi[k], fj = (float)gj[k];
    mw0 = __fadd_rn(mw0, __fmul_rn(fi, px[k])); mw1 = __fadd_rn(mw1, __fmul_rn(fj, px[k]));
    smw = __fadd_rn(smw, px[k]);
    // fi/px = fi (1/px) exactly for fi in {0, 1, 2}; px is an f16 value (rcp_f16v)
    const float inv = rcp_f16v(px[k]);
    mb0 = __fadd_rn(mb0, __fmul_rn(fi, inv)); mb1 = __fadd_rn(mb1, __fmul_rn(fj, inv));
    smb = __fadd_rn(smb, inv);
  }
  {
    const float yw = __frcp_rn(smw), yb = __frcp_rn(smb);
    const bool okw = div_ok(smw), okb = div_ok(smb);
    mw0 = div_ry(mw0, smw, yw, okw); mw1 = div_ry(mw1, smw, yw, okw);
    mb0 = div_ry(mb0, smb, yb, okb); mb1 = div_ry(mb1, smb, yb, okb);
  }
  float Sw00 = 0, Sw01 = 0, Sw10 = 0, Sw11 = 0, Sb00 = 0, Sb01 = 0, Sb10 = 0, Sb11 = 0, sw = 0, sb = 0;
#pragma unroll
  for(int k = 0; k < 5; k++)
  {
    float p2 = __fmul_rn(px[k], px[k]);
    float q0 = __fsub_rn((float)gi[k], mw0), q1 = __fsub_rn((float)gj[k], mw1);
    Sw00 = __fadd_rn(Sw00, __fmul_rn(__fmul_rn(p2, q0), q0));
    Sw01 = __fadd_rn(Sw01, __fmul_rn(__fmul_rn(p2, q0), q1));
    Sw10 = __fadd_rn(Sw10, __fmul_rn(__fmul_rn(p2, q1), q0));
    Sw11 = __fadd_rn(Sw11, __fmul_rn(__fmul_rn(p2, q1), q1));
    sw = __fadd_rn(sw, p2);
    q0 = __fsub_rn((float)gi[k], mb0); q1 = __fsub_rn((float)gj[k], mb1);
    p2 = rcp_f16v(p2);
    Sb00 = __fadd_rn(Sb00, __fmul_rn(__fmul_rn(p2, q0), q0));
    Sb01 = __fadd_rn(Sb01, __fmul_rn(__fmul_rn(p2, q0), q1));
    Sb10 = __fadd_rn(Sb10, __fmul_rn(__fmul_rn(p2, q1), q0));
    Sb11 = __fadd_rn(Sb11, __fmul_rn(__fmul_rn(p2, q1), q1));
    sb = __fadd_rn(sb, p2);
  }
  {
    const float yw = __frcp_rn(sw), yb = __frcp_rn(sb);
    const bool okw = div_ok(sw), okb = div_ok(sb);
    Sw00 = div_ry(Sw00, sw, yw, okw); Sw01 = div_ry(Sw01, sw, yw, okw);
    Sw10 = div_ry(Sw10, sw, yw, okw); Sw11 = div_ry(Sw11, sw, yw, okw);
    Sb00 = div_ry(Sb00, sb, yb, okb); Sb01 = div_ry(Sb01, sb, yb, okb);
    Sb10 = div_ry(Sb10, sb, yb, okb); Sb11 = div_ry(Sb11, sb, yb, okb);
  }
  const float detw = __fsub_rn(__fmul_rn(Sw00, Sw11), __fmul_rn(Sw10, Sw01));
  const float detb = __fsub_rn(__fmul_rn(Sb00, Sb11), __fmul_rn(Sb10, Sb01));
  float eval[2], e0[2], e1[2];
  const bool usew = detw < detb;
  if(usew) evd2x2(eval, e0, e1, Sw00, Sw10, Sw11);
  else     evd2x2(eval, e0, e1, Sb00, Sb10, Sb11);
  eval[0] = __fmul_rn(eval[0], 0.4f); eval[1] = __fmul_rn(eval[1], 0.4f);
  int snap;
  if(fabsf(e0[0]) > __fmul_rn(2.0f, fabsf(e0[1])))      { e0[0] = 1.0f; e0[1] = 0.0f; snap = 0; }
  else if(fabsf(e0[1]) > __fmul_rn(2.0f, fabsf(e0[0]))) { e0[0] = 0.0f; e0[1] = 1.0f; snap = 1; }
  else { eval[0] = 0.1f; eval[1] = 0.1f; snap = 2; }
  p.cov[(size_t)y * p.hw + x] = mk_half4(eval[0], eval[1], e0[0], e0[1]);
  if(p.dbg_gauss) p.dbg_gauss[(size_t)y * p.hw + x] = (uint8_t)((usew ? GAUSS_DEC_USEW : 0) | (snap << GAUSS_DEC_SNAP_SHIFT));
}

DEV void cov_z(const dev_nodes_t &p, int x, int y, float c[4])
{ // texelFetch of the gauss output (hw x hh), 0 out of range
  if(x < 0 || y < 0 || x >= p.hw || y >= p.hh) { c[0] = c[1] = c[2] = c[3] = 0.0f; return; }
  ld_half4(p.cov + (size_t)y * p.hw + x, c[0], c[1], c[2], c[3]);
}

// exp(-0.5 (of0^2 / e0 + of1^2 / e1)) with of0 = c i + s j, of1 = -s i + c j
// (c, s the covariance's eigenvector) as a quadratic form in the tap offset:
// exp2(qa i^2 + qb i j + qc j^2), the coefficients made once per pixel (the
// same weight up to the rounding of the products, before an f16 store)
struct xt_quad_t { float qa, qb, qc; };
DEV xt_quad_t xt_quad(float c, float s, float ie0, float ie1)
{
  const float k = -0.5f * 1.4426950408889634f;
  xt_quad_t q;
  q.qa = k * (c * c * ie0 + s * s * ie1);
  q.qb = k * 2.0f * c * s * (ie0 - ie1);
  q.qc = k * (s * s * ie0 + c * c * ie1);
  return q;
}
DEV float xt_weight(const xt_quad_t &q, int i, int j)
{
  float w;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(w) : "f"(q.qa * (float)(i * i) + q.qb * (float)(i * j) + q.qc * (float)(j * j)));
  return w;
}

// tiles of the x-trans splat and fix kernels: multiples of the 6x6 CFA period
// and of the 3x3 blocks of the covariance; the mosaic (and the splat output)
// the taps read is staged once per tile with the halo the taps reach. A warp
// takes the 32 pixels of one CFA phase of the tile (8 x 4 periods), so which
// taps are green, red or blue is the same in all its lanes.
constexpr int XT_TX = 48, XT_TY = 24;
DEV void xt_item(int t, int &lx, int &ly)
{ // item t of the tile: phase t / 32, period t % 32
  const int ph = t >> 5, k = t & 31;
  lx = 6 * (k & 7) + ph % 6;
  ly = 6 * (k >> 3) + ph / 6;
}

// demosaic/splat.comp:142-266 (x-trans): 5x5 anisotropic gaussian splat of
// the greens (only the green sums form the output), taps wrapped by the CFA
// period 6 at the borders, centre weight 666
__global__ void __launch_bounds__(256) k_nd_splat_xt(const dev_nodes_t p)
{
  __shared__ float sh[XT_TY + 4][XT_TX + 4 + 1];     // hilite output at the wrapped tap positions, halo 2
  __shared__ uint8_t sgreen[XT_TY + 4][XT_TX + 4];   // the CFA colour of the tap position is green
  const int X0 = blockIdx.x * XT_TX, Y0 = blockIdx.y * XT_TY;
  for(int i = threadIdx.x; i < (XT_TY + 4) * (XT_TX + 4); i += blockDim.x)
  {
    const int sy = i / (XT_TX + 4), sx = i % (XT_TX + 4);
    const int gx = X0 - 2 + sx, gy = Y0 - 2 + sy;
    int px = gx, py = gy;   // taps past the border wrap by the CFA period 6
    if(px < 0) px += 6;
    if(py < 0) py += 6;
    if(px >= p.W) px -= 6;
    if(py >= p.H) py -= 6;
    sh[sy][sx] = dn_z(p, p.hl, px, py);
    sgreen[sy][sx] = cfa_xtrans(gx + 6, gy + 6) == 1;
  }
  __syncthreads();
  for(int t = threadIdx.x; t < XT_TX * XT_TY; t += blockDim.x)
  {
    int lx, ly;
    xt_item(t, lx, ly);
    const int x = X0 + lx, y = Y0 + ly;
    if(x >= p.W || y >= p.H) continue;
    float cov[4];
    cov_z(p, x / 3, y / 3, cov);
    const float e0 = gclamp(cov[0], 0.01f, 25.0f), e1 = gclamp(cov[1], 0.01f, 25.0f);
    const xt_quad_t q = xt_quad(cov[2], cov[3], 1.0f / e0, 1.0f / e1);
    float gs = 0.0f, gw = 0.0f;
#pragma unroll
    for(int j = -2; j <= 2; j++)
#pragma unroll
      for(int i = -2; i <= 2; i++)
      {
        if(!sgreen[ly + 2 + j][lx + 2 + i]) continue;   // the same in all lanes (one CFA phase per warp)
        const float col = sh[ly + 2 + j][lx + 2 + i];
        const float w = (i == 0 && j == 0) ? 666.0f : gclamp(xt_weight(q, i, j), 1e-4f, 1.0f);
        gs += col * w;
        gw += w;
      }
    p.g[(size_t)y * p.W + x] = f2h(gs / fmaxf(1e-8f, gw));
  }
}

// demosaic/fix.comp:55-135 (x-trans): red and blue from the taps of radius R
// (2, or 3 with the colour param), weighted by the covariance of the block of
// (x+1, y+1) and scaled by the splat green ratio; the centre keeps its green
template<int R> __global__ void __launch_bounds__(256) k_nd_fix_xt(const dev_nodes_t p)
{
  // mirrored, halo 3: hilite output, splat output and 1 / (1e-4 + splat output)
  __shared__ float shl[XT_TY + 6][XT_TX + 6 + 1], sgh[XT_TY + 6][XT_TX + 6 + 1], srg[XT_TY + 6][XT_TX + 6 + 1];
  __shared__ uint8_t scls[XT_TY + 6][XT_TX + 6];   // 0 red, 1 green, 2 blue of the tap position
  const int X0 = blockIdx.x * XT_TX, Y0 = blockIdx.y * XT_TY;
  for(int i = threadIdx.x; i < (XT_TY + 6) * (XT_TX + 6); i += blockDim.x)
  {
    const int sy = i / (XT_TX + 6), sx = i % (XT_TX + 6);
    const int px = X0 - 3 + sx, py = Y0 - 3 + sy;
    // slots past the image's last pixel + 3 are read by no pixel: clamped there (in mirror range)
    const int mx = min(px, p.W + 2), my = min(py, p.H + 2);
    shl[sy][sx] = dn_m(p, p.hl, mx, my);
    sgh[sy][sx] = dn_m(p, p.g, mx, my);
    srg[sy][sx] = 1.0f / (1e-4f + sgh[sy][sx]);
    // the shader's pattern test at the unwrapped position (truncating divisions)
    const bool blue_top = ((px / 3 + py / 3) & 1) > 0;
    const int qx = px - (px / 3) * 3, qy = py - (py / 3) * 3;
    scls[sy][sx] = ((qx + qy) & 1) == 0 ? 1 : ((blue_top ^ (qy == 1)) ? 2 : 0);
  }
  __syncthreads();
  // radius clamp(fixup + 2, 2, 3) (fix.comp:111): the halo of 3 covers both
  constexpr int r = R;
  for(int t = threadIdx.x; t < XT_TX * XT_TY; t += blockDim.x)
  {
    int lx, ly;
    xt_item(t, lx, ly);
    const int x = X0 + lx, y = Y0 + ly;
    if(x >= p.W || y >= p.H) continue;
    const float gc = sgh[ly + 3][lx + 3];
    float cov[4];
    cov_z(p, (x + 1) / 3, (y + 1) / 3, cov);
    cov[0] = gclamp(cov[0], 1.0f, 10.0f); cov[1] = gclamp(cov[1], 1.0f, 10.0f);
    const xt_quad_t q = xt_quad(cov[2], cov[3], 1.0f / (3.0f * cov[0]), 1.0f / (3.0f * cov[1]));
    const float gc4 = 1e-4f + gc;
    float rr = 0.0f, rb = 0.0f, wr = 0.0f, wb = 0.0f;
#pragma unroll
    for(int j = -r; j <= r; j++)
#pragma unroll
      for(int i = -r; i <= r; i++)
      {
        const int c = scls[ly + 3 + j][lx + 3 + i];
        if(c == 1) continue;      // green: the centre's own green is used (the same in all lanes)
        const float col = shl[ly + 3 + j][lx + 3 + i];
        const float w = gclamp(xt_weight(q, i, j), 1e-3f, 1.0f);
        // col (1e-4 + gc) / (1e-4 + gh) w with the reciprocal made once per slot
        const float v = col * gc4 * srg[ly + 3 + j][lx + 3 + i] * w;
        if(c == 2) { rb += v; wb += w; }
        else       { rr += v; wr += w; }
      }
    p.dm[(size_t)y * p.W + x] = mk_half4(rr / fmaxf(1e-8f, wr), gc, rb / fmaxf(1e-8f, wb), 1.0f);
  }
}

// demosaic/halfsize.comp:155-187: one rgb texel per CFA block
template<bool XT> __global__ void __launch_bounds__(256) k_nd_halfsize(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  float r, g, b;
  if(XT)
  {
    float c[9];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++) c[3 * i + j] = dn_z(p, p.hl, 3 * x + i, 3 * y + j);
    g = __fdiv_rn(c[0] + c[2] + c[4] + c[6] + c[8], 5.0f);
    const float c0 = (c[1] + c[7]) * 0.5f, c1 = (c[3] + c[5]) * 0.5f;
    if(((x + y) & 1) > 0) { r = c0; b = c1; }
    else                  { b = c0; r = c1; }
  }
  else
  {
    const float cx = dn_m(p, p.hl, 2 * x, 2 * y + 1), cy = dn_m(p, p.hl, 2 * x + 1, 2 * y + 1);
    const float cz = dn_m(p, p.hl, 2 * x + 1, 2 * y), cw = dn_m(p, p.hl, 2 * x, 2 * y);
    r = cw; g = (cx + cz) * 0.5f; b = cy;
  }
  p.hs[(size_t)y * p.hw + x] = mk_half4(r, g, b, 1.0f);
}

// shared/resample.comp:213-224 with shared.glsl:47-96 sample_catmull_rom:
// nine bilinear taps of the half size image
__global__ void __launch_bounds__(256) k_nd_resample(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.ow || y >= p.oh) return;
  const float sp[2] = { __fmul_rn(__fdiv_rn(__fadd_rn((float)x, 0.5f), (float)p.ow), (float)p.hw),
                        __fmul_rn(__fdiv_rn(__fadd_rn((float)y, 0.5f), (float)p.oh), (float)p.hh) };
  float t[2][3], w[2][3];
#pragma unroll
  for(int k = 0; k < 2; k++)
  {
    const float tp1 = floorf(__fsub_rn(sp[k], 0.5f)) + 0.5f;
    const float f = __fsub_rn(sp[k], tp1);
    const float w0 = f * (-0.5f + f * (1.0f - 0.5f * f));
    const float w1 = 1.0f + f * f * (-2.5f + 1.5f * f);
    const float w2 = f * (0.5f + f * (2.0f - 1.5f * f));
    const float w3 = f * f * (-0.5f + 0.5f * f);
    // the tap between texels 1 and 2 decides its sample position: IEEE
    const float w12 = __fadd_rn(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(f, f), __fadd_rn(-2.5f, __fmul_rn(1.5f, f)))),
                                __fmul_rn(f, __fadd_rn(0.5f, __fmul_rn(f, __fsub_rn(2.0f, __fmul_rn(1.5f, f))))));
    const float w2e = __fmul_rn(f, __fadd_rn(0.5f, __fmul_rn(f, __fsub_rn(2.0f, __fmul_rn(1.5f, f)))));
    t[k][0] = tp1 - 1.0f; t[k][1] = __fadd_rn(tp1, __fdiv_rn(w2e, w12)); t[k][2] = tp1 + 2.0f;
    w[k][0] = w0; w[k][1] = w1 + w2; w[k][2] = w3;
  }
  float res[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
#pragma unroll
  for(int j = 0; j < 3; j++)
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
      float v[4];
      bilinear(p.hs, p.hw, p.hh, t[0][i], t[1][j], v);
#pragma unroll
      for(int k = 0; k < 4; k++) res[k] += v[k] * w[0][i] * w[1][j];
    }
  p.dm[(size_t)y * p.ow + x] = mk_half4(res[0], res[1], res[2], res[3]);
}

// crop/main.comp:19-55 on the demosaic output (ow x oh): per output pixel the
// input position, undoing in reverse order the window's corner, the rotation
// about the input's centre and the homography with its divide (matrix
// products summed column by column as GLSL's mat * vec; IEEE operations, as
// the position decides the texels read); then the nearest texel when there is
// no rotation (r0 == 1), else the Catmull-Rom filter; 0 outside the input;
// alpha 1
__global__ void __launch_bounds__(256) k_nd_crop(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.cw || y >= p.ch) return;
  const float *b = p.crop;
  const float tsx = (float)p.ow, tsy = (float)p.oh;
  const float px = __fadd_rn(__fadd_rn((float)x, 0.5f), __fmul_rn(b[16], tsx));
  const float py = __fadd_rn(__fadd_rn((float)y, 0.5f), __fmul_rn(b[18], tsy));
  const float vx = __fsub_rn(px, __fmul_rn(tsx, 0.5f)), vy = __fsub_rn(py, __fmul_rn(tsy, 0.5f));
  const float qx = __fadd_rn(__fadd_rn(__fmul_rn(b[12], vx), __fmul_rn(b[14], vy)), __fmul_rn(tsx, 0.5f));
  const float qy = __fadd_rn(__fadd_rn(__fmul_rn(b[13], vx), __fmul_rn(b[15], vy)), __fmul_rn(tsy, 0.5f));
  const float hx = __fadd_rn(__fadd_rn(__fmul_rn(b[0], qx), __fmul_rn(b[4], qy)), b[8]);
  const float hy = __fadd_rn(__fadd_rn(__fmul_rn(b[1], qx), __fmul_rn(b[5], qy)), b[9]);
  const float hz = __fadd_rn(__fadd_rn(__fmul_rn(b[2], qx), __fmul_rn(b[6], qy)), b[10]);
  const float rx = __fdiv_rn(__fdiv_rn(hx, hz), tsx), ry = __fdiv_rn(__fdiv_rn(hy, hz), tsy);
  float v[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
  // outside [0,1)^2 the output is 0; so is a position without value (hz = 0), which the
  // shader leaves undefined
  if(rx >= 0.0f && ry >= 0.0f && rx < 1.0f && ry < 1.0f)
  {
    if(b[12] != 1.0f) catmull_rom_uv(p.dm, p.ow, p.oh, rx, ry, v);
    else
    { // texelFetch(ivec2(rd * ts)); rd * ts may round up to ts, a read outside the image: 0
      const int ix = (int)__fmul_rn(rx, tsx), iy = (int)__fmul_rn(ry, tsy);
      if(ix < p.ow && iy < p.oh) ld4(p.dm, p.ow, ix, iy, v);
    }
  }
  p.cr[(size_t)y * p.cw + x] = mk_half4(v[0], v[1], v[2], 1.0f);
}

// ---------------------------------------------------------------- lens
// lens/main.comp:22-57, the double sphere camera model (V. Usenko, N. Demmel, D.
// Cremers, "The Double Sphere Camera Model", 2018): each output position,
// centred and scaled by the output's aspect, is unprojected with the two sphere
// radii (squish0, squish1), projected back to a pinhole, moved by the centre and
// sampled with the Catmull-Rom filter; with chromatic aberration factors other
// than (1, 1) red and blue sample at positions scaled about the image centre.
// The positions decide the texels the filter reads: IEEE operations in the
// shader's order (its divisions by 1 and additions of 0 are exact and left out).
// Extreme parameters can put a position anywhere (or make it NaN): every texel
// index is wrapped by the sampler's mirrored repeat, so no read leaves the image.
__global__ void __launch_bounds__(256) k_lens(const half4 *__restrict__ in, int w, int h, half4 *__restrict__ out,
    int ow, int oh, const lens_par_t q)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= ow || y >= oh) return;
  const float aspx = __fdiv_rn((float)ow, (float)oh);
  const float px = __fmul_rn(__fsub_rn(__fdiv_rn(__fadd_rn((float)x, 0.5f), (float)ow), 0.5f), aspx);
  const float py = __fsub_rn(__fdiv_rn(__fadd_rn((float)y, 0.5f), (float)oh), 0.5f);
  const float mx = __fdiv_rn(px, q.f[0]), my = __fdiv_rn(py, q.f[1]);
  const float r2 = __fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my));
  const float r0 = q.r[0], r1 = q.r[1];
  const float num = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(r0, r0), r2));
  const float sq = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(__fsub_rn(__fmul_rn(2.0f, r0), 1.0f), r2)));
  const float mz = __fdiv_rn(num, __fsub_rn(__fadd_rn(__fmul_rn(r0, sq), 1.0f), r0));
  const float a = __fadd_rn(__fmul_rn(mz, r1), __fsqrt_rn(__fadd_rn(__fmul_rn(mz, mz), __fsub_rn(1.0f, __fmul_rn(r1, r1)))));
  const float sc = __fdiv_rn(a, __fadd_rn(__fmul_rn(mz, mz), r2));
  const float X = __fmul_rn(sc, mx), Y = __fmul_rn(sc, my), Z = __fsub_rn(__fmul_rn(sc, mz), r1);
  const float ux = __fadd_rn(__fadd_rn(__fdiv_rn(__fdiv_rn(X, Z), aspx), 0.5f), q.c[0]);
  const float uy = __fadd_rn(__fadd_rn(__fdiv_rn(Y, Z), 0.5f), q.c[1]);
  float t[4];
  catmull_rom_uv<true>(in, w, h, ux, uy, t);
  float rgb[3] = { t[0], t[1], t[2] };
  if(!(q.ca[0] == 1.0f && q.ca[1] == 1.0f))
  {
    catmull_rom_uv<true>(in, w, h, __fadd_rn(__fmul_rn(__fsub_rn(ux, 0.5f), q.ca[0]), 0.5f),
                   __fadd_rn(__fmul_rn(__fsub_rn(uy, 0.5f), q.ca[0]), 0.5f), t);
    rgb[0] = t[0];
    catmull_rom_uv<true>(in, w, h, __fadd_rn(__fmul_rn(__fsub_rn(ux, 0.5f), q.ca[1]), 0.5f),
                   __fadd_rn(__fmul_rn(__fsub_rn(uy, 0.5f), q.ca[1]), 0.5f), t);
    rgb[2] = t[2];
  }
  out[(size_t)y * ow + x] = mk_half4(rgb[0], rgb[1], rgb[2], 1.0f);
}

// ---------------------------------------------------------------- bayer demosaic, node by node
// (demosaic colour param >= 1: fix.comp:124 widens the fix radius to 2, which
// the fused develop kernel's tile does not hold; gauss, splat and fix then run
// as the reference's nodes, with f16 images in HBM between them)

// demosaic/gauss.comp:24-75 (bayer): one thread per entry, the 8 greens at the
// mirrored texel centres 2 pos + 0.5 + (i, j) of the hilite output
__global__ void __launch_bounds__(256) k_nd_gauss_bayer(const dev_nodes_t p)
{
  const int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
  if(x >= p.hw || y >= p.hh) return;
  float px[8];
  int k = 0;
#pragma unroll
  for(int j = -1; j < 3; j++)
#pragma unroll
  for(int ii = -1; ii < 3; ii++)
  {
    if(((j + ii) & 1) != 1) continue;
    px[k++] = dn_m(p, p.hl, 2 * x + ii, 2 * y + j);
  }
  float v[4];
  int dec;
  gauss_exact(px, v, dec, p.neg_zero);
  p.cov[(size_t)y * p.hw + x] = mk_half4(v[0], v[1], v[2], v[3]);
  if(p.dbg_gauss) p.dbg_gauss[(size_t)y * p.hw + x] = (uint8_t)dec;
}

// exp(-0.5 dot(E o / eval, E o)) for the tap offset o = (i, j), E the
// eigenvector (c, s) and its normal (splat.comp:159-163, fix.comp:21-29)
DEV float gauss_w(float c, float s, float e0, float e1, int i, int j)
{
  const float of0 = c * (float)i + s * (float)j, of1 = -s * (float)i + c * (float)j;
  return expf(-0.5f * (of0 / e0 * of0 + of1 / e1 * of1));
}

// demosaic/splat.comp:142-266 (bayer): the greens of the 3x3 taps, centre
// weight 666, taps past the border wrapped by the CFA period 6
__global__ void __launch_bounds__(256) k_nd_splat_bayer(const dev_nodes_t p)
{
  const int x = blockIdx.x * 32 + threadIdx.x % 32, y = blockIdx.y * 8 + threadIdx.x / 32;
  if(x >= p.W || y >= p.H) return;
  float cov[4];
  cov_z(p, (x + 1) / 2, (y + 1) / 2, cov);
  const float e0 = gclamp(cov[0], 0.01f, 25.0f), e1 = gclamp(cov[1], 0.01f, 25.0f);
  float gs = 0.0f, gw = 0.0f;
#pragma unroll
  for(int j = -1; j <= 1; j++)
#pragma unroll
    for(int i = -1; i <= 1; i++)
    {
      if(cfa_bayer(x + i, y + j) != 1) continue;
      int px = x + i, py = y + j;
      if(px < 0) px += 6;
      if(py < 0) py += 6;
      if(px >= p.W) px -= 6;
      if(py >= p.H) py -= 6;
      const float w = (i == 0 && j == 0) ? 666.0f : gclamp(gauss_w(cov[2], cov[3], e0, e1, i, j), 1e-4f, 1.0f);
      gs += dn_z(p, p.hl, px, py) * w;
      gw += w;
    }
  p.g[(size_t)y * p.W + x] = f2h(gs / fmaxf(1e-8f, gw));
}

// demosaic/fix.comp:99-135 (bayer) with radius R: red and blue from the ratio
// of each tap to its splat green, weighted by the covariance of (x+1, y+1)/2
template<int R> __global__ void __launch_bounds__(256) k_nd_fix_bayer(const dev_nodes_t p)
{
  const int x = blockIdx.x * 32 + threadIdx.x % 32, y = blockIdx.y * 8 + threadIdx.x / 32;
  if(x >= p.W || y >= p.H) return;
  const float gc = dn_m(p, p.g, x, y);
  float cov[4];
  cov_z(p, (x + 1) / 2, (y + 1) / 2, cov);
  const float e0 = 2.0f * gclamp(cov[0], 1.0f, 49.0f), e1 = 2.0f * gclamp(cov[1], 1.0f, 49.0f);
  float rgb[3] = { 0.0f, 0.0f, 0.0f }, w[3] = { 0.0f, 0.0f, 0.0f };
#pragma unroll
  for(int j = -R; j <= R; j++)
#pragma unroll
    for(int i = -R; i <= R; i++)
    {
      const int c = cfa_bayer(x + i, y + j);
      if(c == 1) { rgb[1] = gc; w[1] = 1.0f; continue; }
      const float gh = dn_m(p, p.g, x + i, y + j), col = dn_m(p, p.hl, x + i, y + j);
      const float wt = gclamp(gauss_w(cov[2], cov[3], e0, e1, i, j), 1e-3f, 1.0f);
      rgb[c] += col * (1e-4f + gc) / (1e-4f + gh) * wt;
      w[c] += wt;
    }
  p.dm[(size_t)y * p.W + x] = mk_half4(rgb[0] / fmaxf(1e-8f, w[0]), rgb[1] / fmaxf(1e-8f, w[1]),
                                       rgb[2] / fmaxf(1e-8f, w[2]), 1.0f);
}

// ---------------------------------------------------------------- post
// colour -> histogram -> filmcurv -> llap/curve on the virtual positions
// [X0-1, X0+TX) of a tile and the first llap/reduce level of its outputs
// (the arithmetic of the tail of the fused develop kernel)
constexpr int TX = 32, TY = 32, NT = 256, NPL = 11;
constexpr int LX = TX + 1, LH = (LX + 1) / 2;

DEV int mirror1(int i, int n)
{
  if(i < 0) i = -1 - i;
  if(i >= n) i = 2 * n - 1 - i;
  return min(max(i, 0), n - 1);
}

// FC: the demosaic kernel applied colour, the histogram and filmcurv already
// (p.rgbf holds the filmcurv output); this kernel reads it for the llap curves
template<bool FC> __global__ void __launch_bounds__(NT) k_post(const dev_image_t p, const half4 *__restrict__ dm, int dm_pitch)
{
  __shared__ __half2 L0p[LLAP_PAIRS][LX][2][LH];        // the curve planes in pairs, [y][x & 1][x >> 1]
  __shared__ __align__(4) __half L0g[LX][LX + 1];       // the grey plane, [y][slot], rows of an even length
  __shared__ uint32_t hist[257];
  const int tid = threadIdx.x;
  const int W = p.W, H = p.H;
  // tiles are not shifted (nothing here wraps by the CFA period): slots past
  // the image hold the mirrored texel, as the level 1 reduce reads them
  const int OX = blockIdx.x * TX, OY = blockIdx.y * TY;
  const int X0 = OX, Y0 = OY;
  const int OXe = min(OX + TX, W), OYe = min(OY + TY, H);
  if(p.hist) for(int i = tid; i < 257; i += NT) hist[i] = 0;
  __syncthreads();
  const float sig = p.ll_sigma, shd = p.ll_shadows, hil = p.ll_highlights, cla = p.ll_clarity;
  const float r2s = 1.0f / (2.0f * sig), rden = 1.0f / (2.0f * sig * sig / 3.0f);
  const bool unit_curve = shd == 1.0f && hil == 1.0f;
  for(int t = tid; t < LX * LX; t += NT)
  {
    const int slx = t % LX, sly = t / LX;
    const int vx = X0 - 1 + slx, vy = Y0 - 1 + sly;
    const int px = mirror1(vx, W), py = mirror1(vy, H);
    float fc[3];
    if(FC)
    {
      float a;
      ld_half4(p.rgbf + (size_t)py * W + px, fc[0], fc[1], fc[2], a);
    }
    else
    {
      float d[4];
      ld_half4(dm + (size_t)py * dm_pitch + px, d[0], d[1], d[2], d[3]);
      float co[3];
      colour_px(p, d, co);
      const bool own = vx == px && vy == py && px >= OX && px < OXe && py >= OY && py < OYe;
      if(own && p.dbg_colour) p.dbg_colour[(size_t)py * W + px] = mk_half4(co[0], co[1], co[2], 1.0f);
      if(own && p.hist)
      {
        const uint32_t bin = hist_bin(co[0], co[1], co[2]);
        if(bin > 0) { atomicAdd(&hist[bin], 1u); atomicAdd(&hist[256], 1u); }
      }
      filmcurv_px(p, co, fc);
      if(own) p.rgbf[(size_t)py * W + px] = mk_half4(fc[0], fc[1], fc[2], 1.0f);
    }
    const float yv = lum2020(gclamp(fc[0], -1000.0f, 1000.0f), gclamp(fc[1], -1000.0f, 1000.0f), gclamp(fc[2], -1000.0f, 1000.0f));
    if(unit_curve)
    {
      const float2 X = make_float2(yv, yv), nr = make_float2(-rden, -rden), cl = make_float2(cla, cla);
#pragma unroll
      for(int j = 0; j < LLAP_PAIRS; j++) L0p[j][sly][slx & 1][slx >> 1] = llap_curve_unit2(X, j, nr, cl);
    }
    else
    {
#pragma unroll
      for(int j = 0; j < LLAP_PAIRS; j++)
        L0p[j][sly][slx & 1][slx >> 1] = __floats2half2_rn(llap_curve_rcp(yv, kLlapGamma[2 * j], sig, r2s, rden, shd, hil, cla),
                                                           llap_curve_rcp(yv, kLlapGamma[2 * j + 1], sig, r2s, rden, shd, hil, cla));
    }
    L0g[sly][slx] = f2h(yv);
  }
  __syncthreads();
  // llap/reduce.comp (sample_semisoft) for level 1 outputs [X0/2, X0/2+TX/2): a warp takes 16
  // outputs of row ly and 16 of row ly + 4 (its halves read pair words 16 banks apart)
  {
    const int w = tid >> 5, lx = tid & 15;
    const int ly = (w & 3) + 8 * (w >> 2) + 4 * ((tid >> 4) & 1);
    const int ox = X0 / 2 + lx, oy = Y0 / 2 + ly;
    const bool own = ox >= OX / 2 && ox < min(OX / 2 + TX / 2, p.l1w) && oy >= OY / 2 && oy < min(OY / 2 + TY / 2, p.l1h);
    if(own)
    { // level 0 slot of virtual x = 2ox + a - 1 is 2lx + a: pair words [.][0][lx], [.][1][lx], [.][0][lx + 1]
      const size_t o = (size_t)oy * p.l1pitch + ox;
#pragma unroll
      for(int j = 0; j < LLAP_PAIRS; j++)
      {
        const __half2 *a[3], *b[3], *c[3];
#pragma unroll
        for(int r = 0; r < 3; r++)
        {
          a[r] = &L0p[j][2 * ly + r][0][lx];
          b[r] = &L0p[j][2 * ly + r][1][lx];
          c[r] = &L0p[j][2 * ly + r][0][lx + 1];
        }
        const float2 v = llap_reduce_px2(a, b, c);
        p.l1[(2 * j) * p.l1plane + o] = f2h(v.x);
        p.l1[(2 * j + 1) * p.l1plane + o] = f2h(v.y);
      }
      const __half *const row[3] = { &L0g[2 * ly][2 * lx], &L0g[2 * ly + 1][2 * lx], &L0g[2 * ly + 2][2 * lx] };
      p.l1[(NPL - 1) * p.l1plane + o] = f2h(llap_reduce_px(row));
    }
  }
  if(!FC && p.hist)
  {
    __syncthreads();
    for(int i = tid; i < 257; i += NT) if(hist[i]) atomicAdd(p.hist + i, hist[i]);
  }
}

} // namespace

cudaError_t launch_nodes(const dev_nodes_t &p, int stage, cudaStream_t s)
{
  const bool xt = p.filters == 9u;
  const dim3 gh((p.hw + 15) / 16, (p.hh + 15) / 16), gf((p.W + 31) / 32, (p.H + 7) / 8);
  switch(stage)
  {
    case 0: k_nd_noop<<<dim3((p.W + 63) / 64, (p.H + 3) / 4), 256, 0, s>>>(p); break;
    case 1: if(xt) k_nd_hl_half<true><<<gh, 256, 0, s>>>(p); else k_nd_hl_half<false><<<gh, 256, 0, s>>>(p); break;
    case 2: if(xt) k_nd_hl_doub<true><<<gh, 256, 0, s>>>(p); else k_nd_hl_doub<false><<<gh, 256, 0, s>>>(p); break;
    case 3: if(xt) k_nd_gauss_xt<<<gh, 256, 0, s>>>(p); else k_nd_gauss_bayer<<<gh, 256, 0, s>>>(p); break;
    case 4:
      if(xt) k_nd_splat_xt<<<dim3((p.W + XT_TX - 1) / XT_TX, (p.H + XT_TY - 1) / XT_TY), 256, 0, s>>>(p);
      else k_nd_splat_bayer<<<gf, 256, 0, s>>>(p);
      break;
    case 5:
      if(xt)
      { // fix.comp:111 radius clamp(fixup + 2, 2, 3)
        const dim3 g((p.W + XT_TX - 1) / XT_TX, (p.H + XT_TY - 1) / XT_TY);
        if(p.fixup >= 1) k_nd_fix_xt<3><<<g, 256, 0, s>>>(p); else k_nd_fix_xt<2><<<g, 256, 0, s>>>(p);
      }
      else
      { // fix.comp:124 radius clamp(fixup + 1, 1, 2)
        if(p.fixup >= 1) k_nd_fix_bayer<2><<<gf, 256, 0, s>>>(p); else k_nd_fix_bayer<1><<<gf, 256, 0, s>>>(p);
      }
      break;
    case 6: if(xt) k_nd_halfsize<true><<<gh, 256, 0, s>>>(p); else k_nd_halfsize<false><<<gh, 256, 0, s>>>(p); break;
    case 9: k_nd_crop<<<dim3((p.cw + 15) / 16, (p.ch + 15) / 16), 256, 0, s>>>(p); break;
    case 7: k_nd_resample<<<dim3((p.ow + 15) / 16, (p.oh + 15) / 16), 256, 0, s>>>(p); break;
    case 8: k_nd_hl_bayer<<<gh, 256, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_lens(const half4 *in, int w, int h, half4 *out, int ow, int oh, const lens_par_t &q, cudaStream_t s)
{
  k_lens<<<dim3((ow + 15) / 16, (oh + 15) / 16), 256, 0, s>>>(in, w, h, out, ow, oh, q);
  return cudaGetLastError();
}

cudaError_t launch_post(const dev_image_t &p, const half4 *dm, int dm_pitch, cudaStream_t s)
{
  if(dm) k_post<false><<<dim3((p.W + TX - 1) / TX, (p.H + TY - 1) / TY), NT, 0, s>>>(p, dm, dm_pitch);
  else    k_post<true><<<dim3((p.W + TX - 1) / TX, (p.H + TY - 1) / TY), NT, 0, s>>>(p, dm, dm_pitch);
  return cudaGetLastError();
}
