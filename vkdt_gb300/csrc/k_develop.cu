// The fused full resolution pass of the path (bayer):
//   hilite/doub (with the level 0 hilite/assemble and denoise/noop recomputed
//   from the mosaic) -> demosaic/gauss -> demosaic/splat -> demosaic/fix ->
//   colour/main -> [OpenDRT/hist] -> filmcurv/main -> llap/curve -> the first
//   llap/reduce level.
// Every intermediate image the reference stores (all f16) is rounded to f16
// at the same point here, but lives only in shared memory. HBM sees the u16
// mosaic in, the filmcurv output (rgba f16, needed by llap/colour) and the 11
// level 1 planes of the llap pyramid out.
//
// Tiling: one CTA computes a TX x TY tile of output pixels. Every stage is
// evaluated on the halo its consumer needs (slots indexed by "virtual"
// positions that hold the value of the mirrored real position, which is what
// a MIRRORED_REPEAT texture read returns). The last tile of a row/column is
// shifted inwards so that the 6 pixel wrap of demosaic/splat.comp:153-156
// always lands inside the tile's slots; outputs are written by the owner only.
#include "common.cuh"
#include "hilite.cuh"
#include "kernels.h"
#include "pixel.cuh"

namespace {

constexpr int TX = 32, TY = 32;
constexpr int MX = TX + 8, MY = TY + 8;          // hilite output mosaic: virtual [X0-4, X0+TX+4)
constexpr int CX = TX / 2 + 2, CY = TY / 2 + 2;  // demosaic/gauss: half positions [X0/2-1, X0/2+TX/2+1)
constexpr int GX = TX + 3, GY = TY + 3;          // demosaic/splat: virtual [X0-2, X0+TX+1)
constexpr int LX = TX + 1, LY = TY + 1;          // llap level 0: virtual [X0-1, X0+TX)
constexpr int NPL = 11;                          // NUM_GAMMA curves + grey (llap/config.h:2)
constexpr int NT = 256;

struct smem_t
{
  float M[MY][MX];
  float cov[4][CY][CX];
  float g[GY][GX];
  __half L0[NPL][LY][LX + 1];
  uint32_t hist[257];
};

// the hilite output (module output) of one 2x2 block at real block (bx, by):
// denoise/noop of the block, hilite/half, the level 0 hilite/assemble against
// the stored coarse level, then hilite/doub
DEV void mosaic_block(const dev_image_t &p, int bx, int by, float out[4], float m[4])
{
  const int hw = p.W / 2, hh = p.H / 2;
  m[0] = noop_val(p.mosaic, p.pitch, p.cx, p.cy, p.W, p.H, 2 * bx, 2 * by, p.black, p.white);
  m[1] = noop_val(p.mosaic, p.pitch, p.cx, p.cy, p.W, p.H, 2 * bx + 1, 2 * by, p.black, p.white);
  m[2] = noop_val(p.mosaic, p.pitch, p.cx, p.cy, p.W, p.H, 2 * bx, 2 * by + 1, p.black, p.white);
  m[3] = noop_val(p.mosaic, p.pitch, p.cx, p.cy, p.W, p.H, 2 * bx + 1, 2 * by + 1, p.black, p.white);
  float h[4];
  hilite_half_bayer(m[0], m[1], m[2], m[3], p.hl_white, h);
  h[3] = 1.0f;
  float up[3];
  hilite_expand_px([&](int ix, int iy, float rgb[3]) {
      const int sx = mirror_full(ix, p.hcw), sy = mirror_full(iy, p.hch);
      float w;
      ld_half4(p.hl_coarse + (size_t)sy * p.hcw + sx, rgb[0], rgb[1], rgb[2], w);
    }, bx, by, up);
  float b0[3];
  hilite_assemble_px(h, up, p.hl_white, p.hl_soft, b0);
  (void)hw; (void)hh;
  hilite_doub_bayer(m[0], m[1], m[2], m[3], b0, p.hl_white, out);
}

// colour/main-impl.glsl:200-341 on the matrix path (no clut/pick/rbf, sat 1)
DEV void colour_px(const dev_image_t &p, const float in[3], float o[3])
{
  float r[3], cl[3], q[3];
  for(int i = 0; i < 3; i++) r[i] = p.cam[3 * i + 0] * in[0] + p.cam[3 * i + 1] * in[1] + p.cam[3 * i + 2] * in[2];
  for(int i = 0; i < 3; i++) cl[i] = p.P[3 * i + 0] * r[0] + p.P[3 * i + 1] * r[1] + p.P[3 * i + 2] * r[2];
  for(int i = 0; i < 3; i++) cl[i] *= p.clscale[i];
  for(int i = 0; i < 3; i++) q[i] = p.Q[3 * i + 0] * cl[0] + p.Q[3 * i + 1] * cl[1] + p.Q[3 * i + 2] * cl[2];
  for(int i = 0; i < 3; i++) o[i] = f16r(gclamp(q[i] * p.mulw, -65535.0f, 65535.0f));
}

DEV float weibull_cdf(float x, float il, float k)
{ // filmcurv/params.glsl:15-34
  return 1.0f - expf(-powf(fmaxf(x, 1e-7f) * il, k));
}

// filmcurv/main.comp:106-205, colour modes 1 and 3 (adjust_colour_dng, shared.glsl:371-387)
DEV void filmcurv_px(const dev_image_t &p, const float in[3], float o[3])
{
  float c0[3], c1[3];
  for(int k = 0; k < 3; k++) c0[k] = in[k] + p.fc_bias;
  for(int k = 0; k < 3; k++) c1[k] = weibull_cdf(c0[k], p.fc_il, p.fc_k);
  if(p.fc_mode == 3)
  {
    bool fx = false, fy = false, fz = false;
    float t;
    if(c0[2] > c0[1]) { t = c0[2]; c0[2] = c0[1]; c0[1] = t; t = c1[2]; c1[2] = c1[1]; c1[1] = t; fx = true; }
    if(c0[1] > c0[0]) { t = c0[0]; c0[0] = c0[1]; c0[1] = t; t = c1[0]; c1[0] = c1[1]; c1[1] = t; fy = true; }
    if(c0[2] > c0[1]) { t = c0[2]; c0[2] = c0[1]; c0[1] = t; t = c1[2]; c1[2] = c1[1]; c1[1] = t; fz = true; }
    c1[1] = gmix(c1[2], c1[0], (c0[1] - c0[2] + 1e-6f) / (c0[0] - c0[2] + 1e-6f));
    if(fz) { t = c1[2]; c1[2] = c1[1]; c1[1] = t; }
    if(fy) { t = c1[0]; c1[0] = c1[1]; c1[1] = t; }
    if(fx) { t = c1[2]; c1[2] = c1[1]; c1[1] = t; }
  }
  for(int k = 0; k < 3; k++) o[k] = f16r(c1[k]);
}

} // namespace

namespace {

__global__ void __launch_bounds__(NT) k_develop(const dev_image_t p)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  smem_t &s = *reinterpret_cast<smem_t *>(smem_raw);
  const int tid = threadIdx.x;
  const int W = p.W, H = p.H, hw = W / 2, hh = H / 2;
  // owned output range and the (possibly shifted) tile origin
  const int OX = blockIdx.x * TX, OY = blockIdx.y * TY;
  const int X0 = W >= TX ? min(OX, W - TX) : 0;
  const int Y0 = H >= TY ? min(OY, H - TY) : 0;
  const int OXe = min(OX + TX, W), OYe = min(OY + TY, H);
  if(p.hist) for(int i = tid; i < 257; i += NT) s.hist[i] = 0;

  // ---- hilite output mosaic on virtual blocks [X0/2-2, X0/2+TX/2+2)
  {
    const int hx0 = X0 / 2 - 2, hy0 = Y0 / 2 - 2;
    for(int i = tid; i < (MX / 2) * (MY / 2); i += NT)
    {
      const int sbx = i % (MX / 2), sby = i / (MX / 2);
      const int vbx = hx0 + sbx, vby = hy0 + sby;
      const int rbx = mirror_full(vbx, hw), rby = mirror_full(vby, hh);
      const bool fx = vbx < 0 || vbx >= hw, fy = vby < 0 || vby >= hh;
      float o[4], m[4];
      mosaic_block(p, rbx, rby, o, m);
      for(int dy = 0; dy < 2; dy++) for(int dx = 0; dx < 2; dx++)
        s.M[2 * sby + dy][2 * sbx + dx] = o[(fy ? 1 - dy : dy) * 2 + (fx ? 1 - dx : dx)];
      if(p.dbg_denoise && !fx && !fy && 2 * rbx >= OX && 2 * rbx < OXe && 2 * rby >= OY && 2 * rby < OYe)
        for(int dy = 0; dy < 2; dy++) for(int dx = 0; dx < 2; dx++)
        {
          const size_t idx = (size_t)(2 * rby + dy) * W + 2 * rbx + dx;
          p.dbg_denoise[idx] = f2h(m[dy * 2 + dx]);
          p.dbg_hilite[idx] = f2h(o[dy * 2 + dx]);
        }
    }
  }
  __syncthreads();

  // ---- demosaic/gauss.comp:24-75 (bayer) on half positions [X0/2-1, X0/2+TX/2+1)
  for(int i = tid; i < CX * CY; i += NT)
  {
    const int scx = i % CX, scy = i / CX;
    const int cx = X0 / 2 - 1 + scx, cy = Y0 / 2 - 1 + scy;
    float v[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
    if(cx >= 0 && cy >= 0 && cx < hw && cy < hh)
    {
      // M slot of virtual (2cx+i, 2cy+j) = [2scy+2+j][2scx+2+i]
      float mw0 = 0, mw1 = 0, mb0 = 0, mb1 = 0, smw = 0, smb = 0;
      for(int j = -1; j < 3; j++) for(int ii = -1; ii < 3; ii++)
      {
        if(((j + ii) & 1) != 1) continue;
        const float px = s.M[2 * scy + 2 + j][2 * scx + 2 + ii];
        mw0 += (float)ii * px; mw1 += (float)j * px;
        smw += px;
        mb0 += (float)ii / px; mb1 += (float)j / px;
        smb += 1.0f / px;
      }
      mw0 /= smw; mw1 /= smw;
      mb0 /= smb; mb1 /= smb;
      float Sw00 = 0, Sw01 = 0, Sw10 = 0, Sw11 = 0, Sb00 = 0, Sb01 = 0, Sb10 = 0, Sb11 = 0, sw = 0, sb = 0;
      for(int j = -1; j < 3; j++) for(int ii = -1; ii < 3; ii++)
      {
        if(((j + ii) & 1) != 1) continue;
        const float px = s.M[2 * scy + 2 + j][2 * scx + 2 + ii];
        float p2 = px * px;
        float q0 = (float)ii - mw0, q1 = (float)j - mw1;
        Sw00 += p2 * q0 * q0; Sw01 += p2 * q0 * q1; Sw10 += p2 * q1 * q0; Sw11 += p2 * q1 * q1;
        sw += p2;
        q0 = (float)ii - mb0; q1 = (float)j - mb1;
        p2 = 1.0f / p2;
        Sb00 += p2 * q0 * q0; Sb01 += p2 * q0 * q1; Sb10 += p2 * q1 * q0; Sb11 += p2 * q1 * q1;
        sb += p2;
      }
      Sw00 /= sw; Sw01 /= sw; Sw10 /= sw; Sw11 /= sw;
      Sb00 /= sb; Sb01 /= sb; Sb10 /= sb; Sb11 /= sb;
      const float detw = Sw00 * Sw11 - Sw10 * Sw01, detb = Sb00 * Sb11 - Sb10 * Sb01;
      float eval[2], evec0[2], evec1[2];
      if(detw < detb) evd2x2(eval, evec0, evec1, Sw00, Sw10, Sw11);
      else            evd2x2(eval, evec0, evec1, Sb00, Sb10, Sb11);
      eval[0] *= 0.2f; eval[1] *= 0.2f;
      if(fabsf(evec0[0]) > fabsf(evec0[1])) { evec0[0] = 1.0f; evec0[1] = 0.0f; }
      else                                  { evec0[0] = 0.0f; evec0[1] = 1.0f; }
      v[0] = f16r(eval[0]); v[1] = f16r(eval[1]); v[2] = f16r(evec0[0]); v[3] = f16r(evec0[1]);
    }
    for(int k = 0; k < 4; k++) s.cov[k][scy][scx] = v[k];
  }
  __syncthreads();

  // ---- demosaic/splat.comp:224-266 (bayer) on virtual [X0-2, X0+TX+1)
  for(int i = tid; i < GX * GY; i += NT)
  {
    const int sgx = i % GX, sgy = i / GX;
    const int qx = mirror_full(X0 - 2 + sgx, W), qy = mirror_full(Y0 - 2 + sgy, H);
    const int ccx = (qx + 1) / 2 - (X0 / 2 - 1), ccy = (qy + 1) / 2 - (Y0 / 2 - 1);
    const float c0 = s.cov[0][ccy][ccx], c1 = s.cov[1][ccy][ccx], c2 = s.cov[2][ccy][ccx], c3 = s.cov[3][ccy][ccx];
    const float e0 = gclamp(c0, 0.01f, 25.0f), e1 = gclamp(c1, 0.01f, 25.0f);
    float rg = 0.0f, wg = 0.0f;
#pragma unroll
    for(int j = -1; j <= 1; j++)
#pragma unroll
    for(int ii = -1; ii <= 1; ii++)
    {
      if(cfa_bayer(qx + ii, qy + j) != 1) continue; // only green enters rgb.ggg
      int px = qx + ii, py = qy + j;
      if(px < 0) px += 6;
      if(py < 0) py += 6;
      if(px >= W) px -= 6;
      if(py >= H) py -= 6;
      const float col = s.M[py - (Y0 - 4)][px - (X0 - 4)];
      const float of0 = c2 * (float)ii + c3 * (float)j;
      const float of1 = -c3 * (float)ii + c2 * (float)j;
      float weight = gclamp(expf(-0.5f * (of0 / e0 * of0 + of1 / e1 * of1)), 1e-4f, 1.0f);
      if(ii == 0 && j == 0) weight = 666.0f;
      rg += col * weight;
      wg += weight;
    }
    s.g[sgy][sgx] = f16r(rg / fmaxf(1e-8f, wg));
  }
  __syncthreads();

  // ---- demosaic/fix -> colour -> hist -> filmcurv -> llap/curve on virtual [X0-1, X0+TX)
  const float sig = p.ll_sigma, sh = p.ll_shadows, hl = p.ll_highlights, cl = p.ll_clarity;
  for(int i = tid; i < LX * LY; i += NT)
  {
    const int slx = i % LX, sly = i / LX;
    const int vx = X0 - 1 + slx, vy = Y0 - 1 + sly;
    const int px = mirror_full(vx, W), py = mirror_full(vy, H);
    const float gc = s.g[py - (Y0 - 2)][px - (X0 - 2)];
    const int ccx = (px + 1) / 2 - (X0 / 2 - 1), ccy = (py + 1) / 2 - (Y0 / 2 - 1);
    const float cv2 = s.cov[2][ccy][ccx], cv3 = s.cov[3][ccy][ccx];
    const float e0 = 2.0f * gclamp(s.cov[0][ccy][ccx], 1.0f, 49.0f), e1 = 2.0f * gclamp(s.cov[1][ccy][ccx], 1.0f, 49.0f);
    float rgb[3] = { 0.0f, 0.0f, 0.0f }, w[3] = { 0.0f, 0.0f, 0.0f };
    // demosaic/fix.comp:99-135, radius clamp(fixup+1, 1, 2) = 1 for the
    // default fixup 0 (the host rejects other values for this kernel)
#pragma unroll
    for(int j = -1; j <= 1; j++)
#pragma unroll
    for(int ii = -1; ii <= 1; ii++)
    {
      const int c = cfa_bayer(px + ii, py + j);
      if(c == 1) { rgb[1] = gc; w[1] = 1.0f; continue; }
      const float gh = s.g[py + j - (Y0 - 2)][px + ii - (X0 - 2)];
      const float col = s.M[py + j - (Y0 - 4)][px + ii - (X0 - 4)];
      const float of0 = cv2 * (float)ii + cv3 * (float)j;
      const float of1 = -cv3 * (float)ii + cv2 * (float)j;
      const float weight = gclamp(expf(-0.5f * (of0 / e0 * of0 + of1 / e1 * of1)), 1e-3f, 1.0f);
      rgb[c] += col * (1e-4f + gc) / (1e-4f + gh) * weight;
      w[c] += weight;
    }
    float dm[3];
    for(int k = 0; k < 3; k++) dm[k] = f16r(rgb[k] / fmaxf(1e-8f, w[k]));
    float co[3];
    colour_px(p, dm, co);
    const bool own = vx == px && vy == py && px >= OX && px < OXe && py >= OY && py < OYe;
    if(own && p.hist)
    {
      const uint32_t bin = hist_bin(co[0], co[1], co[2]);
      if(bin > 0) { atomicAdd(&s.hist[bin], 1u); atomicAdd(&s.hist[256], 1u); }
    }
    float fc[3];
    filmcurv_px(p, co, fc);
    if(own) p.rgbf[(size_t)py * W + px] = mk_half4(fc[0], fc[1], fc[2], 1.0f);
    const float yv = lum2020(gclamp(fc[0], -1000.0f, 1000.0f), gclamp(fc[1], -1000.0f, 1000.0f), gclamp(fc[2], -1000.0f, 1000.0f));
#pragma unroll
    for(int k = 0; k < NPL - 1; k++) s.L0[k][sly][slx] = f2h(llap_curve_fn(yv, llap_gamma(k), sig, sh, hl, cl));
    s.L0[NPL - 1][sly][slx] = f2h(yv);
  }
  __syncthreads();

  // ---- llap/reduce.comp (sample_semisoft) for level 1 outputs [X0/2, X0/2+TX/2)
  {
    const int lx = tid % (TX / 2), ly = tid / (TX / 2);
    const int ox = X0 / 2 + lx, oy = Y0 / 2 + ly;
    const bool own = ox >= OX / 2 && ox < min(OX / 2 + TX / 2, p.l1w) && oy >= OY / 2 && oy < min(OY / 2 + TY / 2, p.l1h);
    if(own)
    {
      // level 0 slot of virtual x = 2ox + a - 1 is 2lx + a
      for(int k = 0; k < NPL; k++)
      {
        float t[3][3];
        for(int b = 0; b < 3; b++) for(int a = 0; a < 3; a++) t[b][a] = h2f(s.L0[k][2 * ly + b][2 * lx + a]);
        const float q00 = (t[0][0] * 0.5f + t[0][1] * 0.5f) * 0.5f + (t[1][0] * 0.5f + t[1][1] * 0.5f) * 0.5f;
        const float q10 = (t[0][1] * 0.5f + t[0][2] * 0.5f) * 0.5f + (t[1][1] * 0.5f + t[1][2] * 0.5f) * 0.5f;
        const float q01 = (t[1][0] * 0.5f + t[1][1] * 0.5f) * 0.5f + (t[2][0] * 0.5f + t[2][1] * 0.5f) * 0.5f;
        const float q11 = (t[1][1] * 0.5f + t[1][2] * 0.5f) * 0.5f + (t[2][1] * 0.5f + t[2][2] * 0.5f) * 0.5f;
        const float r = (((q00 + q10) + q01) + q11) / 4.0f;
        p.l1[k * p.l1plane + (size_t)oy * p.l1w + ox] = f2h(r);
      }
    }
  }
  if(p.hist)
  {
    __syncthreads();
    for(int i = tid; i < 257; i += NT) if(s.hist[i]) atomicAdd(p.hist + i, s.hist[i]);
  }
}

} // namespace

cudaError_t launch_develop(const dev_image_t &p, cudaStream_t s)
{
  const size_t smem = sizeof(smem_t);
  static_assert(sizeof(smem_t) <= 48 * 1024, "develop tile needs the opt-in shared memory size");
  dim3 grid((p.W + TX - 1) / TX, (p.H + TY - 1) / TY);
  k_develop<<<grid, NT, smem, s>>>(p);
  return cudaGetLastError();
}
