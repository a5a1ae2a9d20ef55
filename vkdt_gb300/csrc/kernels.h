// Launch interface between the host graph (graph.cpp) and the CUDA kernels.
// Plain structs of pointers and scalars; no torch types.
#pragma once
#include <cuda.h>            // CUtensorMap
#include <cudaTypedefs.h>    // PFN_cuTensorMapEncodeTiled
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stddef.h>

struct half4;

// how the kernels turn a mosaic's u16 codes into the normalised values of the
// path: denoise/noop.comp:36-57 on (black, white) evaluated per code, or, where
// the mosaic pointer reads the wavelet output (f16), the f16 bits themselves
struct dev_codes_t { float black, white; int identity; };

// per image constants of the path, filled by the host from the module
// parameters and the image metadata (the uniforms and push constants the
// modules' commit_params / create_nodes would upload)
struct dev_image_t
{
  // mosaic (source) and its active window
  const uint16_t *mosaic;
  const __half *noop_lut; // denoise/noop of every u16 code (65536 f16)
  dev_codes_t codes;    // the same values evaluated per code
  int pitch;            // elements per mosaic row
  int cx, cy;           // crop offset (denoise push.crop.xy)
  int W, H;             // denoise/hilite output size
  uint32_t filters;
  // denoise noop, channel 0, unorm units
  float black, white;
  float neg_zero;       // -0.0f: an fma addend the compiler cannot fold (gauss_exact)
  // hilite/params
  float hl_white, hl_desat, hl_soft;
  float wb[3];
  // hilite pyramid: coarse input of the level 0 assemble (B_1 or r_1)
  const half4 *hl_coarse;
  int hcw, hch;
  // demosaic/params
  int fixup;
  // colour: camera matrix, cat16 matrices and per channel cone scale, exposure
  float cam[9], P[9], Q[9], clscale[3], mulw;
  float cmat[9];        // their product mulw Q diag(clscale) P cam, made once per image in double precision
  // filmcurv
  float fc_il, fc_k, fc_bias;
  int fc_mode;
  // llap
  float ll_sigma, ll_shadows, ll_highlights, ll_clarity;
  // a crop after demosaic that moves the image by whole texels (crop/main.comp's
  // texelFetch of (x + dx, y + dy)): the outputs below are the window's, at crop
  // coordinates (dx = dy = 0 and the demosaic size without a crop)
  int crop_dx, crop_dy, crop_w, crop_h;
  // outputs of the develop kernel
  half4 *rgbf;          // filmcurv output, crop_w*crop_h rgba f16
  __half *l1;           // llap level 1, 11 planes (null: the develop kernel ends at filmcurv)
  int l1w, l1h;
  int l1pitch;          // elements per row (the width rounded up to 16 bytes)
  size_t l1plane;       // elements per plane
  uint32_t *hist;       // 257 counts or null
  // debug copies (null in production)
  __half *dbg_denoise, *dbg_hilite;
  half4 *dbg_demosaic, *dbg_colour;   // demosaic output (W*H) and colour output (crop_w*crop_h)
  uint8_t *dbg_gauss;                 // demosaic/gauss decisions per entry (GAUSS_DEC bits)
};

// the discrete decisions of demosaic/gauss.comp per entry, written by the
// debug stages: bit 0 det(Sw) < det(Sb) (the structure tensor taken); bits
// 1-2 the snapped direction: 0 (1,0), 1 (0,1), 2 none (x-trans: isotropic)
enum { GAUSS_DEC_USEW = 1, GAUSS_DEC_SNAP_SHIFT = 1 };

struct dev_hilite_k1_t
{
  const uint16_t *mosaic;
  dev_codes_t codes;
  int pitch, cx, cy, W, H;
  uint32_t filters;
  float black, white, hl_white, hl_desat;
  float wb[3];
  int hw, hh;          // h0 size (W/2, H/2)
  half4 *r1;
  int s1w, s1h;
};

struct dev_llap_k3_t
{
  const half4 *rgbf;    // filmcurv output
  int W, H;
  const __half *l1;     // level 1 planes
  int l1w, l1h, l1pitch;
  size_t l1plane;
  const __half *coarse; // A[1] at level 1 size (row pitch l1pitch), or the grey plane of level 1 when the pyramid has 2 levels
  float ll_sigma, ll_shadows, ll_highlights, ll_clarity;
  // grade/main.comp after llap when the graph connects it (0 none, 1 classic, 2 zoned log):
  // lift, gamma, gain, offset with their fourth component added, sh_pivot, hi_pivot
  int grade;
  float gr_lift[3], gr_gamma[3], gr_gain[3], gr_off[3], gr_sp, gr_hp;
  half4 *out;           // rgba f16 W*H
};

// denoise wavelet path (strength > 0): the push constants and uniforms of
// denoise/main.c:133-333 and the half size node buffers
struct dev_denoise_t
{
  const uint16_t *mosaic;
  int pitch, in_w, in_h; // input mosaic layout (mirrored reads cover the full input)
  int cx, cy, W, H;      // crop offset and module output size
  int hw, hh;            // half size (W/block, H/block)
  uint32_t filters;      // 9 x-trans, else bayer
  float black[3], white[3], wb[3];  // unorm black/white per channel, camera white balance
  float wb_norm[3], wb_denorm[3];   // wb / (white - black) and its inverse (assemble)
  float na, nb;          // noise profile (normalised)
  float edge_gain[3];    // exp2(12 edges.rgb + edges.a) of noise_sigma
  float strength, luma, detail, thrs0;  // params; thrs0 = strength^4
  float block_f;         // 1.414213 (bayer), 2.23607 (x-trans)
  int doub_fixed;        // bayer, W = 2 hw, H = 2 hh, doub's taps at fixed places (checked on the host)
  int fuse_half;         // bayer: the downcov launch makes the half image (no half launch)
  float neg_zero;        // -0.0f (an addend the compiler cannot fold, k_dn_downcov)
  float bscale[4];       // 0.7^(l+1) / block_f, l = 0..3 (assemble.comp)
  float pl[4];           // 0.7^level
  float rgb_to_yuv[9], yuv_to_rgb[9];
  half4 *half_img;       // denoise/half output
  half4 *lvl[4];         // downcov, down 1..3 outputs (swizzled)
  half4 *asm_img;        // assemble output
  __half *dn;            // doub output: the denoised normalised mosaic, W*H
  // debug decisions (null in production), per half size texel: cov.glsl
  // response(): bits 0-24 the hot pixel skip of tap (i+2) + 5 (j+2), bit 25
  // det(Sw) < det(Sb); assemble.comp: bit l the threshold switch |d_l| > 10
  uint32_t *dbg_cov;
  uint8_t *dbg_thr;
};
// stage 0 half, 1 downcov, 2..4 down levels 1..3, 5 assemble, 6 doub (k_denoise.cu);
// with fuse_half stage 0 is not launched: stage 1 makes the half image too
cudaError_t launch_denoise(const dev_denoise_t &p, int stage, cudaStream_t s);

// the per-node chain for what the fused develop kernel does not cover
// (x-trans mosaics, reduced output sizes): buffers and sizes (k_nodes.cu)
struct dev_nodes_t
{
  float neg_zero;        // -0.0f: an fma addend the compiler cannot fold (gauss_exact)
  const uint16_t *mosaic;
  const __half *noop_lut; // denoise/noop of every u16 code (L1 resident in these kernels)
  int pitch, cx, cy;     // source layout and crop offset
  int W, H;              // denoise / hilite size
  uint32_t filters;
  int block, hw, hh;     // 2 bayer, 3 x-trans; hw = W / block
  float hl_white;
  int fixup;             // demosaic colour param
  int ow, oh;            // demosaic output size
  __half *dn;            // normalised (or denoised) mosaic, W*H
  half4 *h0;             // hilite/half, hw*hh
  const half4 *b0;       // hilite level 0 assembled (coarse input of doub), hw*hh
  __half *hl;            // hilite/doub output mosaic, W*H
  half4 *cov;            // demosaic/gauss (x-trans), hw*hh
  __half *g;             // demosaic/splat, W*H
  half4 *hs;             // demosaic/halfsize, hw*hh
  half4 *dm;             // demosaic output, ow*oh
  const half4 *coarse;   // assembled hilite level 1 (or reduce level 1 when the pyramid has one level)
  int ccw, cch;          // its size
  float hl_soft;
  uint8_t *dbg_gauss;    // debug: demosaic/gauss decisions per entry (x-trans), or null
  // crop/main.comp between demosaic and colour: its committed block (homography
  // as three padded columns, rotation r0..r3, window x X y Y) and output
  float crop[20];
  int cw, ch;            // crop output size
  half4 *cr;             // crop output, cw*ch
};
// stage: 0 noop, 1 hilite half, 2 hilite doub, 3 gauss, 4 splat, 5 fix, 6 halfsize, 7 resample,
// 8 bayer noop + hilite half + level 0 hilite assemble + hilite doub from the mosaic (dn written when set),
// 9 crop of the demosaic output (dm, ow x oh) into cr
cudaError_t launch_nodes(const dev_nodes_t &p, int stage, cudaStream_t s);
// colour -> histogram -> filmcurv -> llap curve -> llap level 1 reduce on the
// demosaic output (p.W x p.H = the output size; p.mosaic unused); with dm null,
// llap curve -> level 1 reduce on the filmcurv output p.rgbf
// dm: the demosaic output read at rows of dm_pitch texels (a crop by whole texels passes the window's
// first texel and the demosaic output's width)
cudaError_t launch_post(const dev_image_t &p, const half4 *dm, int dm_pitch, cudaStream_t s);

// demosaic RCD (k_rcd.cu): rcd_conv (stage 0) and rcd_fill (stage 1) on the
// bayer hilite output, W x H (even W)
struct dev_rcd_t
{
  const __half *cfa;     // hilite/doub output mosaic, W*H
  int W, H;
  float wb[3];           // white balance of the image (the shader's push.wb)
  __half *vh;            // vertical/horizontal discriminator, W*H
  __half *pq, *lp;       // diagonal discriminator and low pass, (W/2)*H
  half4 *out;            // demosaic output, W*H (with post: only for the debug stage, may be null)
  int post;              // rcd_fill also applies colour, the histogram and filmcurv (writes post->rgbf)
};
// stage 1 with p.post reads the colour/filmcurv constants, rgbf and hist of *post
cudaError_t launch_rcd(const dev_rcd_t &p, const dev_image_t *post, int stage, cudaStream_t s);

// packed raw video unpack (k_unpack.cu)
cudaError_t launch_unpack_mlv(const void *packed, size_t bytes, int bpp, size_t npix, uint16_t *out, cudaStream_t s);

// motioncam raw video decode (k_mcraw.cu)
size_t mcraw_scratch_bytes(int rwd, int ht);
cudaError_t launch_mcraw_decode(const void *bitcnt, const void *refval, const void *data, size_t data_bytes, int rwd,
    int ht, int ox, int oy, int W, int H, void *scratch, uint16_t *out, cudaStream_t s);

// output encode (k_encode.cu): colenc to f16 and/or rgba u8 (M: row major rec2020 to the
// output primaries, null for none); BC1 blocks of an rgba u8 image (rgba 4-byte aligned)
cudaError_t launch_colenc(const void *rgba16, int wd, int ht, const float *M, int trc, void *out16, void *out8, cudaStream_t s);
cudaError_t launch_bc1(const void *rgba, int wd, int ht, void *out, cudaStream_t s);

// rawhist noise statistics (k_rawhist.cu)
struct dev_rawhist_t
{
  const uint16_t *mosaic;
  int wd, ht, pitch;       // mosaic size and row pitch (elements)
  int bw, bh;              // CFA blocks: wd / block, ht / block
  uint32_t filters;
  float black, white;      // collect.comp: black/65536, white/65536 of channel 1
  int bins;                // histogram width (the reference uses 1000)
  unsigned long long *acc; // 3 * rawhist_max_bins() fixed point accumulators (device)
};
cudaError_t launch_rawhist(const dev_rawhist_t &p, double *d_out, cudaStream_t s);
size_t rawhist_scratch_bytes();
int rawhist_max_bins();

// hilite (k_hilite.cu)
cudaError_t launch_hilite_k1(const dev_hilite_k1_t &p, cudaStream_t s);
cudaError_t launch_hilite_reduce(const half4 *in, int iw, int ih, half4 *out, int ow, int oh,
    float white, float desat, const float wb[3], cudaStream_t s);
// the small end of the hilite pyramid in one CTA: reduce levels t..L-1 from
// level t-1 (in, sizes lw[0] x lh[0]) and assemble B[L-2..t], in shared memory;
// writes B[t] (out). lw/lh: sizes of levels t-1 .. L-1 (nr + 1 of them)
constexpr int HL_TAIL_MAX = 16;
struct dev_hilite_tail_t
{
  const half4 *in;
  half4 *out;
  int nr;                       // reduce levels in the tail (>= 2)
  int lw[HL_TAIL_MAX], lh[HL_TAIL_MAX];
  float white, desat, soft, wb[3];
};
size_t hilite_tail_smem_bytes(const int *lw, const int *lh, int nr);
constexpr size_t HL_TAIL_SMEM = 160 * 1024;   // the largest tail taken (dynamic shared memory)
constexpr int HL_TAIL_IN = 2048;               // texels of its input level at most (about one per thread)
cudaError_t launch_hilite_tail(const dev_hilite_tail_t &p, cudaStream_t s);
cudaError_t init_hilite();    // function attributes, once per device (from init_develop)
cudaError_t launch_hilite_assemble(const half4 *fine, int fw, int fh, const half4 *coarse, int cw, int ch,
    half4 *out, float white, float soft, cudaStream_t s);

// develop: hilite doub + demosaic + colour + filmcurv + llap curve + level 1 reduce (k_develop.cu)
// map: the tensor map of develop_tensor_map over p.mosaic (interior tiles stage their window by
// TMA), or null (plain loads). status: as launch_llap_reduce's (may be null with map null)
cudaError_t launch_develop(const dev_image_t &p, const CUtensorMap *map, uint32_t *status, cudaStream_t s);
cudaError_t develop_tensor_map(const void *mosaic, int wd, int ht, int pitch, CUtensorMap *map);
// the driver's cuTensorMapEncodeTiled (null where the driver has none)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
cudaError_t init_develop();   // function attributes, once per device (outside stream capture)

// llap pyramid (k_llap.cu): a level is 11 f16 planes (NUM_GAMMA curves + grey) of w x h texels,
// rows of `pitch` texels (a multiple of 8: 16 byte rows, as TMA copies want them), planes of
// `plane` = pitch * h texels
struct llap_level_t { __half *p; int w, h, pitch; size_t plane; };
// the tensor map k_llap_reduce stages a level through (TMA); map lives in host memory and
// travels as a kernel parameter
cudaError_t llap_reduce_tensor_map(const llap_level_t &in, CUtensorMap *map);
// map null: the kernel stages with 4 byte asynchronous copies. status (device memory, may be
// null only with map null): bit 0 set when a TMA copy did not complete within its bounded wait
cudaError_t launch_llap_reduce(const llap_level_t &in, const llap_level_t &out, const CUtensorMap *map,
    uint32_t *status, cudaStream_t s);
// assemble A[j] (out, at l0's size and pitch) from level l0, the coarse level l1 and A[j+1] (coarse,
// at l1's size and pitch; first: the grey plane of l1 instead)
cudaError_t launch_llap_assemble(const __half *coarse, int first, const llap_level_t &l0, const llap_level_t &l1,
    __half *out, cudaStream_t s);
cudaError_t launch_llap_final(const dev_llap_k3_t &p, cudaStream_t s);
cudaError_t init_llap();      // function attributes, once per device (from init_develop)

// misc (k_misc.cu)
struct scene_layout_t;
cudaError_t launch_scene(const scene_layout_t *d_layout, int wd, int ht, uint16_t *out, cudaStream_t s);
cudaError_t launch_hist_rgba(const half4 *in, int W, int H, uint32_t *hist, cudaStream_t s);
// hist/collect.comp: the rgb waveform of an rgba f16 image into a cleared wo x ho u32 image
cudaError_t launch_waveform(const half4 *in, int W, int H, uint32_t *out, int wo, int ho, cudaStream_t s);
// k_static.cu: the fixed scratch of vkdt_cuda_graph_develop_static (address on the current device)
cudaError_t static_scratch_address(void **ptr);
cudaError_t launch_noop_lut(__half *lut, float black, float white, cudaStream_t s);
