/*
 * CPU oracle for the raw-development hot path of vkdt
 * (denoise -> hilite -> demosaic -> colour -> filmcurv -> llap).
 *
 * TEST INFRASTRUCTURE ONLY. This is a line-by-line restatement of the
 * reference GLSL compute shaders in plain C++, the reference the tests compare
 * the CUDA library against. Only tests/, __graft_entry__.smoke() and the cpu_baseline leg
 * of bench.py may load it. The product library never links it.
 *
 * Every node function cites the shader (path within the vkdt project) it
 * restates. The whole file is templated on the arithmetic type so the same
 * code gives the FP32 build (the timed CPU baseline and the parity reference)
 * and the FP64 build (the error reference). f16 storage is emulated at the
 * exact points where the reference stores an image (every node output).
 *
 * Parity pinning: the reference ships no golden vectors for this path. The
 * restatement is pinned against the reference's own shader sources compiled
 * for the CPU (oracle/glsl, built into oracle/_ref) where that build exists.
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* subset of dt_image_params_t (src/pipe/module.h:72-109) that the path reads */
typedef struct oracle_img_param_t
{
  float    black[4];           /* raw DN */
  float    white[4];           /* raw DN */
  float    whitebalance[4];    /* normalised to green = 1 (i-raw/main.c:214-218) */
  uint32_t filters;            /* 0 rgb, 9 x-trans, else bayer rggb */
  uint32_t crop_aabb[4];       /* x0 y0 x1 y1 */
  float    cam_to_rec2020[9];  /* row major */
  float    noise_a, noise_b;   /* vkdt normalised noise profile */
}
oracle_img_param_t;

/* module parameters in the order of each module's `params` file */
typedef struct oracle_params_t
{
  /* denoise/params */
  float   dn_strength, dn_luma, dn_detail, dn_pad, dn_edges[4];
  int32_t dn_gainmap;
  /* hilite/params */
  float   hl_white, hl_desat, hl_soft;
  /* demosaic/params */
  int32_t dm_colour, dm_method;
  /* colour/params (the parts read by the matrix path) */
  float   co_exposure, co_sat;
  int32_t co_matrix;
  float   co_white[4];
  /* filmcurv/params */
  float   fc_light, fc_contrast, fc_bias;
  int32_t fc_colour;
  float   fc_chroma, fc_rolloff, fc_red, fc_yellow, fc_blue, fc_shadows;
  /* llap/params */
  float   ll_sigma, ll_shadows, ll_hilights, ll_clarity;
  /* pyramid depth override: 0 = automatic as llap/main.c:44-89 */
  int32_t ll_levels;
  /* requested output size of the demosaic module (0 = full size). a smaller
   * size switches to the half-size demosaic + resample (demosaic/main.c:93-111) */
  int32_t out_wd, out_ht;
  /* crop between demosaic and colour (crop/main.comp): 0 off, else its
   * committed uniform block (crop/main.c:276-343: mat3 H as three padded
   * columns, the rotation r0..r3, the window x X y Y) and its output size */
  int32_t cr_on, cr_wd, cr_ht;
  float   cr_block[20];
}
oracle_params_t;

/* optional stage outputs, any pointer may be 0. float arrays, row major. */
typedef struct oracle_stages_t
{
  float    *denoise;   /* denoise module output, W*H, 1 channel (mosaic) */
  float    *hilite;    /* hilite module output, W*H, 1 channel (mosaic) */
  float    *demosaic;  /* demosaic output, ow*oh*4 */
  float    *colour;    /* colour output, ow*oh*4 */
  float    *filmcurv;  /* filmcurv output, ow*oh*4 */
  uint32_t *hist;      /* OpenDRT/hist of the filmcurv input, 257 counts */
  float    *llap;      /* llap output (module output of the path), ow*oh*4 */
  int32_t   out_wd, out_ht; /* written: size of the rgb stages */
  int32_t   llap_levels;    /* written: pyramid depth used */
  int32_t   hilite_levels;  /* written: number of hilite reduce nodes */
  float    *crop;      /* crop output (when cr_on), ow*oh*4 */
}
oracle_stages_t;

/* The discrete decisions of the path, recorded and optionally forced. A test
 * reads the decisions the CUDA path took (vkdt_cuda_graph_debug_decisions),
 * compares them with the oracle's own (recorded here with their margins) and
 * reruns the oracle with the CUDA path's decisions forced, so that every
 * output pixel can be held to the continuous tolerance. Any pointer may be 0.
 * Grids: gauss W/block x H/block, denoise W/block x H/block (the half image). */
typedef struct oracle_decisions_t
{
  /* demosaic/gauss.comp per entry: bit 0 det(Sw) < det(Sb) (gauss.comp:65,117);
   * bits 1-2 the snapped direction 0 (1,0), 1 (0,1), 2 none (gauss.comp:72-73,121-123) */
  uint8_t       *gauss;         /* written: the oracle's own decisions */
  const uint8_t *gauss_force;   /* read: decisions applied in place of its own */
  float         *gauss_margin;  /* written, 2 per entry: |detw-detb|/max(|detw|,|detb|), the snap gap */
  /* denoise/cov.glsl response() per half texel: bits 0-24 hot pixel skip of tap
   * (i+2)+5(j+2) (cov.glsl:130), bit 25 det(Sw) < det(Sb) (cov.glsl:84) */
  uint32_t       *dn_cov;
  const uint32_t *dn_cov_force;
  float          *dn_cov_margin; /* 2 per texel: the det gap, min over taps of |r - 2 mean| / (2 mean) */
  /* denoise/assemble.comp per half texel: bit l where |d_l| > 10 (assemble.comp:144-153) */
  uint8_t       *dn_thr;
  const uint8_t *dn_thr_force;
  float         *dn_thr_margin;  /* 4 per texel: | |d_l| - 10 | / 10 */
}
oracle_decisions_t;

/* demosaic/gauss.comp's decisions (and margins, 2 per entry) on a given mosaic
 * (W x H floats, the hilite output): the grid of oracle_decisions_t.gauss */
void oracle_gauss_decisions(const float *mosaic, int wd, int ht, uint32_t filters, uint8_t *dec, float *margin);

/* the seeded synthetic mosaic of the benchmarks (the recipe the library generates
 * on the device; wd x ht u16 raw DN values) */
void oracle_scene(int wd, int ht, uint32_t seed, uint32_t image_id, uint32_t filters, float black, float white,
    float noise_a, float noise_b, const float wb[3], float pan_x, float pan_y, uint16_t *out);

/* crop/main.c's commit_params and modify_roi_out restated: the committed block
 * (20 floats) and the output size for an input of wd x ht, the params
 * perspect[8], crop[4], rotate and the image's exif orientation */
void oracle_crop_commit(int wd, int ht, const float perspect[8], const float crop[4], float rotate,
    uint32_t orientation, float block[20], int *out_wd, int *out_ht);

/* the default parameters of the six modules plus the darkroom .cfg values
 * (bin/default-darkroom.i-raw:28-32) */
void oracle_default_params(oracle_params_t *p);

/* run the whole path on one u16 mosaic. returns 0 on success. */
int oracle_develop_f32(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out);
int oracle_develop_f64(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out);
/* the same with the decisions recorded / forced (dec may be 0). One call at a time. */
int oracle_develop_dec_f32(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec);
int oracle_develop_dec_f64(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec);
/* sensitivity runs: 0 off (round to nearest); else every f16 store of the
 * following develop calls rounds to a neighbouring f16 value chosen by a hash
 * of the value and this seed (at most one f16 step) */
void oracle_set_perturb(uint32_t seed);
/* the wavelet denoise node by node on another implementation's inputs (FP32):
 * in = half, downcov, down 1..3, assemble (W/block x H/block rgba each, levels
 * swizzled as stored); out = half (from the mosaic), downcov of in half, down
 * l of in level l-1, assemble of in half and levels, (W/block x H/block rgba),
 * doub of the mosaic, in assemble and in half (W x H). dec forces decisions. */
int oracle_denoise_nodes(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip,
    const oracle_params_t *p, const float *const in[6], float *const out[7], oracle_decisions_t *dec);
/* FP32, the path from a given stage on: start 1 hilite (input: the denoise output,
 * W*H), 2 demosaic (input: the hilite output, W*H), 3 crop (input: the demosaic
 * output, rgba; without crop the same as 4), 4 colour (input: the output of
 * the stage before colour, rgba), 5 filmcurv (input: the colour output), 6 llap
 * (input: the filmcurv output); the stages before it are replaced by the input
 * (node-wise checks of another implementation's stages on its own inputs) */
int oracle_develop_from_f32(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip,
    const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec, int start, const float *input);

/* single-node entry points for unit tests */
/* denoise/noop.comp on the whole mosaic -> W*H normalised f16 values */
void oracle_noop(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip, float *out);
/* OpenDRT/hist.comp over an rgba image (float values, already f16) */
void oracle_hist(const float *rgba, int wd, int ht, uint32_t *hist257);
/* hist/collect.comp: the rgb waveform of an rgba image (float values, already f16) into wo x ho u32 */
void oracle_waveform(const float *rgba, int wd, int ht, int wo, int ho, uint32_t *out);
/* the bin index the histogram assigns to a luminance (bit exact with the kernel) */
uint32_t oracle_hist_bin(float r, float g, float b);
/* rawhist/collect.comp statistics: out = counts, sums of means, sums of second moments (3*bins) */
void oracle_rawhist(const uint16_t *mosaic, int wd, int ht, uint32_t filters, float black_dn,
    float white_dn, int bins, double *out);
/* demosaic/rcd_conv.comp + rcd_fill.comp on an f16 bayer mosaic (W*H floats, even W):
 * out = W*H*4 rgba */
void oracle_rcd(const float *cfa, int wd, int ht, const float wb[3], float *out);
/* i-mlv/video_mlv.c:254-274: unpack an uncompressed magic lantern raw frame of
 * bpp bits per pixel (10, 12, 14, 16) into npix u16 values; and its inverse */
void oracle_unpack_mlv(const uint8_t *packed, size_t bytes, int bpp, size_t npix, uint16_t *out);
void oracle_pack_mlv(const uint16_t *in, size_t npix, int bpp, uint8_t *packed, size_t bytes);
/* i-mcraw/prefix.comp + decode.comp: a motioncam frame of rwd x ht samples in
 * blocks of 64 (bit count nibbles, reference values, block data) into the
 * wd_out x ht_out u16 mosaic offset by (ox, oy); and a test encoder (returns the
 * data bytes, 0 if cap is too small; force_cnt >= 0 raises every count to it) */
void oracle_mcraw_decode(const uint8_t *bitcnt, const uint16_t *refval, const uint8_t *data, size_t data_bytes,
    int rwd, int ht, int ox, int oy, int wd_out, int ht_out, uint16_t *out);
size_t oracle_mcraw_encode(const uint16_t *img, int rwd, int ht, int force_cnt,
    uint8_t *bitcnt, uint16_t *refval, uint8_t *data, size_t cap);
/* colenc/main.comp: rec2020 rgba (floats) to the output primaries and transfer curve, FP32 out */
void oracle_colenc(const float *rgba, int wd, int ht, int prim, int trc, float *out);
/* lens/main.comp: a wd x ht rgba image (floats, as stored) resampled to owd x oht through the
 * double sphere model; par = centre (2), scale (2), squish0, squish1, ca red, ca blue; out f16-rounded */
void oracle_lens(const float *rgba, int wd, int ht, int owd, int oht, const float *par, float *out);
// grade/main.comp: rgba (float) in, rgba out; par = lift, gamma, gain, offset (4 floats each)
void oracle_grade(const float *rgba, int wd, int ht, const float *par, int mode, float sh_pivot, float hi_pivot,
                  float *out);
/* o-bc1/main.c:21-47 with its stb_dxt encoder restated: the BC1 blocks (8 bytes each) of
 * the whole 4x4 blocks of an rgba u8 image, row major */
void oracle_bc1_encode(const uint8_t *rgba, int wd, int ht, uint8_t *out);
/* CFA colour index at a pixel: 0 red, 1 green, 2 blue (demosaic/splat.comp:167-222) */
int oracle_cfa_colour(uint32_t filters, int x, int y);
/* round to IEEE half (RTNE) and back */
float oracle_f16(float v);

#ifdef __cplusplus
}
#endif
