// libvkdt_cuda host side: the module layer of the path (parameters, .cfg
// reading, the node lists each module's create_nodes emits, commit_params),
// device memory, the launch sequence, staging copies and the C-ABI of
// include/vkdt_cuda.h.
#include "vkdt_cuda.h"
#include "internal.h"
#include "kernels.h"
#include "lens.h"
#include "scene.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

namespace {

thread_local char g_err[512] = "";
int g_device = -1;

// the address of the static develop scratch per device (vkdt_cuda_graph_develop_static),
// looked up once per device; forgotten at vkdt_cuda_cleanup, after which a reloaded
// module may place the array elsewhere
std::mutex g_static_lock;
void *g_static_base[64] = { nullptr };
void forget_static_scratch()
{
  std::lock_guard<std::mutex> guard(g_static_lock);
  for(auto &p : g_static_base) p = nullptr;
}

// a word of mapped pinned host memory per device in which kernels record a bounded wait that
// ran out (bit 0: a TMA copy did not complete); the host reads it after a run without a device call
uint32_t *g_status_host[64] = { nullptr };
uint32_t *g_status_dev[64] = { nullptr };
uint32_t *device_status()
{
  int d = -1;
  if(cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64) return nullptr;
  return g_status_dev[d];
}
// the recorded status of the current device, cleared
uint32_t take_device_status()
{
  int d = -1;
  if(cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64 || !g_status_host[d]) return 0;
  volatile uint32_t *h = g_status_host[d];
  const uint32_t v = *h;
  if(v) *h = 0;
  return v;
}

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_code(cudaError_t e)
{
  if(e == cudaErrorMemoryAllocation) return VKDT_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  if(e == cudaErrorInvalidValue || e == cudaErrorInvalidConfiguration) return VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED;
  return VKDT_CUDA_ERROR_DEVICE_LOST;
}
#define CU(x) do { cudaError_t e_ = (x); if(e_ != cudaSuccess) return fail(cuda_code(e_), "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); } while(0)

dt_token_t tkn(const char *s)
{ // src/pipe/token.h dt_token: up to 8 chars, little endian packed
  uint64_t t = 0;
  for(int i = 0; i < 8 && s[i]; i++) t |= ((uint64_t)(uint8_t)s[i]) << (8 * i);
  return t;
}
std::string tstr(dt_token_t t)
{
  char c[9] = {0};
  memcpy(c, &t, 8);
  return std::string(c);
}

// ------------------------------------------------------------------ module parameter tables
// name:type:count:defaults of each module's `params` file
struct param_def_t { const char *name; char type; int cnt; std::vector<float> def; };
struct module_def_t { const char *name; std::vector<param_def_t> params; };

const std::vector<module_def_t> &module_defs()
{
  static const std::vector<module_def_t> defs = {
    { "i-raw", {                                                  // i-raw/params
      { "noise a", 'f', 1, { 0.0f } }, { "noise b", 'f', 1, { 0.0f } }, { "startid", 'i', 1, { 0 } } } },
    { "denoise", {                                                // denoise/params:1-6
      { "strength", 'f', 1, { 0.0f } }, { "luma", 'f', 1, { 0.6f } }, { "detail", 'f', 1, { 1.0f } },
      { "pad", 'f', 1, { 0.0f } }, { "edges", 'f', 4, { 0, 0, 0, 0 } }, { "gainmap", 'i', 1, { 1 } } } },
    { "hilite", {                                                 // hilite/params:1-3
      { "white", 'f', 1, { 0.985f } }, { "desat", 'f', 1, { 0.3f } }, { "soft", 'f', 1, { 0.6f } } } },
    { "demosaic", {                                               // demosaic/params:1-2
      { "colour", 'i', 1, { 0 } }, { "method", 'i', 1, { 0 } } } },
    { "colour", {                                                 // colour/params:1-13 (rbmap/import omitted)
      { "exposure", 'f', 1, { 0.0f } }, { "sat", 'f', 1, { 1.0f } }, { "picked", 'i', 1, { 0 } },
      { "matrix", 'i', 1, { 1 } }, { "gamut", 'i', 1, { 0 } }, { "clip", 'i', 1, { 0 } },
      { "clipmax", 'f', 1, { 1.0f } }, { "temp", 'f', 1, { 6504.0f } }, { "white", 'f', 4, { 0, 0, 0, 0 } },
      { "mat", 'f', 9, { -1, -1, -1, -1, -1, -1, -1, -1, -1 } }, { "mode", 'i', 1, { 0 } }, { "cnt", 'i', 1, { 4 } } } },
    { "filmcurv", {                                               // filmcurv/params:1-10
      { "light", 'f', 1, { 3.0f } }, { "contrast", 'f', 1, { 1.2f } }, { "bias", 'f', 1, { 0.0f } },
      { "colour", 'i', 1, { 3 } }, { "chroma", 'f', 1, { 1.0f } }, { "rolloff", 'f', 1, { 0.0f } },
      { "red", 'f', 1, { 0.0f } }, { "yellow", 'f', 1, { 0.0f } }, { "blue", 'f', 1, { 0.0f } },
      { "shadows", 'f', 1, { 0.0f } } } },
    { "llap", {                                                   // llap/params:1-4
      { "sigma", 'f', 1, { 0.12f } }, { "shadows", 'f', 1, { 1.0f } }, { "hilights", 'f', 1, { 1.0f } },
      { "clarity", 'f', 1, { 0.0f } } } },
    { "grade", {                                                  // grade/params:1-7
      { "lift", 'f', 4, { 0, 0, 0, 0 } }, { "gamma", 'f', 4, { 1, 1, 1, 0 } }, { "gain", 'f', 4, { 1, 1, 1, 0 } },
      { "offset", 'f', 4, { 0, 0, 0, 0 } }, { "mode", 'i', 1, { 0 } }, { "sh_pivot", 'f', 1, { 0.3f } },
      { "hi_pivot", 'f', 1, { 0.4f } } } },
    { "crop", {                                                   // crop/params:1-3
      { "perspect", 'f', 8, { 0.25f, 0.25f, 0.75f, 0.25f, 0.75f, 0.75f, 0.25f, 0.75f } },
      { "crop", 'f', 4, { 1, 3, 3, 7 } }, { "rotate", 'f', 1, { 1337 } } } },
  };
  return defs;
}

const module_def_t *find_def(dt_token_t name)
{
  for(auto &d : module_defs()) if(tkn(d.name) == name) return &d;
  return nullptr;
}

struct module_t
{
  dt_token_t name = 0, inst = 0;
  const module_def_t *def = nullptr;
  std::vector<uint32_t> param; // 4 bytes per value, params file order
  int offset(dt_token_t p, int *cnt, char *type) const
  {
    int off = 0;
    for(auto &pd : def->params)
    {
      if(tkn(pd.name) == p) { if(cnt) *cnt = pd.cnt; if(type) *type = pd.type; return off; }
      off += pd.cnt;
    }
    return -1;
  }
  float f(const char *p, int i = 0) const { int o = offset(tkn(p), 0, 0); float v; memcpy(&v, &param[o + i], 4); return v; }
  int   n(const char *p, int i = 0) const { int o = offset(tkn(p), 0, 0); int32_t v; memcpy(&v, &param[o + i], 4); return v; }
  void  setf(const char *p, int i, float v) { int o = offset(tkn(p), 0, 0); memcpy(&param[o + i], &v, 4); }
  void init(const module_def_t *d, dt_token_t nm, dt_token_t in)
  {
    def = d; name = nm; inst = in;
    param.clear();
    for(auto &pd : d->params) for(int i = 0; i < pd.cnt; i++)
    {
      const float dv = pd.def[std::min<int>(i, (int)pd.def.size() - 1)];
      uint32_t u;
      if(pd.type == 'i') { int32_t iv = (int32_t)dv; memcpy(&u, &iv, 4); }
      else memcpy(&u, &dv, 4);
      param.push_back(u);
    }
  }
};

// ------------------------------------------------------------------ device buffers
struct level_t { int w = 0, h = 0, pitch = 0; size_t off = 0; };   // pitch: texels per row (llap: 16 byte rows)

} // namespace

struct vkdt_cuda_graph_t
{
  std::vector<module_t> modules;
  std::vector<dt_token_t> unsupported;
  std::vector<std::pair<std::string, std::string>> connects; // "mod:inst:conn" pairs
  // input
  int in_wd = 0, in_ht = 0;
  vkdt_cuda_img_param_t ip;
  bool have_input = false;
  int req_wd = 0, req_ht = 0;
  int llap_levels_req = 0;
  bool timing = false, want_hist = false, debug = false, use_graph = true;
  // derived by alloc
  bool allocated = false, nodes_ready = false;
  int W = 0, H = 0, out_w = 0, out_h = 0;
  int hw = 0, hh = 0;
  std::vector<level_t> hr, hb;   // hilite reduce outputs r[1..L] (index 0 = r1), assembled B[1..L-1]
  int hl_tail = 0;               // first hr index the one-CTA tail kernel computes (hr.size(): none)
  std::vector<level_t> lp, la;   // llap planes level 1..nl-1 (index 0 = level 1), assembled A[1..nl-2]
  int nl = 0;
  size_t off_src = 0, off_rgbf = 0, off_out = 0, off_hist = 0, off_dbg0 = 0, off_dbg1 = 0, off_lut = 0, arena_bytes = 0;
  bool wavelet = false;          // denoise strength > 0: the wavelet nodes run before hilite
  bool doub_fixed = false;       // bayer: denoise/doub's bilinear taps at fixed places in every row and column
  int block = 2;                 // CFA block: 2 bayer, 3 x-trans
  bool halfsize = false, resample = false;  // demosaic/halfsize (+ shared/resample) for reduced sizes
  bool rcd = false;              // demosaic method 1 (rcd_conv + rcd_fill) at full size
  bool grade = false;            // llap -> grade connected: grade/main applied to the llap output
  bool crop = false;             // demosaic -> crop -> colour connected
  bool crop_stage = false;       // the crop moves or resamples pixels (not the identity): its own launch
  bool crop_given = false;       // its committed block came with the scheduler's nodes (set_nodes)
  bool crop_shift = false;       // the crop moves the image by whole texels: the next launch reads the window
  int crop_dx = 0, crop_dy = 0;  // that shift
  float crop_blk[20];            // crop's committed uniform block (crop/main.c:276-343)
  int crop_w = 0, crop_h = 0;    // its output size
  int dm_w = 0, dm_h = 0;        // the demosaic output size (crop's input; out_w x out_h without crop)
  bool unfused = false;          // x-trans, rcd or reduced size: the per-node chain instead of the fused kernel
  bool k1front = false;          // bayer per-node chain: the fused path's hilite front (k1, pyramid, one kernel to doub)
  std::vector<int64_t> planned_for; // what alloc planned for: a run refuses a graph changed since
  std::vector<int64_t> nodes_for;   // what create_nodes planned for (the static develop checks it)
  float lut_black = -1.0f, lut_white = -1.0f;  // black/white (unorm) the noop code table holds
  // black and white as the denoise node's push constants carry them (DN / 65535, denoise/main.c:165-168)
  float nblack[4] = { 0, 0, 0, 0 }, nwhite[4] = { 1, 1, 1, 1 };
  // colour's committed uniform block when the scheduler hands it over (vkdt_cuda_graph_set_nodes):
  // the white balance multipliers, the exposure factor and the camera matrix as committed
  bool colour_given = false;
  float colour_mul[3] = { 1, 1, 1 }, colour_mulw = 1.0f, colour_cam[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 };
  size_t off_h0 = 0, off_b0 = 0, off_hl = 0, off_cov = 0, off_g = 0, off_hs = 0, off_dm = 0, off_cr = 0;
  size_t off_vh = 0, off_pq = 0, off_lpf = 0;
  size_t off_dnh = 0, off_dnl[4] = { 0, 0, 0, 0 }, off_dna = 0, off_dn = 0, off_idlut = 0;
  // debug stages: demosaic (fused path) and colour outputs, the decisions of gauss and the wavelet denoise
  size_t off_dbg_dm = 0, off_dbg_col = 0, off_dbg_gauss = 0, off_dbg_cov = 0, off_dbg_thr = 0;
  unsigned char *arena = nullptr;
  void *h_src = nullptr, *h_sink = nullptr;
  size_t src_bytes = 0, sink_bytes = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  // tensor maps made for the arena tm_arena: k_llap_reduce's (input level l-1 of reduce launch l)
  // and k_develop's over the source mosaic and over the denoised mosaic
  std::vector<CUtensorMap> tm_reduce;
  CUtensorMap tm_src, tm_dn;
  bool tm_src_ok = false, tm_dn_ok = false;
  unsigned char *tm_arena = nullptr;
  std::vector<vkdt_cuda_node_info_t> nodes;
  // launch list (fused kernels) and timing
  struct launch_t { dt_token_t name, kernel; };
  std::vector<launch_t> launches;
  std::vector<cudaEvent_t> ev;
  std::vector<float> times;
  cudaGraphExec_t gexec = nullptr;
  bool graph_dirty = true;
  const void *gsrc = nullptr;     // the buffers the captured launch sequence reads and writes
  void *gdst = nullptr;
  const void *ext_src = nullptr;  // device buffers bound for the current run
  void *ext_dst = nullptr;

  module_t *mod(const char *name)
  {
    for(auto &m : modules) if(m.name == tkn(name)) return &m;
    return nullptr;
  }
  template<class T> T *at(size_t off) { return reinterpret_cast<T *>(arena + off); }
};

namespace {

module_t *ensure_module(vkdt_cuda_graph_t *g, const char *name)
{
  module_t *m = g->mod(name);
  if(m) return m;
  module_t nm;
  nm.init(find_def(tkn(name)), tkn(name), tkn("01"));
  g->modules.push_back(nm);
  return &g->modules.back();
}

void default_modules(vkdt_cuda_graph_t *g)
{
  const char *path[] = { "i-raw", "denoise", "hilite", "demosaic", "colour", "filmcurv", "llap" };
  for(const char *p : path) ensure_module(g, p);
  // the darkroom graph's llap values (bin/default-darkroom.i-raw:29-32)
  g->mod("llap")->setf("clarity", 0, 0.2f);
}

void add_node(vkdt_cuda_graph_t *g, const char *name, const char *kernel, int wd, int ht, int dp, int fused)
{
  vkdt_cuda_node_info_t n;
  n.name = tkn(name); n.kernel = tkn(kernel);
  n.wd = wd; n.ht = ht; n.dp = dp; n.fused = fused;
  g->nodes.push_back(n);
}

// 3x3 helpers in float with the same summation order as the shader constant folding
void m3_mul(const double *A, const double *B, float *r)
{
  float a[9], b[9];
  for(int i = 0; i < 9; i++) { a[i] = (float)A[i]; b[i] = (float)B[i]; }
  for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)
  {
    volatile float s = a[3 * i + 0] * b[0 + j];
    s = s + a[3 * i + 1] * b[3 + j];
    s = s + a[3 * i + 2] * b[6 + j];
    r[3 * i + j] = s;
  }
}
void m3_apply(const float *A, const float *v, float *o)
{
  for(int i = 0; i < 3; i++)
  {
    volatile float s = A[3 * i + 0] * v[0];
    s = s + A[3 * i + 1] * v[1];
    s = s + A[3 * i + 2] * v[2];
    o[i] = s;
  }
}

// colour matrices (src/pipe/modules/matrices.h, row major)
const double M_cat16_Mi[9] = { 1.86206786, -1.01125463,  0.14918677, 0.38752654,  0.62144744, -0.00897398, -0.01584150, -0.03412294,  1.04996444 };
const double M_cat16_M[9]  = { 0.401288, 0.650173, -0.051461, -0.250268, 1.204414,  0.045854, -0.002079, 0.048952,  0.953127 };
const double M_rec2020_to_xyz[9] = { 0.636958048301290991, 0.144616903586208406, 0.168880975164172054, 0.26270021201126692, 0.677998071518871148, 0.0593017164698619384, 4.9999999999999999e-17, 0.0280726930490874452, 1.06098505771079066 };
const double M_xyz_to_rec2020[9] = { 1.71665119, -0.35567078, -0.25336628, -0.66668435,  1.61648124,  0.01576855, 0.01763986, -0.04277061, 0.94210312 };
const double M_rec709_to_rec2020[9] = { 0.62750375, 0.32927542, 0.04330266, 0.06910828, 0.91951916, 0.0113596, 0.01639406, 0.08801125, 0.89538035 };
const double M_rec2020_to_rec709[9] = { 1.66022677, -0.58754761, -0.07283825, -0.12455334,  1.13292605, -0.00834963, -0.01815514, -0.10060303,  1.11899817 };
const double M_rec709_to_yuv[9] = { 0.299, 0.587, 0.114, -0.147, -0.289, 0.436, 0.615, -0.515, -0.100 };
const double M_yuv_to_rec709[9] = { 1.0, -3.94570707e-05, 1.13982797, 1.0, -3.94610164e-01, -5.80500316e-01, 1.0, 2.03199968, -4.81376263e-04 };

// colour/main.c:219-292 commit_params (matrix path): writes p_wb back into the
// module's params when it was derived from the camera coefficients
// the white balance part of colour's commit_params (colour/main.c:241-253): the
// white derived from the camera coefficients when the param is zero, written back
// into the params as the reference does
void colour_commit_white(vkdt_cuda_graph_t *g, float p_wb[3])
{
  module_t *m = g->mod("colour");
  p_wb[0] = m->f("white", 0); p_wb[1] = m->f("white", 1); p_wb[2] = m->f("white", 2);
  if(g->colour_given)
  { // the block the reference's commit_params wrote (vkdt_cuda_graph_set_nodes)
    p_wb[0] = g->colour_mul[0]; p_wb[1] = 1.0f; p_wb[2] = g->colour_mul[2];
  }
  if(p_wb[0] == 0.0f && p_wb[1] == 0.0f && p_wb[2] == 0.0f)
  {
    float w0[3] = {0}, w[] = { g->ip.whitebalance[0], g->ip.whitebalance[1], g->ip.whitebalance[2] };
    for(int j = 0; j < 3; j++) for(int i = 0; i < 3; i++) w0[j] += g->ip.cam_to_rec2020[3 * j + i] / w[i];
    w0[0] /= w0[1]; w0[2] /= w0[1]; w0[1] = 1.0f;
    p_wb[0] = 1 / w0[0]; p_wb[1] = 1; p_wb[2] = 1 / w0[2];
  }
  if(!(p_wb[0] == p_wb[0]) || p_wb[0] == 0.0f || p_wb[1] == 0.0f || p_wb[2] == 0.0f)
    p_wb[0] = p_wb[1] = p_wb[2] = 1.0f;
  if(!g->colour_given) for(int k = 0; k < 3; k++) m->setf("white", k, p_wb[k]);
}

void colour_commit(vkdt_cuda_graph_t *g, dev_image_t &d)
{
  module_t *m = g->mod("colour");
  float p_wb[3];
  colour_commit_white(g, p_wb);
  const float mul[3] = { p_wb[0] / p_wb[1], 1.0f, p_wb[2] / p_wb[1] };
  d.mulw = g->colour_given ? g->colour_mulw : powf(2.0f, m->f("exposure"));
  if(g->colour_given) for(int i = 0; i < 9; i++) d.cam[i] = g->colour_cam[i];
  else if(m->n("matrix") == 1) for(int i = 0; i < 9; i++) d.cam[i] = g->ip.cam_to_rec2020[i];
  else for(int i = 0; i < 9; i++) d.cam[i] = (i % 4 == 0) ? 1.0f : 0.0f;
  m3_mul(M_cat16_M, M_rec2020_to_xyz, d.P);
  m3_mul(M_xyz_to_rec2020, M_cat16_Mi, d.Q);
  const float one[3] = { 1, 1, 1 };
  float src[3], dst[3];
  m3_apply(d.P, one, src);
  m3_apply(d.P, mul, dst);
  for(int k = 0; k < 3; k++) d.clscale[k] = dst[k] / src[k];
  // the chain as one matrix: the kernels apply it per pixel (continuous values
  // before an f16 store; a few f32 ulp from the three products in sequence)
  double a[9], b[9];
  for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)
  {
    double s = 0.0;
    for(int k = 0; k < 3; k++) s += (double)d.P[3 * i + k] * d.cam[3 * k + j];
    a[3 * i + j] = s * d.clscale[i];
  }
  for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)
  {
    double s = 0.0;
    for(int k = 0; k < 3; k++) s += (double)d.Q[3 * i + k] * a[3 * k + j];
    b[3 * i + j] = s * d.mulw;
  }
  for(int i = 0; i < 9; i++) d.cmat[i] = (float)b[i];
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// ------------------------------------------------------------------ crop (crop/main.c)

// the linear system of crop's perspective quad (core/gaussian_elimination.h:40-109, after H.
// Spaeth, "Numerik", 1994): elimination with partial pivoting as LINPACK's dgefa/dgesl order it.
// The operations follow the reference's order so that the homography it commits comes out to the
// same bits: the first row of largest magnitude pivots; pivot rows swap right of the pivot column
// only; the negated multipliers stay where they are formed; the right hand side is permuted as
// it is reduced.
bool solve_linpack(double *A, double *b, int n)
{
  std::vector<int> piv(n);
  for(int k = 0; k < n; k++)
  {
    double *rk = A + (size_t)k * n;
    int m = k;
    for(int r = k + 1; r < n; r++) if(std::fabs(A[(size_t)r * n + k]) > std::fabs(A[(size_t)m * n + k])) m = r;
    piv[k] = m;
    double *rm = A + (size_t)m * n;
    const double pv = rm[k];
    rm[k] = rk[k];
    rk[k] = pv;
    if(pv == 0.0) return false;
    for(int r = k + 1; r < n; r++) A[(size_t)r * n + k] /= -pv;
    if(m != k) for(int c = k + 1; c < n; c++) std::swap(rm[c], rk[c]);
    for(int r = k + 1; r < n; r++)
    {
      double *rr = A + (size_t)r * n;
      for(int c = k + 1; c < n; c++) rr[c] += rr[k] * rk[c];
    }
  }
  for(int k = 0; k < n - 1; k++)
  {
    std::swap(b[piv[k]], b[k]);
    for(int r = k + 1; r < n; r++) b[r] += A[(size_t)r * n + k] * b[k];
  }
  for(int k = n - 1; k >= 0; k--)
  {
    b[k] /= A[(size_t)k * n + k];
    for(int r = 0; r < k; r++) b[r] -= A[(size_t)r * n + k] * b[k];
  }
  return true;
}

// crop/main.c:175-226 get_crop_rot: rotation 1337 follows the exif orientation (3: 180, 8: 90,
// 6: 270 degrees, else none); the window 1,3,3,7 is a 3 px safety margin for resampling (none at
// 400 px or less), its axes exchanged for the quarter turns
void crop_window(uint32_t orient, double wd, double ht, const module_t *m, float win[4], float *rot)
{
  const float prot = m->f("rotate");
  *rot = prot;
  for(int k = 0; k < 4; k++) win[k] = m->f("crop", k);
  if(prot == 1337.0f) *rot = orient == 3 ? 180.0f : orient == 8 ? 90.0f : orient == 6 ? 270.0f : 0.0f;
  if(!(win[0] == 1.0f && win[1] == 3.0f && win[2] == 3.0f && win[3] == 7.0f)) return;
  const double mw = wd > 400 ? 3.0 / wd : 0.0, mh = ht > 400 ? 3.0 / ht : 0.0;
  const float r = *rot;
  if((r >= 45 && r < 135) || (r >= 225 && r < 315))
  {
    win[0] = 0.5 - (.5 - mh) * ht / wd; win[1] = 0.5 + (.5 - mh) * ht / wd;
    win[2] = 0.5 - (.5 - mw) * wd / ht; win[3] = 0.5 + (.5 - mw) * wd / ht;
  }
  else { win[0] = mw; win[1] = 1.0 - mw; win[2] = mh; win[3] = 1.0 - mh; }
}

// crop's output size (crop/main.c:252-275 modify_roi_out: the window's share of the input, at
// most 32768) and its committed block (:276-343 commit_params: the homography of the perspective
// quad as three padded columns, the rotation matrix, the window), for a wd x ht input. With
// automatic rotation the resolved window and rotation are written back into the params, as the
// reference does.
void crop_commit(vkdt_cuda_graph_t *g, int wd, int ht, float blk[20], int *ow, int *oh)
{
  module_t *m = g->mod("crop");
  float win[4], rot;
  crop_window(g->ip.orientation, (float)wd, (float)ht, m, win, &rot);
  const float sw = win[1] - win[0], sh = win[3] - win[2];
  *ow = (int)(uint32_t)std::fmin(32768.0f, (float)(uint32_t)wd * sw);
  *oh = (int)(uint32_t)std::fmin(32768.0f, (float)(uint32_t)ht * sh);
  // the homography taking the axis aligned quad (a,b) (A,b) (A,B) (a,B) to the given corners
  // (P. Heckbert, "Fundamentals of Texture Mapping and Image Warping", 1989, pp. 17-21)
  float c[8];
  for(int k = 0; k < 4; k++) { c[2 * k] = (float)(uint32_t)wd * m->f("perspect", 2 * k); c[2 * k + 1] = (float)(uint32_t)ht * m->f("perspect", 2 * k + 1); }
  const float ax = c[0], bx = c[2], ay = c[1], by = c[7];
  const float q[8] = { ax, ay, bx, ay, bx, by, ax, by };
  double A[64] = { 0 }, x[9];
  for(int k = 0; k < 4; k++)
  {
    const float qx = q[2 * k], qy = q[2 * k + 1];
    double *ex = A + 8 * k, *ey = A + 8 * (4 + k);
    ex[0] = qx; ex[1] = qy; ex[2] = 1; ex[6] = -c[2 * k] * qx; ex[7] = -c[2 * k] * qy;   // float products
    ey[3] = qx; ey[4] = qy; ey[5] = 1; ey[6] = -c[2 * k + 1] * qx; ey[7] = -c[2 * k + 1] * qy;
    x[k] = c[2 * k]; x[4 + k] = c[2 * k + 1];
  }
  x[8] = 1.0;
  solve_linpack(A, x, 8);
  for(int col = 0; col < 3; col++)
  {
    for(int row = 0; row < 3; row++) blk[4 * col + row] = (float)x[3 * row + col];
    blk[4 * col + 3] = 0.0f;
  }
  const float rad = rot * 3.1415629 / 180.0f;
  blk[12] = cosf(rad); blk[13] = sinf(rad); blk[14] = -sinf(rad); blk[15] = cosf(rad);
  for(int k = 0; k < 4; k++) blk[16 + k] = win[k];
  if(m->f("rotate") == 1337.0f)
  {
    for(int k = 0; k < 4; k++) m->setf("crop", k, win[k]);
    m->setf("rotate", 0, rot);
  }
}

// the position crop/main.comp samples for output pixel (x, y) on a dw x dh input, normalised,
// with the operations and rounding of k_nd_crop (IEEE single precision, nothing contracted)
void crop_src(const float b[20], int dw, int dh, int x, int y, float &rx, float &ry)
{
  const float tsx = (float)dw, tsy = (float)dh;
  const float px = ((float)x + 0.5f) + b[16] * tsx, py = ((float)y + 0.5f) + b[18] * tsy;
  const float vx = px - tsx * 0.5f, vy = py - tsy * 0.5f;
  const float qx = (b[12] * vx + b[14] * vy) + tsx * 0.5f, qy = (b[13] * vx + b[15] * vy) + tsy * 0.5f;
  const float hx = (b[0] * qx + b[4] * qy) + b[8], hy = (b[1] * qx + b[5] * qy) + b[9];
  const float hz = (b[2] * qx + b[6] * qy) + b[10];
  rx = hx / hz / tsx; ry = hy / hz / tsy;
}

// a crop that fetches input texel (x + dx, y + dy) for every output pixel (x, y), all inside the
// input: no rotation (r0 = 1, so texelFetch), the identity homography, and a window whose every
// row and column lands on the same whole texel offset (checked position by position; with the
// identity and no rotation the cross terms are exact zeros, so x and y are independent)
bool crop_whole_texels(const float b[20], int dw, int dh, int cw, int ch, int *dx, int *dy)
{
  static const float id[16] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 1, 0, 0, 1 };
  for(int k = 0; k < 16; k++) if(b[k] != id[k]) return false;   // -0 == 0
  int sx = 0, sy = 0;
  for(int x = 0; x < cw; x++)
  {
    float rx, ry;
    crop_src(b, dw, dh, x, 0, rx, ry);
    if(!(rx >= 0.0f && rx < 1.0f)) return false;
    const int ix = (int)(rx * (float)dw);
    if(x == 0) sx = ix;
    if(ix != x + sx || ix >= dw) return false;
  }
  for(int y = 0; y < ch; y++)
  {
    float rx, ry;
    crop_src(b, dw, dh, 0, y, rx, ry);
    if(!(ry >= 0.0f && ry < 1.0f)) return false;
    const int iy = (int)(ry * (float)dh);
    if(y == 0) sy = iy;
    if(iy != y + sy || iy >= dh) return false;
  }
  *dx = sx; *dy = sy;
  return true;
}

// a block that copies its input unchanged: the identity homography and rotation, the whole frame
bool crop_identity(const float b[20], int wd, int ht, int ow, int oh)
{
  static const float id[20] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 1, 0, 0, 1, 0, 1, 0, 1 };
  for(int k = 0; k < 20; k++) if(b[k] != id[k]) return false;   // -0 == 0
  return ow == wd && oh == ht;
}

// everything the node plan and the arena depend on
std::vector<int64_t> plan_key(vkdt_cuda_graph_t *g)
{
  const module_t *dn = g->mod("denoise");
  const int wavelet = dn && dn->f("strength") > 0.0f;
  const int fixup = g->mod("demosaic") ? g->mod("demosaic")->n("colour") : 0;
  const int method = g->mod("demosaic") ? g->mod("demosaic")->n("method") : 0;
  std::vector<int64_t> k = { g->in_wd, g->in_ht, g->ip.crop_aabb[0], g->ip.crop_aabb[1], g->ip.crop_aabb[2],
      g->ip.crop_aabb[3], g->ip.filters, g->req_wd, g->req_ht, g->llap_levels_req, wavelet, g->want_hist, g->debug,
      fixup, method, g->crop, g->ip.orientation, g->crop_given };
  if(const module_t *c = g->crop ? g->mod("crop") : nullptr) for(uint32_t v : c->param) k.push_back(v);
  if(g->crop_given) for(float v : g->crop_blk) { uint32_t u; memcpy(&u, &v, 4); k.push_back(u); }
  return k;
}

int check_supported_params(vkdt_cuda_graph_t *g)
{
  if(g->crop)
  { // crop/main.c:228-251: with a scaled output crop's input size follows its output's
    // (modify_roi_in); only full resolution is built
    if(!g->mod("crop")) return fail(VKDT_CUDA_INCOMPLETE, "crop connected but not declared");
    if(g->req_wd > 0 || g->req_ht > 0) return fail(VKDT_CUDA_INCOMPLETE, "crop with a scaled output size is not built");
  }
  const int method = g->mod("demosaic")->n("method");
  if(method < 0 || method > 2) return fail(VKDT_CUDA_INCOMPLETE, "demosaic method %d not supported", method);
  const int fm = g->mod("filmcurv")->n("colour");
  if(fm != 1 && fm != 3) return fail(VKDT_CUDA_INCOMPLETE, "filmcurv colour mode %d not supported", fm);
  if(g->mod("colour")->f("sat") != 1.0f) return fail(VKDT_CUDA_INCOMPLETE, "colour saturation != 1 not supported");
  if(g->mod("colour")->n("clip") != 0 || g->mod("colour")->n("mode") != 0 || g->mod("colour")->n("gamut") != 0)
    return fail(VKDT_CUDA_INCOMPLETE, "colour clip/mode/gamut not supported");
  const int mat = g->mod("colour")->n("matrix");
  if(mat != 0 && mat != 1) return fail(VKDT_CUDA_INCOMPLETE, "colour matrix %d not supported", mat);
  return 0;
}

llap_level_t llap_level(vkdt_cuda_graph_t *g, const level_t &l)
{
  return { g->at<__half>(l.off), l.w, l.h, l.pitch, (size_t)l.pitch * l.h };
}

// fill the per image constants for the kernels (create_nodes push constants + commit_params uniforms)
int fill_image(vkdt_cuda_graph_t *g, dev_image_t &d, const void *d_src, void *d_out)
{
  memset(&d, 0, sizeof(d));
  d.neg_zero = -0.0f;
  d.mosaic = (const uint16_t *)d_src;
  d.noop_lut = g->at<__half>(g->off_lut);
  d.pitch = g->in_wd;
  d.cx = (int)g->ip.crop_aabb[0]; d.cy = (int)g->ip.crop_aabb[1];
  d.W = g->W; d.H = g->H;
  d.filters = g->ip.filters;
  d.black = g->nblack[0];                     // denoise/main.c:165-168
  d.white = g->nwhite[0];
  d.codes.black = d.black; d.codes.white = d.white; d.codes.identity = 0;
  module_t *hl = g->mod("hilite");
  d.hl_white = hl->f("white"); d.hl_desat = hl->f("desat"); d.hl_soft = hl->f("soft");
  for(int k = 0; k < 3; k++) d.wb[k] = g->ip.whitebalance[k];
  if(g->hb.empty()) { d.hl_coarse = g->at<half4>(g->hr[0].off); d.hcw = g->hr[0].w; d.hch = g->hr[0].h; }
  else              { d.hl_coarse = g->at<half4>(g->hb[0].off); d.hcw = g->hb[0].w; d.hch = g->hb[0].h; }
  d.fixup = g->mod("demosaic")->n("colour");
  colour_commit(g, d);
  module_t *fc = g->mod("filmcurv");
  d.fc_il = fmaxf(5e-3f, fc->f("light"));
  d.fc_k = fmaxf(1e-4f, fc->f("contrast"));
  d.fc_bias = fc->f("bias");
  d.fc_mode = fc->n("colour");
  module_t *ll = g->mod("llap");
  d.ll_sigma = ll->f("sigma"); d.ll_shadows = ll->f("shadows"); d.ll_highlights = ll->f("hilights"); d.ll_clarity = ll->f("clarity");
  d.crop_dx = g->crop_shift ? g->crop_dx : 0; d.crop_dy = g->crop_shift ? g->crop_dy : 0;
  d.crop_w = g->crop_shift ? g->out_w : g->W; d.crop_h = g->crop_shift ? g->out_h : g->H;
  d.rgbf = g->at<half4>(g->off_rgbf);
  d.l1 = g->at<__half>(g->lp[0].off);
  d.l1w = g->lp[0].w; d.l1h = g->lp[0].h; d.l1pitch = g->lp[0].pitch;
  d.l1plane = (size_t)g->lp[0].pitch * g->lp[0].h;
  d.hist = g->want_hist ? g->at<uint32_t>(g->off_hist) : nullptr;
  if(g->debug)
  {
    d.dbg_denoise = g->at<__half>(g->off_dbg0); d.dbg_hilite = g->at<__half>(g->off_dbg1);
    d.dbg_demosaic = g->at<half4>(g->off_dbg_dm); d.dbg_colour = g->at<half4>(g->off_dbg_col);
    d.dbg_gauss = g->at<uint8_t>(g->off_dbg_gauss);
  }
  (void)d_out;
  return 0;
}

// the arena plan: offsets of every device buffer of the graph; returns the bytes
size_t plan_arena(vkdt_cuda_graph_t *g)
{
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off = align_up(off + bytes); return o; };
  g->src_bytes = (size_t)g->in_wd * g->in_ht * 2;
  g->sink_bytes = (size_t)g->out_w * g->out_h * 8;
  g->off_src = take(g->src_bytes);
  for(auto &l : g->hr) l.off = take((size_t)l.w * l.h * 8);
  for(auto &l : g->hb) l.off = take((size_t)l.w * l.h * 8);
  g->off_rgbf = take((size_t)g->out_w * g->out_h * 8);
  for(auto &l : g->lp) l.off = take((size_t)l.pitch * l.h * 2 * 11);
  for(auto &l : g->la) l.off = take((size_t)l.pitch * l.h * 2);
  g->off_out = take(g->sink_bytes);
  g->off_hist = take(257 * 4);
  g->off_lut = take(65536 * 2);
  if(g->debug)
  {
    g->off_dbg0 = take((size_t)g->W * g->H * 2); g->off_dbg1 = take((size_t)g->W * g->H * 2);
    g->off_dbg_dm = take((size_t)g->dm_w * g->dm_h * 8); g->off_dbg_col = take((size_t)g->out_w * g->out_h * 8);
    g->off_dbg_gauss = take((size_t)g->hw * g->hh);
    if(g->wavelet) { g->off_dbg_cov = take((size_t)g->hw * g->hh * 4); g->off_dbg_thr = take((size_t)g->hw * g->hh); }
  }
  const size_t hbytes = (size_t)g->hw * g->hh * 8;
  if(g->wavelet)
  { // the half size nodes of the wavelet denoise
    g->off_dnh = take(hbytes);
    for(int i = 0; i < 4; i++) g->off_dnl[i] = take(hbytes);
    g->off_dna = take(hbytes);
  }
  // the (denoised) normalised mosaic: wavelet output, or the noop output of the per-node chain
  if(g->wavelet || g->unfused) g->off_dn = take((size_t)g->W * g->H * 2);
  if(g->wavelet && (!g->unfused || g->k1front)) g->off_idlut = take(65536 * 2);
  if(g->unfused)
  { // the per-node chain's images (intermediate f16 images like the reference's)
    if(!g->k1front)
    {
      g->off_h0 = take(hbytes);
      g->off_b0 = take(hbytes);
    }
    g->off_hl = take((size_t)g->W * g->H * 2);
    if(g->halfsize)
    {
      g->off_hs = take(hbytes);
      g->off_dm = g->resample ? take((size_t)g->dm_w * g->dm_h * 8) : g->off_hs;
    }
    else if(g->rcd)
    { // demosaic/main.c:113-125: vh at full size, pq and lp at half width
      g->off_vh = take((size_t)g->W * g->H * 2);
      g->off_pq = take((size_t)(g->W / 2) * g->H * 2);
      g->off_lpf = take((size_t)(g->W / 2) * g->H * 2);
      g->off_dm = take((size_t)g->W * g->H * 8);
    }
    else
    {
      g->off_cov = take(hbytes);
      g->off_g = take((size_t)g->W * g->H * 2);
      g->off_dm = take((size_t)g->W * g->H * 8);
    }
    if(g->crop_stage && !g->crop_shift) g->off_cr = take((size_t)g->out_w * g->out_h * 8);
  }
  return off;
}

// denoise/doub.comp:35-40 samples the coarse levels by texture() at the
// normalised centre of output position x of n, on a level of size h = n / 2.
// True when, in the kernel's IEEE single operations and the sampler's 8 bit
// sub-texel position, that is texel x/2 - 1 at fraction 0.75 for even x and
// texel x/2 at 0.25 for odd x, for every x (the fixed taps of k_dn_doub_quad).
bool doub_taps_fixed(int n, int h)
{
  if(n != 2 * h) return false;
  for(int x = 0; x < n; x++)
  {
    volatile float u = ((float)x + 0.5f) / (float)n;
    volatile float t = u * (float)h;
    volatile float v = t - 0.5f;
    volatile float s = v * 256.0f;
    volatile float r = s + 0.5f;
    volatile float xs = std::floor(r) * 0.00390625f;
    const float fx = std::floor(xs);
    const float ax = xs - fx;
    const int want = (x & 1) ? x / 2 : x / 2 - 1;
    if((int)fx != want || ax != ((x & 1) ? 0.25f : 0.75f)) return false;
  }
  return true;
}

// the push constants and uniforms of the wavelet denoise nodes (denoise/main.c:133-333)
void fill_denoise(vkdt_cuda_graph_t *g, dev_denoise_t &p, const void *d_src)
{
  memset(&p, 0, sizeof(p));
  p.mosaic = (const uint16_t *)d_src;
  p.pitch = g->in_wd; p.in_w = g->in_wd; p.in_h = g->in_ht;
  p.cx = (int)g->ip.crop_aabb[0]; p.cy = (int)g->ip.crop_aabb[1];
  p.W = g->W; p.H = g->H; p.hw = g->hw; p.hh = g->hh;
  p.filters = g->ip.filters;
  for(int k = 0; k < 3; k++)
  {
    p.black[k] = g->nblack[k];
    p.white[k] = g->nwhite[k];
    p.wb[k] = g->ip.whitebalance[k];
    p.wb_norm[k] = p.wb[k] / (p.white[k] - p.black[k]);
    p.wb_denorm[k] = (p.white[k] - p.black[k]) / p.wb[k];
  }
  p.na = g->ip.noise_a; p.nb = g->ip.noise_b;
  module_t *dn = g->mod("denoise");
  for(int k = 0; k < 3; k++) p.edge_gain[k] = std::exp2(12.0f * dn->f("edges", k) + dn->f("edges", 3));
  p.strength = dn->f("strength"); p.luma = dn->f("luma"); p.detail = dn->f("detail");
  p.thrs0 = std::pow(p.strength, 4.0f);
  p.block_f = g->ip.filters == 9u ? 2.23607f : 1.414213f;   // denoise/main.c:235-238 (block 3 / 2)
  p.doub_fixed = g->doub_fixed;
  p.fuse_half = g->ip.filters != 9u;
  p.neg_zero = -0.0f;
  const float bl[4] = { 0.7000f, 0.4900f, 0.3430f, 0.2401f };
  for(int l = 0; l < 4; l++) p.bscale[l] = bl[l] / p.block_f;
  for(int l = 0; l < 4; l++) p.pl[l] = std::pow(0.7f, (float)l);
  m3_mul(M_rec709_to_yuv, M_rec2020_to_rec709, p.rgb_to_yuv);
  m3_mul(M_rec709_to_rec2020, M_yuv_to_rec709, p.yuv_to_rgb);
  p.half_img = g->at<half4>(g->off_dnh);
  for(int i = 0; i < 4; i++) p.lvl[i] = g->at<half4>(g->off_dnl[i]);
  p.asm_img = g->at<half4>(g->off_dna);
  p.dn = g->at<__half>(g->off_dn);
  if(g->debug) { p.dbg_cov = g->at<uint32_t>(g->off_dbg_cov); p.dbg_thr = g->at<uint8_t>(g->off_dbg_thr); }
}

// buffers and sizes of the per-node chain (x-trans, reduced output sizes)
void fill_nodes(vkdt_cuda_graph_t *g, dev_nodes_t &p, const void *d_src)
{
  memset(&p, 0, sizeof(p));
  p.neg_zero = -0.0f;
  p.mosaic = (const uint16_t *)d_src;
  p.noop_lut = g->at<__half>(g->off_lut);
  p.pitch = g->in_wd; p.cx = (int)g->ip.crop_aabb[0]; p.cy = (int)g->ip.crop_aabb[1];
  p.W = g->W; p.H = g->H;
  p.filters = g->ip.filters;
  p.block = g->block; p.hw = g->hw; p.hh = g->hh;
  p.hl_white = g->mod("hilite")->f("white");
  p.fixup = g->mod("demosaic")->n("colour");
  p.ow = g->dm_w; p.oh = g->dm_h;
  p.dn = g->at<__half>(g->off_dn);
  p.h0 = g->at<half4>(g->off_h0);
  p.b0 = g->at<half4>(g->off_b0);
  p.hl = g->at<__half>(g->off_hl);
  p.cov = g->at<half4>(g->off_cov);
  p.g = g->at<__half>(g->off_g);
  p.hs = g->at<half4>(g->off_hs);
  p.dm = g->at<half4>(g->off_dm);
  const level_t &c = g->hb.empty() ? g->hr[0] : g->hb[0];
  p.coarse = g->at<half4>(c.off); p.ccw = c.w; p.cch = c.h;
  p.hl_soft = g->mod("hilite")->f("soft");
  if(g->debug) p.dbg_gauss = g->at<uint8_t>(g->off_dbg_gauss);
  if(g->crop_stage)
  {
    for(int k = 0; k < 20; k++) p.crop[k] = g->crop_blk[k];
    p.cw = g->out_w; p.ch = g->out_h;
    p.cr = g->at<half4>(g->off_cr);
  }
  // the bayer front writes the noop output only for the debug stage (the wavelet writes its own)
  if(g->k1front && (g->wavelet || !g->debug)) p.dn = nullptr;
}

// the kernel sequence of one run. ev != null records timing events around each launch.
int enqueue(vkdt_cuda_graph_t *g, cudaStream_t s, const void *d_src, void *d_out, bool timed)
{
  dev_image_t d;
  int r = fill_image(g, d, d_src, d_out);
  if(r) return r;
  dev_denoise_t dd;
  if(g->wavelet)
    fill_denoise(g, dd, d_src);
  const bool k1 = !g->unfused || g->k1front;   // the hilite front of the fused path
  if(g->wavelet && k1)
  { // the develop kernels read the denoised f16 mosaic through the identity code table
    d.mosaic = reinterpret_cast<const uint16_t *>(dd.dn);
    d.noop_lut = g->at<__half>(g->off_idlut);
    d.codes.identity = 1;
    d.pitch = g->W; d.cx = 0; d.cy = 0;
  }
  module_t *hl = g->mod("hilite");
  const float white = hl->f("white"), desat = hl->f("desat"), soft = hl->f("soft");
  const float wb[3] = { g->ip.whitebalance[0], g->ip.whitebalance[1], g->ip.whitebalance[2] };
  int li = 0;
  auto mark = [&]() -> int {
    if(timed) { CU(cudaEventRecord(g->ev[li], s)); }
    li++;
    return 0;
  };
  if(g->nblack[0] != g->lut_black || g->nwhite[0] != g->lut_white)
  { // new black/white since the code table was built: rebuild it on the device (same IEEE arithmetic)
    CU(launch_noop_lut(g->at<__half>(g->off_lut), g->nblack[0], g->nwhite[0], s));
    g->lut_black = g->nblack[0]; g->lut_white = g->nwhite[0];
  }
  if(g->want_hist) CU(cudaMemsetAsync(g->at<uint32_t>(g->off_hist), 0, 257 * sizeof(uint32_t), s));
  if((r = mark())) return r;
  // 0. wavelet denoise (strength > 0): half, downcov, down x3, assemble, doub
  if(g->wavelet)
    for(int stage = dd.fuse_half ? 1 : 0; stage < 7; stage++)
    {
      CU(launch_denoise(dd, stage, s));
      if((r = mark())) return r;
    }
  dev_nodes_t np;
  if(g->unfused)
  {
    fill_nodes(g, np, d_src);
    if(k1) { np.mosaic = d.mosaic; np.noop_lut = d.noop_lut; np.pitch = d.pitch; np.cx = d.cx; np.cy = d.cy; }
  }
  if(!k1)
  { // 1'. denoise/noop (unless the wavelet ran), hilite half, all hilite reduce levels
    if(!g->wavelet)
    {
      CU(launch_nodes(np, 0, s));
      if((r = mark())) return r;
    }
    CU(launch_nodes(np, 1, s));
    if((r = mark())) return r;
    for(size_t l = 0; l < g->hr.size() && (int)l < g->hl_tail; l++)
    {
      const half4 *in = l == 0 ? np.h0 : g->at<half4>(g->hr[l - 1].off);
      const int iw = l == 0 ? g->hw : g->hr[l - 1].w, ih = l == 0 ? g->hh : g->hr[l - 1].h;
      CU(launch_hilite_reduce(in, iw, ih, g->at<half4>(g->hr[l].off), g->hr[l].w, g->hr[l].h, white, desat, wb, s));
      if((r = mark())) return r;
    }
  }
  else
  {
  // 1. noop + hilite half + first hilite reduce
  dev_hilite_k1_t k1;
  memset(&k1, 0, sizeof(k1));
  k1.mosaic = d.mosaic; k1.codes = d.codes; k1.pitch = d.pitch; k1.cx = d.cx; k1.cy = d.cy; k1.W = d.W; k1.H = d.H;
  k1.filters = d.filters; k1.black = d.black; k1.white = d.white; k1.hl_white = white; k1.hl_desat = desat;
  for(int k = 0; k < 3; k++) k1.wb[k] = wb[k];
  k1.hw = g->hw; k1.hh = g->hh;
  k1.r1 = g->at<half4>(g->hr[0].off); k1.s1w = g->hr[0].w; k1.s1h = g->hr[0].h;
  CU(launch_hilite_k1(k1, s));
  if((r = mark())) return r;
  // 2. hilite reduce levels 2..L
  for(size_t l = 1; l < g->hr.size() && (int)l < g->hl_tail; l++)
  {
    CU(launch_hilite_reduce(g->at<half4>(g->hr[l - 1].off), g->hr[l - 1].w, g->hr[l - 1].h,
        g->at<half4>(g->hr[l].off), g->hr[l].w, g->hr[l].h, white, desat, wb, s));
    if((r = mark())) return r;
  }
  }
  if(g->hl_tail < (int)g->hr.size())
  { // 2'. the small end: reduce levels hl_tail.., assemble B[L-1] .. B[hl_tail] in one CTA
    dev_hilite_tail_t ht;
    memset(&ht, 0, sizeof(ht));
    const int t = g->hl_tail;
    ht.nr = (int)g->hr.size() - t;
    for(int l = 0; l <= ht.nr; l++) { ht.lw[l] = g->hr[t - 1 + l].w; ht.lh[l] = g->hr[t - 1 + l].h; }
    ht.in = g->at<half4>(g->hr[t - 1].off);
    ht.out = g->at<half4>(g->hb[t].off);
    ht.white = white; ht.desat = desat; ht.soft = soft;
    for(int k = 0; k < 3; k++) ht.wb[k] = wb[k];
    CU(launch_hilite_tail(ht, s));
    if((r = mark())) return r;
  }
  // 3. hilite assemble B[L-1] .. B[1]
  for(int l = (int)g->hb.size() - 1; l >= 0; l--)
  {
    if(l >= g->hl_tail) continue;   // made by the tail
    const level_t &f = g->hr[l];
    const level_t &c = (l + 1 < (int)g->hb.size()) ? g->hb[l + 1] : g->hr[l + 1];
    CU(launch_hilite_assemble(g->at<half4>(f.off), f.w, f.h, g->at<half4>(c.off), c.w, c.h,
        g->at<half4>(g->hb[l].off), white, soft, s));
    if((r = mark())) return r;
  }
  // the develop kernel's tensor map: the buffer d.mosaic points at, where one was made for it
  const CUtensorMap *dmap = nullptr;
  if(g->tm_arena == g->arena)
  {
    if(d.codes.identity && g->tm_dn_ok && (const void *)d.mosaic == (const void *)(g->arena + g->off_dn)) dmap = &g->tm_dn;
    else if(!d.codes.identity && g->tm_src_ok && (const void *)d.mosaic == (const void *)(g->arena + g->off_src)) dmap = &g->tm_src;
  }
  if(g->unfused)
  { // 4'. hilite level 0 assemble, doub, demosaic, colour .. first llap reduce
    if(g->k1front)
    { // noop + half + level 0 assemble + doub in one pass over the mosaic
      CU(launch_nodes(np, 8, s));
      if((r = mark())) return r;
    }
    else
    {
      const level_t &c = g->hb.empty() ? g->hr[0] : g->hb[0];
      CU(launch_hilite_assemble(np.h0, g->hw, g->hh, g->at<half4>(c.off), c.w, c.h, g->at<half4>(g->off_b0), white, soft, s));
      if((r = mark())) return r;
      CU(launch_nodes(np, 2, s));
      if((r = mark())) return r;
    }
    if(g->rcd)
    { // demosaic/rcd_conv, demosaic/rcd_fill
      dev_rcd_t rp;
      rp.cfa = np.hl; rp.W = g->W; rp.H = g->H;
      for(int k = 0; k < 3; k++) rp.wb[k] = g->ip.whitebalance[k];
      rp.vh = g->at<__half>(g->off_vh); rp.pq = g->at<__half>(g->off_pq); rp.lp = g->at<__half>(g->off_lpf);
      // rcd_fill applies colour, the histogram and filmcurv to its output pixels;
      // the demosaic output itself is kept only for the debug stage
      // (with a crop stage after it, rcd_fill writes the demosaic output and k_post the rest)
      rp.out = g->debug || g->crop_stage ? np.dm : nullptr;
      rp.post = !g->crop_stage;
      dev_image_t dp = d;
      dp.W = g->out_w; dp.H = g->out_h;
      for(int stage = 0; stage < 2; stage++)
      {
        CU(launch_rcd(rp, &dp, stage, s));
        if((r = mark())) return r;
      }
    }
    else
    {
      const int stages_half[2] = { 6, 7 }, stages_full[3] = { 3, 4, 5 };
      const int *st = g->halfsize ? stages_half : stages_full;
      const int nst = g->halfsize ? (g->resample ? 2 : 1) : 3;
      for(int i = 0; i < nst; i++)
      {
        CU(launch_nodes(np, st[i], s));
        if((r = mark())) return r;
      }
    }
    if(g->crop_stage && !g->crop_shift)
    { // crop/main on the demosaic output
      CU(launch_nodes(np, 9, s));
      if((r = mark())) return r;
    }
    dev_image_t dp = d;
    dp.W = g->out_w; dp.H = g->out_h;
    // the post kernel's input: the crop output, the window of the demosaic output, the demosaic
    // output, or nothing (rcd_fill applied colour and filmcurv itself)
    const half4 *window = g->at<half4>(g->off_dm + ((size_t)g->crop_dy * g->dm_w + g->crop_dx) * 8);
    const half4 *pin = g->crop_stage ? (g->crop_shift ? window : np.cr) : g->rcd ? nullptr : np.dm;
    CU(launch_post(dp, pin, g->crop_shift ? g->dm_w : g->out_w, s));
    if((r = mark())) return r;
  }
  else if(g->crop_shift)
  { // 4. fused develop pass to filmcurv on the crop window, then llap curve + first reduce on it
    dev_image_t dc = d;
    dc.l1 = nullptr;
    CU(launch_develop(dc, dmap, dmap ? device_status() : nullptr, s));
    if((r = mark())) return r;
    dev_image_t dp = d;
    dp.W = g->out_w; dp.H = g->out_h;
    CU(launch_post(dp, nullptr, g->out_w, s));
    if((r = mark())) return r;
  }
  else
  { // 4. fused develop pass
    CU(launch_develop(d, dmap, dmap ? device_status() : nullptr, s));
    if((r = mark())) return r;
  }
  // 5. llap reduce levels 2..nl-1 (TMA staged through the tensor maps made for this arena)
  const bool maps = g->tm_arena == g->arena && g->tm_reduce.size() + 1 == g->lp.size();
  for(size_t l = 1; l < g->lp.size(); l++)
  {
    CU(launch_llap_reduce(llap_level(g, g->lp[l - 1]), llap_level(g, g->lp[l]), maps ? &g->tm_reduce[l - 1] : nullptr,
        maps ? device_status() : nullptr, s));
    if((r = mark())) return r;
  }
  // 6. llap assemble A[nl-2] .. A[1]
  for(int j = (int)g->la.size(); j >= 1; j--)
  { // A[j] at level j (lp index j-1), l1 = level j+1 (lp index j)
    const bool first = (j == (int)g->la.size());
    const __half *coarse = first ? nullptr : g->at<__half>(g->la[j].off);
    CU(launch_llap_assemble(coarse, first ? 1 : 0, llap_level(g, g->lp[j - 1]), llap_level(g, g->lp[j]),
        g->at<__half>(g->la[j - 1].off), s));
    if((r = mark())) return r;
  }
  // 7. level 0 assemble + llap colour
  dev_llap_k3_t k3;
  memset(&k3, 0, sizeof(k3));
  if(g->grade)
  { // grade/main.comp:32-35: the fourth component is added to each channel
    const module_t *m = g->mod("grade");
    k3.grade = m->n("mode") == 0 ? 1 : 2;
    for(int k = 0; k < 3; k++)
    {
      k3.gr_lift[k] = m->f("lift", k) + m->f("lift", 3);
      k3.gr_gamma[k] = fmaxf(m->f("gamma", k) + m->f("gamma", 3), 1e-6f);
      k3.gr_gain[k] = fmaxf(m->f("gain", k) + m->f("gain", 3), 0.0f);
      k3.gr_off[k] = m->f("offset", k) + m->f("offset", 3);
    }
    k3.gr_sp = m->f("sh_pivot"); k3.gr_hp = m->f("hi_pivot");
  }
  k3.rgbf = d.rgbf; k3.W = g->out_w; k3.H = g->out_h;
  k3.l1 = d.l1; k3.l1w = d.l1w; k3.l1h = d.l1h; k3.l1pitch = d.l1pitch; k3.l1plane = d.l1plane;
  k3.coarse = g->la.empty() ? d.l1 + 10 * d.l1plane : g->at<__half>(g->la[0].off);
  k3.ll_sigma = d.ll_sigma; k3.ll_shadows = d.ll_shadows; k3.ll_highlights = d.ll_highlights; k3.ll_clarity = d.ll_clarity;
  k3.out = (half4 *)d_out;
  CU(launch_llap_final(k3, s));
  if((r = mark())) return r;
  return 0;
}

} // namespace

// error text for the calling thread (also used by the develop server)
int vkdt_set_error(int code, const char *msg)
{
  return fail(code, "%s", msg);
}

// ================================================================== C-ABI

#pragma GCC visibility push(default)
extern "C" {

const char *vkdt_cuda_last_error(void) { return g_err; }

int vkdt_cuda_init(int device_id, uint32_t flags)
{
  (void)flags;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if(e != cudaSuccess || n <= 0) return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "no CUDA device: %s", cudaGetErrorString(e));
  if(device_id < 0 || device_id >= n) return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "device %d out of range (%d)", device_id, n);
  cudaDeviceProp prop;
  CU(cudaGetDeviceProperties(&prop, device_id));
  if(prop.major != 10 || prop.minor != 3)
    return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "device %d is sm_%d%d, the library is built for sm_103a", device_id, prop.major, prop.minor);
  CU(cudaSetDevice(device_id));
  CU(init_develop());
  if(!g_status_host[device_id])
  {
    void *h = nullptr, *d = nullptr;
    CU(cudaHostAlloc(&h, 64, cudaHostAllocMapped | cudaHostAllocPortable));
    memset(h, 0, 64);
    CU(cudaHostGetDevicePointer(&d, h, 0));
    g_status_host[device_id] = (uint32_t *)h;
    g_status_dev[device_id] = (uint32_t *)d;
  }
  g_device = device_id;
  return VKDT_CUDA_SUCCESS;
}

void vkdt_cuda_cleanup(void)
{
  g_device = -1;
  forget_static_scratch();
}

int vkdt_cuda_supports(dt_token_t name, dt_token_t kernel)
{
  static const char *sup[][2] = {
    { "denoise", "noop" }, { "denoise", "half" }, { "denoise", "downcov" }, { "denoise", "down" },
    { "denoise", "assemble" }, { "denoise", "doub" }, { "demosaic", "halfsize" }, { "shared", "resample" },
    { "hilite", "half" }, { "hilite", "reduce" }, { "hilite", "assemble" }, { "hilite", "doub" },
    { "demosaic", "down" }, { "demosaic", "gauss" }, { "demosaic", "splat" }, { "demosaic", "fix" },
    { "demosaic", "rcd_conv" }, { "demosaic", "rcd_fill" },
    { "colour", "main" }, { "filmcurv", "main" }, { "OpenDRT", "hist" }, { "hist", "collect" },
    { "llap", "curve" }, { "llap", "reduce" }, { "llap", "assemble" }, { "llap", "colour" } };
  for(auto &s : sup) if(tkn(s[0]) == name && tkn(s[1]) == kernel) return 1;
  return 0;
}

int vkdt_cuda_graph_create(vkdt_cuda_graph_t **graph)
{
  if(!graph) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph pointer");
  vkdt_cuda_graph_t *g = new (std::nothrow) vkdt_cuda_graph_t();
  if(!g) return fail(VKDT_CUDA_ERROR_OUT_OF_HOST_MEMORY, "out of host memory");
  memset(&g->ip, 0, sizeof(g->ip));
  default_modules(g);
  *graph = g;
  return VKDT_CUDA_SUCCESS;
}

static void release(vkdt_cuda_graph_t *g)
{
  if(g->gexec) cudaGraphExecDestroy(g->gexec);
  g->gexec = nullptr;
  for(auto e : g->ev) cudaEventDestroy(e);
  g->ev.clear();
  if(g->done) cudaEventDestroy(g->done);
  g->done = nullptr;
  if(g->stream) cudaStreamDestroy(g->stream);
  g->stream = nullptr;
  if(g->arena) cudaFree(g->arena);
  g->arena = nullptr;
  g->tm_reduce.clear();
  g->tm_src_ok = g->tm_dn_ok = false;
  g->tm_arena = nullptr;
  if(g->h_src) cudaFreeHost(g->h_src);
  if(g->h_sink) cudaFreeHost(g->h_sink);
  g->h_src = g->h_sink = nullptr;
  g->allocated = false;
}

void vkdt_cuda_graph_destroy(vkdt_cuda_graph_t *g)
{
  if(!g) return;
  release(g);
  delete g;
}

int vkdt_cuda_graph_read_config(vkdt_cuda_graph_t *g, const char *cfg, size_t len)
{
  if(!g || !cfg) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null argument");
  std::string text(cfg, len);
  g->modules.clear(); g->unsupported.clear(); g->connects.clear();
  size_t pos = 0;
  int lineno = 0;
  bool seen_llap_clarity = false;
  while(pos <= text.size())
  {
    size_t e = text.find('\n', pos);
    if(e == std::string::npos) e = text.size();
    std::string line = text.substr(pos, e - pos);
    pos = e + 1;
    lineno++;
    while(!line.empty() && (line.back() == '\r' || line.back() == ' ')) line.pop_back();
    if(line.empty() || line[0] == '#') continue;
    std::vector<std::string> f;
    size_t a = 0;
    while(true)
    {
      size_t c = line.find(':', a);
      if(c == std::string::npos) { f.push_back(line.substr(a)); break; }
      f.push_back(line.substr(a, c - a));
      a = c + 1;
    }
    if(f[0] == "module" && f.size() >= 3)
    {
      const dt_token_t nm = tkn(f[1].c_str());
      const module_def_t *d = find_def(nm);
      if(!d)
      {
        if(std::find(g->unsupported.begin(), g->unsupported.end(), nm) == g->unsupported.end()) g->unsupported.push_back(nm);
        continue;
      }
      if(g->mod(f[1].c_str())) continue; // one instance per module on the path
      module_t m;
      m.init(d, nm, tkn(f[2].c_str()));
      g->modules.push_back(m);
    }
    else if(f[0] == "connect" && f.size() >= 7)
    {
      g->connects.push_back({ f[1] + ":" + f[2] + ":" + f[3], f[4] + ":" + f[5] + ":" + f[6] });
    }
    else if(f[0] == "param" && f.size() >= 5)
    {
      module_t *m = g->mod(f[1].c_str());
      if(!m) continue; // parameter of a module outside the path
      int cnt = 0; char type = 0;
      const int off = m->offset(tkn(f[3].c_str()), &cnt, &type);
      if(off < 0) continue;
      for(int i = 0; i < cnt && 4 + i < (int)f.size(); i++)
      {
        uint32_t u;
        if(type == 'i') { int32_t v = (int32_t)strtol(f[4 + i].c_str(), 0, 10); memcpy(&u, &v, 4); }
        else { float v = strtof(f[4 + i].c_str(), 0); memcpy(&u, &v, 4); }
        m->param[off + i] = u;
      }
      if(f[1] == "llap" && f[3] == "clarity") seen_llap_clarity = true;
    }
    else if(f[0] == "frames" || f[0] == "fps" || f[0] == "feedback" || f[0] == "keyframe" || f[0] == "paramsub")
      continue;
    else return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "cfg line %d not understood: %s", lineno, line.c_str());
  }
  (void)seen_llap_clarity;
  // the path must be present and chained
  const char *path[] = { "i-raw", "denoise", "hilite", "demosaic", "colour", "filmcurv", "llap" };
  for(const char *p : path) if(!g->mod(p)) return fail(VKDT_CUDA_INCOMPLETE, "module %s missing from the cfg", p);
  auto connected = [&](const char *from, const char *to) {
    for(auto &c : g->connects)
    {
      const std::string a = c.first.substr(0, c.first.find(':')), b = c.second.substr(0, c.second.find(':'));
      if(a == from && b == to) return true;
    }
    return false;
  };
  const bool ok = connected("i-raw", "denoise") && connected("denoise", "hilite") && connected("hilite", "demosaic")
      && (connected("demosaic", "colour") || (connected("demosaic", "crop") && connected("crop", "colour")))
      && connected("colour", "filmcurv") && connected("filmcurv", "llap");
  if(!ok) return fail(VKDT_CUDA_INCOMPLETE, "the cfg does not chain i-raw -> denoise -> hilite -> demosaic -> [crop] -> colour -> filmcurv -> llap");
  g->crop = !connected("demosaic", "colour");
  g->grade = g->mod("grade") && connected("llap", "grade");
  g->graph_dirty = true;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_unsupported(vkdt_cuda_graph_t *g, dt_token_t *names, int max)
{
  if(!g) return 0;
  for(int i = 0; i < (int)g->unsupported.size() && i < max; i++) if(names) names[i] = g->unsupported[i];
  return (int)g->unsupported.size();
}

static int param_access(vkdt_cuda_graph_t *g, dt_token_t module, dt_token_t inst, dt_token_t param, size_t bytes, int *off)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  module_t *m = nullptr;
  for(auto &mm : g->modules) if(mm.name == module && (inst == 0 || mm.inst == inst)) m = &mm;
  if(!m) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "no module %s:%s", tstr(module).c_str(), tstr(inst).c_str());
  int cnt = 0;
  *off = m->offset(param, &cnt, 0);
  if(*off < 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "module %s has no parameter %s", tstr(module).c_str(), tstr(param).c_str());
  if(bytes != (size_t)cnt * 4) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "parameter %s wants %d bytes", tstr(param).c_str(), cnt * 4);
  return 0;
}

int vkdt_cuda_graph_set_param(vkdt_cuda_graph_t *g, dt_token_t module, dt_token_t inst, dt_token_t param, const void *value, size_t bytes)
{
  int off, r = param_access(g, module, inst, param, bytes, &off);
  if(r) return r;
  for(auto &m : g->modules) if(m.name == module && (inst == 0 || m.inst == inst)) memcpy(&m.param[off], value, bytes);
  g->graph_dirty = true;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_get_param(vkdt_cuda_graph_t *g, dt_token_t module, dt_token_t inst, dt_token_t param, void *value, size_t bytes)
{
  int off, r = param_access(g, module, inst, param, bytes, &off);
  if(r) return r;
  for(auto &m : g->modules) if(m.name == module && (inst == 0 || m.inst == inst)) { memcpy(value, &m.param[off], bytes); break; }
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_set_input(vkdt_cuda_graph_t *g, int wd, int ht, const vkdt_cuda_img_param_t *ip)
{
  if(!g || !ip) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null argument");
  if(wd <= 0 || ht <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad input size %dx%d", wd, ht);
  g->in_wd = wd; g->in_ht = ht; g->ip = *ip;
  for(int k = 0; k < 4; k++) { g->nblack[k] = ip->black[k] / 65535.0f; g->nwhite[k] = ip->white[k] / 65535.0f; }
  g->colour_given = false;
  g->crop_given = false;
  // i-raw/main.c:214-218 normalises the white balance to green
  if(g->ip.whitebalance[1] > 0.0f && g->ip.whitebalance[1] != 1.0f)
  {
    g->ip.whitebalance[0] /= g->ip.whitebalance[1];
    g->ip.whitebalance[2] /= g->ip.whitebalance[1];
    g->ip.whitebalance[3] /= g->ip.whitebalance[1];
    g->ip.whitebalance[1] = 1.0f;
  }
  g->have_input = true;
  g->graph_dirty = true;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_set_output_size(vkdt_cuda_graph_t *g, int wd, int ht)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  g->req_wd = wd; g->req_ht = ht;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_set_llap_levels(vkdt_cuda_graph_t *g, int levels)
{
  if(!g || levels < 0 || levels == 1 || levels > 12) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "llap levels %d", levels);
  g->llap_levels_req = levels;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_set_timing(vkdt_cuda_graph_t *g, int enable) { if(!g) return -11; g->timing = enable != 0; return 0; }
int vkdt_cuda_graph_set_hist(vkdt_cuda_graph_t *g, int enable) { if(!g) return -11; g->want_hist = enable != 0; g->graph_dirty = true; return 0; }
int vkdt_cuda_graph_set_debug(vkdt_cuda_graph_t *g, int enable) { if(!g) return -11; g->debug = enable != 0; return 0; }

int vkdt_cuda_graph_create_nodes(vkdt_cuda_graph_t *g)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  if(!g->have_input) return fail(VKDT_CUDA_INCOMPLETE, "no input set");
  int r = check_supported_params(g);
  if(r) return r;
  const uint32_t filters = g->ip.filters;
  if(filters == 0) return fail(VKDT_CUDA_INCOMPLETE, "rgb input: the path starts on a mosaic");
  g->nodes.clear();
  // denoise modify_roi_out: output = crop window
  const uint32_t *b = g->ip.crop_aabb;
  if(b[2] <= b[0] || b[3] <= b[1] || (int)b[2] > g->in_wd || (int)b[3] > g->in_ht)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "crop window outside the mosaic");
  g->W = (int)(b[2] - b[0]); g->H = (int)(b[3] - b[1]);
  const bool xt = filters == 9u;
  g->block = xt ? 3 : 2;
  if(!xt && ((g->W & 1) || (g->H & 1) || (b[0] & 1) || (b[1] & 1) || (g->in_wd & 1)))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bayer mosaic width and crop window must be even");
  if(g->W < 16 || g->H < 16) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "image smaller than 16x16");
  g->hw = g->W / g->block; g->hh = g->H / g->block;
  g->doub_fixed = !xt && doub_taps_fixed(g->W, g->hw) && doub_taps_fixed(g->H, g->hh);
  // demosaic/main.c:18-41, 92-111: a requested size of 1/(1.5 block) or less
  // takes the half size demosaic, resampled unless the scale is the block
  const int method = g->mod("demosaic")->n("method");
  {
    // method 2 always takes the half size demosaic; its full output size is then (W+1)/2
    const int fw = method == 2 ? (g->W + 1) / 2 : g->W, fh = method == 2 ? (g->H + 1) / 2 : g->H;
    const int ow = g->req_wd > 0 ? g->req_wd : fw, oh = g->req_ht > 0 ? g->req_ht : fh;
    const float scale = (float)g->W / (float)ow;
    g->halfsize = method == 2 || ((ow != g->W || oh != g->H) && scale >= 1.5f * g->block);
    if(!g->halfsize && (ow != g->W || oh != g->H))
      return fail(VKDT_CUDA_INCOMPLETE, "resampling after the full size demosaic is not built in this version");
    g->resample = g->halfsize && (float)g->block != scale;
    if(!g->halfsize) { g->out_w = g->W; g->out_h = g->H; }
    else if(g->resample) { g->out_w = ow; g->out_h = oh; }
    else { g->out_w = g->hw; g->out_h = g->hh; }
  }
  // crop between demosaic and colour (crop/main.c:252-343): the stages after it run at its size;
  // a crop that copies its input (the identity at the input's size) has no launch of its own
  g->dm_w = g->out_w; g->dm_h = g->out_h;
  g->crop_stage = false;
  if(g->crop)
  {
    if(!g->crop_given) crop_commit(g, g->dm_w, g->dm_h, g->crop_blk, &g->crop_w, &g->crop_h);
    if(g->crop_w < 16 || g->crop_h < 16)
      return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "crop output %dx%d smaller than 16x16", g->crop_w, g->crop_h);
    g->crop_stage = !crop_identity(g->crop_blk, g->dm_w, g->dm_h, g->crop_w, g->crop_h);
    g->out_w = g->crop_w; g->out_h = g->crop_h;
  }
  // demosaic/main.c:113: rcd at full size, whatever the pattern (its tiles need an even width)
  g->rcd = method == 1 && !g->halfsize;
  if(g->rcd && (g->W & 1)) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "rcd needs an even width");
  // bayer at full size runs fused; x-trans, rcd and reduced sizes run node by node,
  // bayer with the fused path's hilite front
  // a demosaic colour param >= 1 widens the bayer fix radius to 2 (fix.comp:124): node by node
  const bool wide_fix = !xt && g->mod("demosaic")->n("colour") >= 1;
  // a crop by whole texels rides on the fused kernel, or on the post kernel of the per-node chain
  // (it reads the window of the demosaic output); any other crop resamples (its own launch)
  g->crop_shift = g->crop_stage
               && crop_whole_texels(g->crop_blk, g->dm_w, g->dm_h, g->out_w, g->out_h, &g->crop_dx, &g->crop_dy);
  g->unfused = xt || g->halfsize || g->rcd || wide_fix || (g->crop_stage && !g->crop_shift);
  g->k1front = g->unfused && !xt;

  // node lists as the modules' create_nodes emit them
  g->wavelet = g->mod("denoise")->f("strength") > 0.0f;
  if(!g->wavelet) add_node(g, "denoise", "noop", g->W, g->H, 1, -1);
  else
  { // denoise/main.c:225-333: 4 scales at the half size, assemble, half, doub
    add_node(g, "denoise", "downcov", g->hw, g->hh, 1, -1);
    for(int i = 1; i < 4; i++) add_node(g, "denoise", "down", g->hw, g->hh, 1, -1);
    add_node(g, "denoise", "assemble", g->hw, g->hh, 1, -1);
    add_node(g, "denoise", "half", g->hw, g->hh, 1, -1);
    add_node(g, "denoise", "doub", g->W, g->H, 1, -1);
  }
  // hilite/main.c:5-90
  add_node(g, "hilite", "half", g->hw, g->hh, 1, -1);
  add_node(g, "hilite", "doub", g->hw, g->hh, 1, -1);
  g->hr.clear(); g->hb.clear();
  {
    int rw = (g->hw - 1) / 2 + 1, rh = (g->hh - 1) / 2 + 1;
    const int max_nl = 15;
    for(int l = 1; l < max_nl; l++)
    {
      level_t lv; lv.w = rw; lv.h = rh;
      g->hr.push_back(lv);
      rw = (rw - 1) / 2 + 1; rh = (rh - 1) / 2 + 1;
      if(rw <= 1 || rh <= 1 || l + 1 == max_nl) break;
    }
    for(size_t l = 0; l + 1 < g->hr.size(); l++) g->hb.push_back(g->hr[l]);
    // the small end of the pyramid in one CTA (k_hilite_tail): from the first
    // level of at most HL_TAIL_IN texels whose working set fits its shared
    // memory, if two or more levels follow (one SM: larger levels take longer
    // there than their own launches)
    const int L = (int)g->hr.size();
    g->hl_tail = L;
    for(int t = 1; t + 2 <= L; t++)
    {
      const int nr = L - t;
      if(nr >= HL_TAIL_MAX) continue;
      int lw[HL_TAIL_MAX], lh[HL_TAIL_MAX];
      for(int l = 0; l <= nr; l++) { lw[l] = g->hr[t - 1 + l].w; lh[l] = g->hr[t - 1 + l].h; }
      if(lw[0] * lh[0] <= HL_TAIL_IN && hilite_tail_smem_bytes(lw, lh, nr) <= HL_TAIL_SMEM) { g->hl_tail = t; break; }
    }
  }
  const int OW = g->out_w, OH = g->out_h;
  if(g->halfsize)
  { // demosaic/main.c:92-111
    add_node(g, "demosaic", "halfsize", g->hw, g->hh, 1, -1);
    if(g->resample) add_node(g, "shared", "resample", g->dm_w, g->dm_h, 1, -1);
  }
  else if(g->rcd)
  { // demosaic/main.c:113-155: one rcd_fill workgroup (8 invocations of the node size) per 58x26 tile
    add_node(g, "demosaic", "rcd_conv", g->W, g->H, 1, -1);
    add_node(g, "demosaic", "rcd_fill", (g->W + 57) / 58 * 8, (g->H + 25) / 26 * 8, 1, -1);
  }
  else
  { // demosaic/main.c:159-202 (gaussian splats, full size)
    add_node(g, "demosaic", "down", g->hw, g->hh, 1, -1);
    add_node(g, "demosaic", "gauss", g->hw, g->hh, 1, -1);
    add_node(g, "demosaic", "splat", g->W, g->H, 1, -1);
    add_node(g, "demosaic", "fix", g->W, g->H, 1, -1);
  }
  if(g->crop) add_node(g, "crop", "main", OW, OH, 1, -1);   // crop/main.c: the default create_nodes
  add_node(g, "colour", "main", OW, OH, 1, -1);
  add_node(g, "OpenDRT", "hist", (OW + 15) / 16 * 8, (OH + 15) / 16 * 8, 1, -1);
  add_node(g, "filmcurv", "main", OW, OH, 1, -1);
  // llap/main.c:6-106
  add_node(g, "llap", "curve", OW, OH, 1, -1);
  g->lp.clear(); g->la.clear();
  {
    int rw = (OW - 1) / 2 + 1, rh = (OH - 1) / 2 + 1;
    int nl = 12;
    for(int l = 1; l < nl; l++)
    {
      level_t lv; lv.w = rw; lv.h = rh; lv.pitch = (rw + 7) & ~7;
      g->lp.push_back(lv);
      rw = (rw - 1) / 2 + 1; rh = (rh - 1) / 2 + 1;
      if(rw <= 1 || rh <= 1) { nl = l + 1; break; }
      if(g->llap_levels_req > 0 && l + 1 == g->llap_levels_req) { nl = l + 1; break; }
    }
    g->nl = nl;
    for(int j = 1; j <= nl - 2; j++) g->la.push_back(g->lp[j - 1]);
  }
  // the launches and which nodes they compute
  g->launches.clear();
  auto launch = [&](const char *n, const char *k) { g->launches.push_back({ tkn(n), tkn(k) }); return (int)g->launches.size() - 1; };
  int L_dn[7] = { -1, -1, -1, -1, -1, -1, -1 };
  if(g->wavelet)
  {
    const char *dk[7] = { "half", "downcov", "down", "down", "down", "assemble", "doub" };
    // bayer: the downcov launch makes the half image as well
    for(int i = g->ip.filters != 9u ? 1 : 0; i < 7; i++) L_dn[i] = launch("denoise", dk[i]);
    if(L_dn[0] < 0) L_dn[0] = L_dn[1];
  }
  std::vector<int> L_hr, L_ha, L_lr, L_la;
  int L_noop = -1, L_half = -1, L_a0 = -1, L_doub = -1, L_gauss = -1, L_splat = -1, L_fix = -1, L_hs = -1, L_rs = -1;
  int L_rcdc = -1, L_rcdf = -1, L_crop = -1, L_curve = -1;
  int L_post, L_k1 = -1;
  const bool k1 = !g->unfused || g->k1front;
  int L_tail = -1;   // the one-CTA tail computes hr[hl_tail..] and hb[hl_tail..]
  auto hl_reduce = [&](size_t l) {
    if((int)l < g->hl_tail) return launch("hilite", "reduce");
    if(L_tail < 0) L_tail = launch("hilite", "reduce");
    return L_tail;
  };
  auto hl_assemble = [&](size_t l) { return (int)l < g->hl_tail ? launch("hilite", "assemble") : L_tail; };
  if(k1)
  {
    L_k1 = launch("hilite", "reduce");
    for(size_t l = 1; l < g->hr.size(); l++) L_hr.push_back(hl_reduce(l));
    for(size_t l = 0; l < g->hb.size(); l++) L_ha.push_back(hl_assemble(l));
  }
  if(!g->unfused)
  {
    L_post = launch("demosaic", "fix");
    if(g->crop_shift) L_curve = launch("llap", "curve");   // llap curve + first reduce on the cropped image
  }
  else
  {
    if(!k1)
    {
      if(!g->wavelet) L_noop = launch("denoise", "noop");
      L_half = launch("hilite", "half");
      for(size_t l = 0; l < g->hr.size(); l++) L_hr.push_back(hl_reduce(l));
      for(size_t l = 0; l < g->hb.size(); l++) L_ha.push_back(hl_assemble(l));
      L_a0 = launch("hilite", "assemble");
    }
    L_doub = launch("hilite", "doub");
    if(g->halfsize)
    {
      L_hs = launch("demosaic", "halfsize");
      if(g->resample) L_rs = launch("shared", "resample");
    }
    else if(g->rcd)
    {
      L_rcdc = launch("demosaic", "rcd_conv");
      L_rcdf = launch("demosaic", "rcd_fill");
    }
    else
    {
      L_gauss = launch("demosaic", "gauss");
      L_splat = launch("demosaic", "splat");
      L_fix = launch("demosaic", "fix");
    }
    if(g->crop_stage && !g->crop_shift) L_crop = launch("crop", "main");
    L_post = launch("llap", "curve");
  }
  for(size_t l = 1; l < g->lp.size(); l++) L_lr.push_back(launch("llap", "reduce"));
  for(size_t j = 0; j < g->la.size(); j++) L_la.push_back(launch("llap", "assemble"));
  const int L_fin = launch("llap", "colour");
  for(auto &n : g->nodes)
  {
    if(n.name == tkn("denoise") && g->wavelet)
    { // one launch per node, in create_nodes order: downcov, down x3, assemble, half, doub
      static const int map[7] = { 1, 2, 3, 4, 5, 0, 6 };
      n.fused = L_dn[map[&n - &g->nodes[0]]];
      continue;
    }
    if(!g->unfused)
    {
      if(n.name == tkn("denoise") || n.kernel == tkn("doub") || n.name == tkn("demosaic") || n.name == tkn("colour")
          || n.name == tkn("OpenDRT") || n.name == tkn("filmcurv") || n.kernel == tkn("curve") || n.name == tkn("crop"))
        n.fused = L_post;
      if(n.kernel == tkn("curve") && g->crop_shift) n.fused = L_curve;
      if(n.name == tkn("hilite") && n.kernel == tkn("half")) n.fused = L_k1;
      continue;
    }
    if(n.name == tkn("denoise")) n.fused = k1 ? L_doub : L_noop;
    else if(n.name == tkn("hilite")) n.fused = n.kernel == tkn("half") ? (k1 ? L_k1 : L_half) : L_doub;
    else if(n.kernel == tkn("halfsize")) n.fused = L_hs;
    else if(n.kernel == tkn("resample")) n.fused = L_rs;
    else if(n.kernel == tkn("rcd_conv")) n.fused = L_rcdc;
    else if(n.kernel == tkn("rcd_fill")) n.fused = L_rcdf;
    else if(n.kernel == tkn("gauss") || n.kernel == tkn("down")) n.fused = L_gauss;
    else if(n.kernel == tkn("splat")) n.fused = L_splat;
    else if(n.kernel == tkn("fix")) n.fused = L_fix;
    else if(n.name == tkn("crop")) n.fused = g->crop_stage && !g->crop_shift ? L_crop : L_post;
    else n.fused = L_post;   // colour, histogram, filmcurv, llap curve
  }
  // per level nodes (reduce and assemble pairs in create_nodes order)
  for(size_t l = 0; l < g->hr.size(); l++)
  {
    const int lr = !k1 ? L_hr[l] : (l == 0 ? L_k1 : L_hr[l - 1]);
    const int la = l == 0 ? (!g->unfused ? L_post : (k1 ? L_doub : L_a0)) : L_ha[l - 1];
    add_node(g, "hilite", "reduce", g->hr[l].w, g->hr[l].h, 1, lr);
    const int fw = l == 0 ? g->hw : g->hr[l - 1].w, fh = l == 0 ? g->hh : g->hr[l - 1].h;
    add_node(g, "hilite", "assemble", fw, fh, 1, la);
  }
  for(size_t l = 0; l < g->lp.size(); l++)
  {
    add_node(g, "llap", "reduce", g->lp[l].w, g->lp[l].h, 11, l == 0 ? (!g->unfused && g->crop_shift ? L_curve : L_post) : L_lr[l - 1]);
    const int fw = l == 0 ? OW : g->lp[l - 1].w, fh = l == 0 ? OH : g->lp[l - 1].h;
    add_node(g, "llap", "assemble", fw, fh, 1, l == 0 ? L_fin : L_la[l - 1]);
  }
  add_node(g, "llap", "colour", OW, OH, 1, L_fin);
  if(g->grade) add_node(g, "grade", "main", OW, OH, 1, L_fin);

  g->nodes_ready = true;
  g->nodes_for = plan_key(g);
  { // the scheduler commits the modules' params with their nodes
    float p_wb[3];
    colour_commit_white(g, p_wb);
  }
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_alloc(vkdt_cuda_graph_t *g, uint64_t *device_bytes)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  if(g_device < 0) return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "vkdt_cuda_init was not called");
  release(g);
  int r = vkdt_cuda_graph_create_nodes(g);
  if(r) return r;
  g->arena_bytes = plan_arena(g);
  CU(cudaMalloc((void **)&g->arena, g->arena_bytes));
  CU(cudaMemset(g->arena, 0, g->arena_bytes));
  { // tensor maps of the llap levels the reduce launches stage by TMA (else 4 byte copies)
    std::vector<CUtensorMap> maps(g->lp.empty() ? 0 : g->lp.size() - 1);
    bool ok = device_status() != nullptr;
    for(size_t l = 1; l < g->lp.size() && ok; l++) ok = llap_reduce_tensor_map(llap_level(g, g->lp[l - 1]), &maps[l - 1]) == cudaSuccess;
    if(ok) { g->tm_reduce = maps; g->tm_arena = g->arena; }
    // the develop kernel's mosaic windows: the source (16 byte aligned crop origin) or the denoised mosaic
    g->tm_src_ok = ok && !(g->ip.crop_aabb[0] & 7)
                && develop_tensor_map(g->arena + g->off_src, g->in_wd, g->in_ht, g->in_wd, &g->tm_src) == cudaSuccess;
    g->tm_dn_ok = ok && g->wavelet
               && develop_tensor_map(g->arena + g->off_dn, g->W, g->H, g->W, &g->tm_dn) == cudaSuccess;
  }
  if(g->wavelet && (!g->unfused || g->k1front))
  {
    std::vector<uint16_t> id(65536);
    for(int v = 0; v < 65536; v++) id[v] = (uint16_t)v;
    CU(cudaMemcpy(g->arena + g->off_idlut, id.data(), 65536 * 2, cudaMemcpyHostToDevice));
  }
  { // denoise/noop.comp:385 for every u16 code, channel 0 black/white (denoise/main.c:165-168)
    std::vector<__half> lut(65536);
    const float black = g->nblack[0], white = g->nwhite[0];
    for(int v = 0; v < 65536; v++)
    {
      const float x = (float)v / 65535.0f;
      lut[v] = __float2half_rn(std::fmax(0.0f, (x - black) / (white - black)));
    }
    CU(cudaMemcpy(g->arena + g->off_lut, lut.data(), 65536 * 2, cudaMemcpyHostToDevice));
    g->lut_black = g->nblack[0]; g->lut_white = g->nwhite[0];
  }
  CU(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
  g->ev.resize(g->launches.size() + 1);
  for(auto &e : g->ev) CU(cudaEventCreate(&e));
  g->times.assign(g->launches.size(), 0.0f);
  g->allocated = true;
  g->graph_dirty = true;
  g->planned_for = plan_key(g);
  if(device_bytes) *device_bytes = g->arena_bytes;
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_plan_bytes(vkdt_cuda_graph_t *g, uint64_t *device_bytes)
{
  if(!g || !device_bytes) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null argument");
  if(g->allocated) { *device_bytes = g->arena_bytes; return 0; }
  int r = vkdt_cuda_graph_create_nodes(g);
  if(r) return r;
  *device_bytes = plan_arena(g);
  return 0;
}


int vkdt_cuda_graph_node_count(vkdt_cuda_graph_t *g) { return g ? (int)g->nodes.size() : 0; }
namespace {
// little endian 4-byte fields of a push constant or uniform block
float fat(const void *p, uint32_t size, int i) { float v = 0; if(p && (uint32_t)(4 * i + 4) <= size) memcpy(&v, (const uint8_t *)p + 4 * i, 4); return v; }
int32_t iat(const void *p, uint32_t size, int i) { int32_t v = 0; if(p && (uint32_t)(4 * i + 4) <= size) memcpy(&v, (const uint8_t *)p + 4 * i, 4); return v; }
}

int vkdt_cuda_graph_set_nodes(vkdt_cuda_graph_t *g, int in_wd, int in_ht, const vkdt_cuda_node_desc_t *nodes, int count)
{
  if(!g || !nodes || count <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "no nodes");
  if(g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph already allocated");
  auto find = [&](const char *name, const char *kernel) -> const vkdt_cuda_node_desc_t * {
    for(int i = 0; i < count; i++) if(nodes[i].name == tkn(name) && nodes[i].kernel == tkn(kernel)) return nodes + i;
    return nullptr;
  };
  auto module_uniform = [&](const char *name) -> const vkdt_cuda_node_desc_t * {
    for(int i = 0; i < count; i++) if(nodes[i].name == tkn(name) && nodes[i].uniform) return nodes + i;
    return nullptr;
  };
  vkdt_cuda_img_param_t ip;
  memset(&ip, 0, sizeof(ip));
  float nblack[4], nwhite[4];
  // ---- denoise (denoise/main.c:133-333): noop, or the wavelet nodes
  const vkdt_cuda_node_desc_t *noop = find("denoise", "noop"), *half = find("denoise", "half");
  const vkdt_cuda_node_desc_t *doub = find("denoise", "doub");
  if(noop)
  { // {crop[4], black[4], white[4], map_os[4], filters, gainmap}
    const uint32_t ps = noop->push_size;
    for(int k = 0; k < 4; k++)
    {
      ip.crop_aabb[k] = (uint32_t)iat(noop->push, ps, k);
      nblack[k] = fat(noop->push, ps, 4 + k); nwhite[k] = fat(noop->push, ps, 8 + k);
    }
    ip.filters = (uint32_t)iat(noop->push, ps, 16);
    if(iat(noop->push, ps, 17)) return fail(VKDT_CUDA_INCOMPLETE, "denoise with a dng gain map is not built");
  }
  else if(half && doub)
  { // half: {wb[4], black[4], white[4], crop[4], filters}; doub adds {noise a, noise b, gainmap, ...}
    const uint32_t ps = half->push_size;
    for(int k = 0; k < 4; k++)
    {
      nblack[k] = fat(half->push, ps, 4 + k); nwhite[k] = fat(half->push, ps, 8 + k);
      ip.crop_aabb[k] = (uint32_t)iat(half->push, ps, 12 + k);
    }
    ip.filters = (uint32_t)iat(half->push, ps, 16);
    ip.noise_a = fat(doub->push, doub->push_size, 17);
    ip.noise_b = fat(doub->push, doub->push_size, 18);
    if(iat(doub->push, doub->push_size, 19)) return fail(VKDT_CUDA_INCOMPLETE, "denoise with a dng gain map is not built");
  }
  else return fail(VKDT_CUDA_INCOMPLETE, "no denoise nodes on a mosaic (rgb input, or another chain)");
  // crop_aabb is (x0, y0, x1, y1) at full resolution when the input is not scaled
  // ---- white balance and CFA from the demosaic (or hilite) push constants {wb[4], filters}
  const vkdt_cuda_node_desc_t *wbn = nullptr;
  for(const char *k : { "gauss", "splat", "fix", "rcd_fill", "halfsize", "down" }) if(!wbn) wbn = find("demosaic", k);
  if(!wbn) wbn = find("hilite", "half");
  if(!wbn) return fail(VKDT_CUDA_INCOMPLETE, "no demosaic or hilite nodes");
  for(int k = 0; k < 4; k++) ip.whitebalance[k] = fat(wbn->push, wbn->push_size, k);
  if((uint32_t)iat(wbn->push, wbn->push_size, 4) != ip.filters) return fail(VKDT_CUDA_INCOMPLETE, "inconsistent CFA");
  // black/white in DN for the metadata; the kernels take the normalised values as pushed
  for(int k = 0; k < 4; k++) { ip.black[k] = nblack[k] * 65535.0f; ip.white[k] = nwhite[k] * 65535.0f; }
  for(int i = 0; i < 9; i++) ip.cam_to_rec2020[i] = (i % 4 == 0) ? 1.0f : 0.0f;
  // ---- module parameters from the uniform blocks (the params files' order, 4 bytes each)
  auto set_f = [&](const char *mod, const char *par, int n, const vkdt_cuda_node_desc_t *u, int at) {
    module_t *m = ensure_module(g, mod);
    for(int k = 0; k < n; k++) m->setf(par, k, fat(u->uniform, u->uniform_size, at + k));
  };
  auto set_i = [&](const char *mod, const char *par, const vkdt_cuda_node_desc_t *u, int at) {
    module_t *m = ensure_module(g, mod);
    const int32_t v = iat(u->uniform, u->uniform_size, at);
    int o = m->offset(tkn(par), 0, 0);
    memcpy(&m->param[o], &v, 4);
  };
  const vkdt_cuda_node_desc_t *u;
  if((u = module_uniform("denoise")))
  { // strength, luma, detail, pad, edges[4], gainmap
    set_f("denoise", "strength", 1, u, 0); set_f("denoise", "luma", 1, u, 1); set_f("denoise", "detail", 1, u, 2);
    set_f("denoise", "edges", 4, u, 4); set_i("denoise", "gainmap", u, 8);
  }
  if((u = module_uniform("hilite"))) { set_f("hilite", "white", 1, u, 0); set_f("hilite", "desat", 1, u, 1); set_f("hilite", "soft", 1, u, 2); }
  if((u = module_uniform("demosaic"))) { set_i("demosaic", "colour", u, 0); set_i("demosaic", "method", u, 1); }
  if((u = module_uniform("filmcurv")))
  {
    set_f("filmcurv", "light", 1, u, 0); set_f("filmcurv", "contrast", 1, u, 1); set_f("filmcurv", "bias", 1, u, 2);
    set_i("filmcurv", "colour", u, 3);
    const char *rest[] = { "chroma", "rolloff", "red", "yellow", "blue", "shadows" };
    for(int k = 0; k < 6; k++) set_f("filmcurv", rest[k], 1, u, 4 + k);
  }
  if((u = module_uniform("llap")))
  {
    set_f("llap", "sigma", 1, u, 0); set_f("llap", "shadows", 1, u, 1); set_f("llap", "hilights", 1, u, 2);
    set_f("llap", "clarity", 1, u, 3);
  }
  // colour/main.c:219-365: the committed block. off = 4+12+4+12+4*24+4*24
  u = module_uniform("colour");
  if(!u || u->uniform_size < 4 * (224 + 8)) return fail(VKDT_CUDA_INCOMPLETE, "no colour uniform block");
  {
    const int off = 224;
    if(iat(u->uniform, u->uniform_size, off + 1) != 0) return fail(VKDT_CUDA_INCOMPLETE, "colour clut mode not built");
    if(fat(u->uniform, u->uniform_size, off + 2) != 1.0f) return fail(VKDT_CUDA_INCOMPLETE, "colour saturation != 1 not built");
    if(iat(u->uniform, u->uniform_size, off + 3) != 0 || iat(u->uniform, u->uniform_size, off + 4) != 0)
      return fail(VKDT_CUDA_INCOMPLETE, "colour picker / gamut not built");
    if(fat(u->uniform, u->uniform_size, off + 7) != 0.0f) return fail(VKDT_CUDA_INCOMPLETE, "colour clip not built");
    if(iat(u->uniform, u->uniform_size, 16) != 0) return fail(VKDT_CUDA_INCOMPLETE, "colour rbf mode not built");
    g->colour_mul[0] = fat(u->uniform, u->uniform_size, 0);
    g->colour_mul[1] = 1.0f;
    g->colour_mul[2] = fat(u->uniform, u->uniform_size, 2);
    g->colour_mulw = fat(u->uniform, u->uniform_size, 3);
    for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)   // f[4+4i+j] = cam[3j+i]
      g->colour_cam[3 * j + i] = fat(u->uniform, u->uniform_size, 4 + 4 * i + j);
  }
  // ---- sizes: the llap depth from its reduce nodes, the output size from llap/colour
  int reduces = 0;
  for(int i = 0; i < count; i++) reduces += nodes[i].name == tkn("llap") && nodes[i].kernel == tkn("reduce");
  const vkdt_cuda_node_desc_t *fin = find("llap", "colour");
  if(!fin || !find("colour", "main") || !find("filmcurv", "main")) return fail(VKDT_CUDA_INCOMPLETE, "not the development chain");
  int r = vkdt_cuda_graph_set_input(g, in_wd, in_ht, &ip);
  if(r) return r;
  for(int k = 0; k < 4; k++) { g->nblack[k] = nblack[k]; g->nwhite[k] = nwhite[k]; }
  g->colour_given = true;
  g->llap_levels_req = reduces + 1;
  const int W = (int)(ip.crop_aabb[2] - ip.crop_aabb[0]), H = (int)(ip.crop_aabb[3] - ip.crop_aabb[1]);
  const int method = g->mod("demosaic")->n("method");
  const int fw = method == 2 ? (W + 1) / 2 : W, fh = method == 2 ? (H + 1) / 2 : H;
  const vkdt_cuda_node_desc_t *cr = find("crop", "main");
  g->crop = cr != nullptr;
  if(cr)
  { // crop/main.c:276-343: the committed block {mat3 H (padded columns), r0..r3, x X y Y} and its size
    if(!cr->uniform || cr->uniform_size < 20 * 4) return fail(VKDT_CUDA_INCOMPLETE, "no crop uniform block");
    ensure_module(g, "crop");
    for(int k = 0; k < 20; k++) g->crop_blk[k] = fat(cr->uniform, cr->uniform_size, k);
    g->crop_w = cr->wd; g->crop_h = cr->ht;
    g->crop_given = true;
    if(fin->wd != cr->wd || fin->ht != cr->ht) return fail(VKDT_CUDA_INCOMPLETE, "crop with a scaled output size is not built");
    g->req_wd = g->req_ht = 0;
  }
  else
  {
    g->req_wd = (fin->wd != fw || fin->ht != fh) ? fin->wd : 0;
    g->req_ht = (fin->wd != fw || fin->ht != fh) ? fin->ht : 0;
  }
  if((r = vkdt_cuda_graph_create_nodes(g))) return r;
  // ---- the plan covers exactly these nodes
  std::vector<std::array<int64_t, 5>> want, have;
  for(int i = 0; i < count; i++)
  {
    const vkdt_cuda_node_desc_t &n = nodes[i];
    if(n.name == tkn("filmcurv") && n.kernel == tkn("dspy")) continue;   // the display curve, not on the path
    if(n.name == tkn("shared") && n.kernel == tkn("resample") && n.wd == g->W && n.ht == g->H && !g->halfsize) continue;
    want.push_back({ (int64_t)n.name, (int64_t)n.kernel, n.wd, n.ht, n.dp });
  }
  for(auto &n : g->nodes) have.push_back({ (int64_t)n.name, (int64_t)n.kernel, (int64_t)n.wd, (int64_t)n.ht, (int64_t)n.dp });
  std::sort(want.begin(), want.end());
  std::sort(have.begin(), have.end());
  if(want != have)
  {
    g->nodes_ready = false;
    return fail(VKDT_CUDA_INCOMPLETE, "the library's plan (%zu nodes) does not cover the given %zu nodes", have.size(), want.size());
  }
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_graph_node(vkdt_cuda_graph_t *g, int i, vkdt_cuda_node_info_t *info)
{
  if(!g || !info || i < 0 || i >= (int)g->nodes.size()) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "node %d", i);
  *info = g->nodes[i];
  return 0;
}
int vkdt_cuda_graph_output_size(vkdt_cuda_graph_t *g, int *wd, int *ht)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  if(wd) *wd = g->out_w;
  if(ht) *ht = g->out_h;
  return 0;
}

// the pinned staging buffers are made on first use: graphs that only develop
// device buffers (vkdt_cuda_graph_develop, the server) never hold them
static void *staging(void **p, size_t bytes)
{
  if(!*p && cudaMallocHost(p, bytes) != cudaSuccess) { *p = nullptr; fail(VKDT_CUDA_ERROR_OUT_OF_HOST_MEMORY, "pinned staging of %zu bytes", bytes); }
  return *p;
}
void *vkdt_cuda_graph_map_source(vkdt_cuda_graph_t *g, size_t *bytes)
{
  if(!g || !g->allocated) return nullptr;
  if(bytes) *bytes = g->src_bytes;
  return staging(&g->h_src, g->src_bytes);
}
void *vkdt_cuda_graph_map_sink(vkdt_cuda_graph_t *g, size_t *bytes)
{
  if(!g || !g->allocated) return nullptr;
  if(bytes) *bytes = g->sink_bytes;
  return staging(&g->h_sink, g->sink_bytes);
}
int vkdt_cuda_graph_device_buffers(vkdt_cuda_graph_t *g, void **d_source, void **d_sink)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  if(d_source) *d_source = g->arena + g->off_src;
  if(d_sink) *d_sink = g->arena + g->off_out;
  return 0;
}

// The launch sequence runs as a CUDA graph: captured once and replayed while nothing changes.
// New buffers or per-image values (another image of the same shape: white balance, black and
// white, noise) capture the sequence again and update the executable graph in place (its
// topology is the plan's, so only kernel parameters change); a graph that cannot be updated
// is instantiated anew.
static int run_kernels(vkdt_cuda_graph_t *g, cudaStream_t s, const void *src, void *dst)
{
  if(plan_key(g) != g->planned_for)
    return fail(VKDT_CUDA_INCOMPLETE, "sizes or node-changing parameters differ from the last vkdt_cuda_graph_alloc: allocate again");
  if(g->timing || !g->use_graph) return enqueue(g, s, src, dst, g->timing);
  if(g->graph_dirty || !g->gexec || src != g->gsrc || dst != g->gdst)
  {
    CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int r = enqueue(g, s, src, dst, false);
    cudaGraph_t cap = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s, &cap);
    if(r) { if(cap) cudaGraphDestroy(cap); return r; }
    CU(e);
    if(g->gexec)
    {
      cudaGraphExecUpdateResultInfo info;
      if(cudaGraphExecUpdate(g->gexec, cap, &info) != cudaSuccess)
      {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(g->gexec);
        g->gexec = nullptr;
      }
    }
    cudaError_t ie = g->gexec ? cudaSuccess : cudaGraphInstantiate(&g->gexec, cap, 0);
    cudaGraphDestroy(cap);
    CU(ie);
    g->gsrc = src; g->gdst = dst;
    g->graph_dirty = false;
  }
  CU(cudaGraphLaunch(g->gexec, s));
  return 0;
}

int vkdt_cuda_graph_run(vkdt_cuda_graph_t *g, void *stream, uint32_t flags)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  if((flags & VKDT_CUDA_RUN_UPLOAD_SOURCE) && !staging(&g->h_src, g->src_bytes)) return VKDT_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  if((flags & VKDT_CUDA_RUN_DOWNLOAD_SINK) && !staging(&g->h_sink, g->sink_bytes)) return VKDT_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  if(flags & VKDT_CUDA_RUN_UPLOAD_SOURCE)
    CU(cudaMemcpyAsync(g->arena + g->off_src, g->h_src, g->src_bytes, cudaMemcpyHostToDevice, s));
  if(g->timing) CU(cudaEventRecord(g->ev[0], s));
  int r = run_kernels(g, s, g->arena + g->off_src, g->arena + g->off_out);
  if(r) return r;
  if(flags & VKDT_CUDA_RUN_DOWNLOAD_SINK)
    CU(cudaMemcpyAsync(g->h_sink, g->arena + g->off_out, g->sink_bytes, cudaMemcpyDeviceToHost, s));
  CU(cudaEventRecord(g->done, s));
  if(flags & VKDT_CUDA_RUN_WAIT_DONE) return vkdt_cuda_graph_wait(g, 600000);
  return 0;
}

int vkdt_cuda_graph_set_capture(vkdt_cuda_graph_t *g, int enable)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  g->use_graph = enable != 0;
  return 0;
}

void *vkdt_cuda_graph_stream(vkdt_cuda_graph_t *g)
{
  return g ? (void *)g->stream : nullptr;
}

int vkdt_cuda_graph_develop(vkdt_cuda_graph_t *g, const void *d_mosaic, void *d_rgba, void *stream)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  if(!d_mosaic || !d_rgba) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null device buffer");
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  int r = run_kernels(g, s, d_mosaic, d_rgba);
  if(r) return r;
  CU(cudaEventRecord(g->done, s));
  return 0;
}

// Callers that may not allocate device memory when they develop (a display
// or video callback beside busy streams, where cudaMalloc/cudaFree can
// synchronise the device; an embedding that owns every allocation) get the
// same kernel sequence on a fixed scratch array instead of the graph's arena.
int vkdt_cuda_graph_develop_static(vkdt_cuda_graph_t *g, const void *d_mosaic, void *d_rgba, void *stream)
{
  if(!g) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null graph");
  if(g_device < 0) return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "vkdt_cuda_init was not called");
  if(g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph owns device buffers: use vkdt_cuda_graph_develop");
  if(!g->nodes_ready) return fail(VKDT_CUDA_INCOMPLETE, "call vkdt_cuda_graph_create_nodes first");
  if(g->debug || g->timing || g->want_hist || g->wavelet || g->unfused)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED,
                "debug stages, timing, the histogram, the wavelet denoise, x-trans and reduced sizes need an allocated graph");
  if(!d_mosaic || !d_rgba) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null device buffer");
  // a graph changed since create_nodes (size, crop, CFA, output size, denoise, demosaic, depth)
  // would run a stale plan on buffers the caller sized for the new one
  if(plan_key(g) != g->nodes_for) return fail(VKDT_CUDA_INCOMPLETE, "graph changed since vkdt_cuda_graph_create_nodes");
  // the arena plan of vkdt_cuda_graph_alloc without the caller's source, sink and debug buffers
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off = align_up(off + bytes); return o; };
  for(auto &l : g->hr) l.off = take((size_t)l.w * l.h * 8);
  for(auto &l : g->hb) l.off = take((size_t)l.w * l.h * 8);
  g->off_rgbf = take((size_t)g->W * g->H * 8);
  for(auto &l : g->lp) l.off = take((size_t)l.pitch * l.h * 2 * 11);
  for(auto &l : g->la) l.off = take((size_t)l.pitch * l.h * 2);
  g->off_hist = take(257 * 4);
  g->off_lut = take(65536 * 2);
  if(off > VKDT_CUDA_STATIC_SCRATCH_BYTES)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED,
                "%dx%d needs %zu bytes of scratch, the static scratch holds %u: use an allocated graph",
                g->W, g->H, off, VKDT_CUDA_STATIC_SCRATCH_BYTES);
  int dev = -1;
  CU(cudaGetDevice(&dev));
  if(dev < 0 || dev >= 64) return fail(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "device %d out of range", dev);
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> guard(g_static_lock);
    if(!g_static_base[dev])
    {
      void *p = nullptr;
      const cudaError_t e = static_scratch_address(&p);
      if(e != cudaSuccess || !p)
        return fail(e != cudaSuccess ? cuda_code(e) : VKDT_CUDA_ERROR_INITIALIZATION_FAILED,
                    "no address for the static scratch on device %d: %s", dev, cudaGetErrorString(e));
      g_static_base[dev] = p;
    }
    base = (unsigned char *)g_static_base[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  CU(cudaMemsetAsync(base, 0, off, s));
  CU(launch_noop_lut((__half *)(base + g->off_lut), g->nblack[0], g->nwhite[0], s));
  // the kernels address the scratch for this call only; the table just built is the one
  // enqueue would build, so it is marked as current (and the graph's own marks restored)
  const float keep_black = g->lut_black, keep_white = g->lut_white;
  g->lut_black = g->nblack[0]; g->lut_white = g->nwhite[0];
  g->arena = base;
  const int r = enqueue(g, s, d_mosaic, d_rgba, false);
  g->arena = nullptr;
  g->lut_black = keep_black; g->lut_white = keep_white;
  return r;
}

int vkdt_cuda_graph_wait(vkdt_cuda_graph_t *g, uint32_t timeout_ms)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  const auto t0 = std::chrono::steady_clock::now();
  int spin = 0;
  while(true)
  {
    const cudaError_t e = cudaEventQuery(g->done);
    if(e == cudaSuccess) break;
    if(e != cudaErrorNotReady) return fail(cuda_code(e), "device error: %s", cudaGetErrorString(e));
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if(ms > timeout_ms) return fail(VKDT_CUDA_TIMEOUT, "wait timed out after %u ms", timeout_ms);
    if(++spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  if(take_device_status() & 1u) return fail(VKDT_CUDA_TIMEOUT, "a TMA copy of the llap reduce did not complete in its bounded wait");
  if(g->timing)
  {
    for(size_t i = 0; i < g->launches.size(); i++)
    {
      float ms = 0.0f;
      CU(cudaEventElapsedTime(&ms, g->ev[i], g->ev[i + 1]));
      g->times[i] = ms;
    }
  }
  return 0;
}

int vkdt_cuda_graph_query_times(vkdt_cuda_graph_t *g, float *ms, dt_token_t *names, dt_token_t *kernels, int max)
{
  if(!g || !g->allocated) return 0;
  const int n = (int)g->launches.size();
  for(int i = 0; i < n && i < max; i++)
  {
    if(ms) ms[i] = g->times[i];
    if(names) names[i] = g->launches[i].name;
    if(kernels) kernels[i] = g->launches[i].kernel;
  }
  return n;
}

int vkdt_cuda_graph_hist(vkdt_cuda_graph_t *g, uint32_t *hist257)
{
  if(!g || !g->allocated || !g->want_hist) return fail(VKDT_CUDA_INCOMPLETE, "histogram not enabled");
  CU(cudaMemcpy(hist257, g->arena + g->off_hist, 257 * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int vkdt_cuda_hist_rgba_f16(const void *d_rgba, int wd, int ht, uint32_t *d_hist, void *stream)
{
  if(!d_rgba || !d_hist || wd <= 0 || ht <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad histogram arguments");
  CU(launch_hist_rgba((const half4 *)d_rgba, wd, ht, d_hist, (cudaStream_t)stream));
  return 0;
}

int vkdt_cuda_waveform_rgba_f16(const void *d_rgba, int wd, int ht, uint32_t *d_out, int out_wd, int out_ht, void *stream)
{
  if(!d_rgba || !d_out || wd <= 0 || ht <= 0 || out_wd <= 0 || out_ht <= 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad waveform arguments");
  if(((uintptr_t)d_rgba & 7) || ((uintptr_t)d_out & 3))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "waveform: unaligned buffer");
  CU(launch_waveform((const half4 *)d_rgba, wd, ht, d_out, out_wd, out_ht, (cudaStream_t)stream));
  return 0;
}

int vkdt_cuda_lens_rgba_f16(const void *d_in, int wd, int ht, void *d_out, int out_wd, int out_ht,
    const float params[8], void *stream)
{
  if(!d_in || !d_out || !params || wd <= 0 || ht <= 0 || out_wd <= 0 || out_ht <= 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad lens arguments");
  if(((uintptr_t)d_in & 7) || ((uintptr_t)d_out & 7))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "lens: unaligned buffer");
  lens_par_t q;
  memcpy(&q, params, sizeof(q));
  CU(launch_lens((const half4 *)d_in, wd, ht, (half4 *)d_out, out_wd, out_ht, q, (cudaStream_t)stream));
  return 0;
}

int vkdt_cuda_graph_debug_stage_size(vkdt_cuda_graph_t *g, int stage, int *wd, int *ht, int *channels)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  int w, h, c = 4;
  if(stage == 0 || stage == 1) { w = g->W; h = g->H; c = 1; }
  else if(stage == 3) { w = g->dm_w; h = g->dm_h; }
  else if(stage == 2 || stage == 4 || stage == 11) { w = g->out_w; h = g->out_h; }
  else if(stage >= 5 && stage <= 10) { w = g->hw; h = g->hh; }
  else return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "stage %d", stage);
  if(wd) *wd = w;
  if(ht) *ht = h;
  if(channels) *channels = c;
  return 0;
}

int vkdt_cuda_graph_debug_stage(vkdt_cuda_graph_t *g, int stage, float *out, size_t count)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  CU(cudaStreamSynchronize(g->stream));
  const size_t npx = (size_t)g->W * g->H, nout = (size_t)g->out_w * g->out_h;
  if(stage == 0 || stage == 1)
  {
    if(!g->debug) return fail(VKDT_CUDA_INCOMPLETE, "debug stages not enabled");
    if(count < npx) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "buffer too small");
    std::vector<__half> h(npx);
    // the per-node chain keeps both images; the fused kernel writes debug copies
    const size_t off = g->unfused ? (stage == 0 ? g->off_dn : g->off_hl) : (stage == 0 ? g->off_dbg0 : g->off_dbg1);
    CU(cudaMemcpy(h.data(), g->arena + off, npx * 2, cudaMemcpyDeviceToHost));
    for(size_t i = 0; i < npx; i++) out[i] = __half2float(h[i]);
    return 0;
  }
  if(stage >= 5 && stage <= 10)
  { // the wavelet denoise's half size images: half, downcov, down 1..3 (swizzled as the reference stores them), assemble
    if(!g->debug || !g->wavelet) return fail(VKDT_CUDA_INCOMPLETE, "no wavelet denoise debug stages");
    const size_t nh = (size_t)g->hw * g->hh;
    if(count < nh * 4) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "buffer too small");
    const size_t off = stage == 5 ? g->off_dnh : stage == 10 ? g->off_dna : g->off_dnl[stage - 6];
    std::vector<__half> h(nh * 4);
    CU(cudaMemcpy(h.data(), g->arena + off, nh * 8, cudaMemcpyDeviceToHost));
    for(size_t i = 0; i < nh * 4; i++) out[i] = __half2float(h[i]);
    return 0;
  }
  if(stage == 2 || stage == 3 || stage == 4 || stage == 11)
  {
    if(stage != 2 && !g->debug) return fail(VKDT_CUDA_INCOMPLETE, "debug stages not enabled");
    if(stage == 11 && !g->crop_stage) return fail(VKDT_CUDA_INCOMPLETE, "no crop stage in this graph");
    if(stage == 11 && g->crop_shift)
    { // the kernel after demosaic reads the window of its output: that window, alpha 1
      if(count < nout * 4) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "buffer too small");
      std::vector<__half> h((size_t)g->dm_w * g->dm_h * 4);
      CU(cudaMemcpy(h.data(), g->arena + (g->unfused ? g->off_dm : g->off_dbg_dm), h.size() * 2, cudaMemcpyDeviceToHost));
      for(int y = 0; y < g->out_h; y++) for(int x = 0; x < g->out_w; x++)
      {
        const size_t i = (size_t)y * g->out_w + x, j = (size_t)(y + g->crop_dy) * g->dm_w + x + g->crop_dx;
        for(int k = 0; k < 3; k++) out[4 * i + k] = __half2float(h[4 * j + k]);
        out[4 * i + 3] = 1.0f;
      }
      return 0;
    }
    const size_t n = stage == 3 ? (size_t)g->dm_w * g->dm_h : nout;
    if(count < n * 4) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "buffer too small");
    std::vector<__half> h(n * 4);
    // the per-node chain keeps the demosaic and crop outputs; the fused kernel and rcd_fill write debug copies
    const size_t off = stage == 2 ? g->off_rgbf : stage == 4 ? g->off_dbg_col : stage == 11 ? g->off_cr
                     : (g->unfused ? g->off_dm : g->off_dbg_dm);
    CU(cudaMemcpy(h.data(), g->arena + off, n * 8, cudaMemcpyDeviceToHost));
    for(size_t i = 0; i < n * 4; i++) out[i] = __half2float(h[i]);
    return 0;
  }
  return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "stage %d", stage);
}

int vkdt_cuda_graph_debug_decisions(vkdt_cuda_graph_t *g, int kind, void *out, size_t bytes, int *wd, int *ht)
{
  if(!g || !g->allocated) return fail(VKDT_CUDA_INCOMPLETE, "graph not allocated");
  if(!g->debug) return fail(VKDT_CUDA_INCOMPLETE, "debug stages not enabled");
  size_t off, esz;
  if(kind == 0)
  { // demosaic/gauss entries: the fused bayer kernel and the x-trans gauss node write them
    if(g->halfsize || g->rcd) return fail(VKDT_CUDA_INCOMPLETE, "no demosaic/gauss in this graph");
    off = g->off_dbg_gauss; esz = 1;
  }
  else if(kind == 1 || kind == 2)
  {
    if(!g->wavelet) return fail(VKDT_CUDA_INCOMPLETE, "no wavelet denoise in this graph");
    off = kind == 1 ? g->off_dbg_cov : g->off_dbg_thr; esz = kind == 1 ? 4 : 1;
  }
  else return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "decision kind %d", kind);
  if(wd) *wd = g->hw;
  if(ht) *ht = g->hh;
  const size_t n = (size_t)g->hw * g->hh * esz;
  if(!out) return 0;
  if(bytes < n) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "buffer too small");
  CU(cudaStreamSynchronize(g->stream));
  CU(cudaMemcpy(out, g->arena + off, n, cudaMemcpyDeviceToHost));
  return 0;
}

// ---------------------------------------------------------------- noise statistics

int vkdt_cuda_unpack_mlv(const void *d_packed, size_t bytes, int bits_per_pixel, int wd, int ht, void *d_mosaic,
                         void *stream)
{
  if(bits_per_pixel != 10 && bits_per_pixel != 12 && bits_per_pixel != 14 && bits_per_pixel != 16)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "unpack_mlv: %d bits per pixel", bits_per_pixel);
  if(!d_packed || !d_mosaic || wd <= 0 || ht <= 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "unpack_mlv: null buffer or empty frame");
  if(((uintptr_t)d_packed & 1) || ((uintptr_t)d_mosaic & 1))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "unpack_mlv: buffers must be 16-bit aligned");
  const size_t npix = (size_t)wd * ht;
  if(bytes < npix * (size_t)bits_per_pixel / 8)   // video_mlv.c:213 raw_frame_size
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "unpack_mlv: %zu bytes for %zu samples of %d bits", bytes, npix, bits_per_pixel);
  CU(launch_unpack_mlv(d_packed, bytes, bits_per_pixel, npix, (uint16_t *)d_mosaic, (cudaStream_t)stream));
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_colenc(const void *d_rgba_f16, int wd, int ht, int primaries, int trc, void *d_out_f16, void *d_out_u8,
                     void *stream)
{
  // colenc/main.comp:23-36 (matrices.h, row major): rec2020 to the output primaries
  static const double M_p3d65[9] = { 1.34353337, -0.28218904, -0.06142427, -0.06530851, 1.07578268, -0.01048453, 0.00282971, -0.01961215, 1.01717851 };
  static const double M_adobe[9] = { 1.15194302, -0.09753232, -0.05448118, -0.12454585, 1.13290963, -0.00837122, -0.02253539, -0.04979918, 1.07275365 };
  static const double M_ap0[9] = { 6.68685575e-01, 1.51817679e-01, 1.77189677e-01, 4.49002044e-02, 8.62145497e-01, 1.01922441e-01, -2.66851927e-09, 2.78271109e-02, 1.05170358 };
  static const double M_ap1[9] = { 9.62918591e-01, 1.16137050e-02, 2.55863361e-02, 4.16800770e-04, 9.99378426e-01, -8.82457347e-05, 5.31123331e-03, 2.18655328e-02, 9.75907920e-01 };
  static const double M_redwg[9] = { 0.853263, 0.079695, 0.067042, 0.029375, 0.809195, 0.161430, 0.051575, 0.208097, 0.740329 };
  if(!d_rgba_f16 || wd <= 0 || ht <= 0 || (!d_out_f16 && !d_out_u8) || trc < 0 || trc > 6)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "colenc: null buffer, empty image or trc %d", trc);
  if(((uintptr_t)d_rgba_f16 & 7) || ((uintptr_t)d_out_f16 & 7) || ((uintptr_t)d_out_u8 & 3))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "colenc: unaligned buffer");
  const double *m = primaries == 1 ? M_rec2020_to_rec709 : primaries == 3 ? M_adobe : primaries == 4 ? M_p3d65
                  : primaries == 5 ? M_rec2020_to_xyz : primaries == 6 ? M_ap0 : primaries == 7 ? M_ap1
                  : primaries == 10 ? M_redwg : nullptr;
  float M[9];
  if(m) for(int i = 0; i < 9; i++) M[i] = (float)m[i];
  CU(launch_colenc(d_rgba_f16, wd, ht, m ? M : nullptr, trc, d_out_f16, d_out_u8, (cudaStream_t)stream));
  return VKDT_CUDA_SUCCESS;
}

int vkdt_cuda_bc1_encode(const void *d_rgba_u8, int wd, int ht, void *d_blocks, void *stream)
{
  if(!d_rgba_u8 || !d_blocks || wd <= 0 || ht <= 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bc1_encode: null buffer or empty image");
  if(((uintptr_t)d_rgba_u8 & 3) || ((uintptr_t)d_blocks & 7))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bc1_encode: unaligned buffer");
  CU(launch_bc1(d_rgba_u8, wd, ht, d_blocks, (cudaStream_t)stream));
  return VKDT_CUDA_SUCCESS;
}

size_t vkdt_cuda_mcraw_scratch_bytes(int rwd, int ht)
{
  return rwd > 0 && ht > 0 ? mcraw_scratch_bytes(rwd, ht) : 0;
}

int vkdt_cuda_mcraw_decode(const void *d_bitcnt, const void *d_refval, const void *d_data, size_t data_bytes,
                           int rwd, int ht, int ox, int oy, int wd, int hgt, void *d_mosaic, void *d_scratch,
                           void *stream)
{
  if(rwd <= 0 || ht <= 0 || rwd % 64 || ht % 4)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "mcraw_decode: encoded size %dx%d (width a multiple of 64, height of 4)", rwd, ht);
  if(!d_bitcnt || !d_refval || !d_data || !d_mosaic || !d_scratch || wd <= 0 || hgt <= 0 || ox < 0 || oy < 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "mcraw_decode: null buffer or empty output");
  if(((uintptr_t)d_refval & 1) || ((uintptr_t)d_mosaic & 1) || ((uintptr_t)d_scratch & 7))
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "mcraw_decode: unaligned buffer");
  CU(launch_mcraw_decode(d_bitcnt, d_refval, d_data, data_bytes, rwd, ht, ox, oy, wd, hgt, d_scratch,
                         (uint16_t *)d_mosaic, (cudaStream_t)stream));
  return VKDT_CUDA_SUCCESS;
}

size_t vkdt_cuda_rawhist_scratch_bytes(void) { return rawhist_scratch_bytes(); }

int vkdt_cuda_rawhist(const void *d_mosaic, int wd, int ht, const vkdt_cuda_img_param_t *ip, int bins,
    void *d_scratch, double *h_out, void *stream)
{
  if(!d_mosaic || !ip || !d_scratch || !h_out || wd <= 0 || ht <= 0)
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad rawhist arguments");
  if(bins <= 0 || bins > rawhist_max_bins())
    return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "rawhist bins %d outside 1..%d", bins, rawhist_max_bins());
  if(ip->filters == 0) return fail(VKDT_CUDA_INCOMPLETE, "rawhist needs a mosaic");
  dev_rawhist_t p;
  memset(&p, 0, sizeof(p));
  p.mosaic = (const uint16_t *)d_mosaic;
  p.wd = wd; p.ht = ht; p.pitch = wd;
  const int block = ip->filters == 9u ? 3 : 2;
  p.bw = wd / block; p.bh = ht / block;
  p.filters = ip->filters;
  // rawhist/main.c:17-28 commit_params: MAX(1, black[1]) and white[1] as uint, /65536 in the shader
  const uint32_t black = (uint32_t)std::max(1.0f, ip->black[1]), white = (uint32_t)ip->white[1];
  p.black = (float)black / 65536.0f;
  p.white = (float)white / 65536.0f;
  p.bins = bins;
  p.acc = (unsigned long long *)d_scratch;
  double *d_out = (double *)((unsigned char *)d_scratch + 3 * rawhist_max_bins() * sizeof(unsigned long long));
  cudaStream_t st = (cudaStream_t)stream;
  CU(launch_rawhist(p, d_out, st));
  CU(cudaMemcpyAsync(h_out, d_out, 3 * (size_t)bins * sizeof(double), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return 0;
}

int vkdt_cuda_nprof_fit(const double *h, int wd, float *a_out, float *b_out)
{ // nprof/main.c:82-198 write_sink: pairs of bins give line fits sigma^2 = a + b x;
  // a bin is kept once enough of its pairs give a, b > 0; the standard falls by 2x
  // per round (up to 7) until some bin is kept; then the count weighted regression
  if(!h || !a_out || !b_out || wd <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad nprof arguments");
  std::vector<int> valid;
  float a = 0.0f, b = 0.0f;
  for(int f = 0; f < 7; f++)
  {
    const double fk = 1.0 / std::pow(2.0, f);
    for(int i = 0; i < wd; i++)
    {
      int score = 0;
      for(int j = i + 1; j < wd * (0.8 - fk); j++)
      {
        double c = h[i];
        if(c < fk * 64) continue;
        double m1 = h[i + wd], m2 = h[i + 2 * wd];
        const double x1 = m1 / c, y1 = m2 / c - (m1 / c) * (m1 / c);
        c = h[j];
        if(c < fk * 64) continue;
        m1 = h[j + wd]; m2 = h[j + 2 * wd];
        const double x2 = m1 / c, y2 = m2 / c - (m1 / c) * (m1 / c);
        if(y1 <= 0 || y2 <= 0) continue;
        const double eb = (y2 - y1) / (x2 - x1);
        const double ea = y1 - x1 * eb;
        if(!(eb > 0.0)) continue;
        if(!(ea > 0.0)) continue;
        if(++score > fk * 32) { a = (float)ea; b = (float)eb; valid.push_back(i); break; }
      }
    }
    if(!valid.empty()) break;
  }
  double sx = 0.0, sx2 = 0.0, sy = 0.0, sxy = 0.0, cnt = 0.0;
  for(int i : valid)
  {
    const double c = h[i], m1 = h[i + wd], m2 = h[i + 2 * wd];
    const double x = m1 / c;
    const double y = std::max(0.0, m2 / c - m1 / c * m1 / c);
    cnt += c; sx += x * c; sx2 += x * x * c; sy += y * c; sxy += x * y * c;
  }
  const float denom = (float)(cnt * sx2 - sx * sx);
  if(std::fabs(denom) > 1e-10f)
  {
    b = (float)std::max(0.0, (cnt * sxy - sx * sy) / denom);
    a = (float)std::max(0.0, (sy * sx2 - sx * sxy) / denom);
  }
  if(valid.empty()) { a = 100.0f; b = 1.0f; }   // the reference's default when nothing fits
  *a_out = a; *b_out = b;
  return valid.empty() ? VKDT_CUDA_INCOMPLETE : 0;
}

// ---------------------------------------------------------------- scenes

static void scene_layout(const vkdt_cuda_scene_t *sc, scene_layout_t *s)
{
  scene_layout_make(s, sc->wd, sc->ht, sc->seed, sc->image_id, sc->filters, sc->black, sc->white, sc->noise_a,
                    sc->noise_b, sc->wb, sc->pan_x, sc->pan_y);
}

int vkdt_cuda_scene_generate(const vkdt_cuda_scene_t *sc, void *d_mosaic, void *stream)
{
  if(!sc || !d_mosaic || sc->wd <= 0 || sc->ht <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad scene");
  scene_layout_t s;
  scene_layout(sc, &s);
  cudaStream_t st = (cudaStream_t)stream;
  scene_layout_t *d = nullptr;
  CU(cudaMalloc((void **)&d, sizeof(s)));
  cudaError_t e = cudaMemcpyAsync(d, &s, sizeof(s), cudaMemcpyHostToDevice, st);
  if(e == cudaSuccess) e = launch_scene(d, s.wd, s.ht, (uint16_t *)d_mosaic, st);
  if(e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  CU(e);
  return 0;
}

int vkdt_cuda_scene_generate_host(const vkdt_cuda_scene_t *sc, uint16_t *mosaic)
{
  if(!sc || !mosaic || sc->wd <= 0 || sc->ht <= 0) return fail(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad scene");
  scene_layout_t s;
  scene_layout(sc, &s);
  const int nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for(int t = 0; t < nt; t++)
    th.emplace_back([&, t]() {
      for(int y = t; y < s.ht; y += nt) for(int x = 0; x < s.wd; x++) mosaic[(size_t)y * s.wd + x] = scene_pixel(&s, x, y);
    });
  for(auto &t : th) t.join();
  return 0;
}

} // extern "C"
#pragma GCC visibility pop
