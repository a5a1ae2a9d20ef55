// CPU oracle (test infrastructure only): restatement of the vkdt raw
// development shaders. See oracle.h for the rules of use.
//
// Conventions shared by every node below (the reference's sampler and storage
// semantics, src/qvk/qvk.c:596-611, src/pipe/graph-run-nodes-allocate.h:39-96):
// - texture()/textureLod() use LINEAR filtering with MIRRORED_REPEAT wrap and
//   normalised coordinates. At texel centres this is the texel itself, which
//   is how the restatement reads it (fetch_m). Elsewhere the sample position
//   is rounded to 8 sub-texel bits and the bilinear weights are then
//   evaluated in the arithmetic type (tex_bilinear).
//
// Pinned: at even sizes every stage of the float build is bit-identical to
// the reference's own GLSL shaders compiled for the CPU (oracle/glsl, run by
// oracle/glsl_ref.py), with and without the wavelet denoise.
// - texelFetch() has no wrap; out-of-range reads are undefined in the
//   reference and read as 0 here (fetch_z).
// - textureGather(.., 0) returns component 0 of the 2x2 quad in the order
//   (i0,j1) (i1,j1) (i1,j0) (i0,j0).
// - a one-channel image reads as (r, 0, 0, 1).
// - every imageStore to an f16 image rounds to IEEE half (RTNE).
// - min/max/clamp follow IEEE minNum/maxNum: a NaN operand yields the other
//   operand, as the min/max instructions of GPUs do.
// - R16_UNORM decodes as v/65535.
#include "oracle.h"
// the seeded synthetic scene of the benchmarks and tests (inputs, not the path)
#include "../vkdt_gb300/csrc/scene.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

namespace {

// ------------------------------------------------------------------ helpers

// Sensitivity runs: with a nonzero seed every f16 store rounds to one of the
// two neighbouring f16 values at random (a hash of the value and the seed)
// instead of to the nearest: a perturbation of at most one f16 step at every
// stored intermediate, in the manner of discrete stochastic arithmetic (J.
// Vignes, "A stochastic arithmetic for reliable scientific computation",
// Math. Comput. Simul. 35, 1993). How far such runs move a result measures
// how much precision the f16 storage of the path leaves it.
static uint32_t g_perturb = 0;

static inline uint32_t perturb_bit(double v)
{
  uint64_t x;
  memcpy(&x, &v, 8);
  x ^= (uint64_t)g_perturb * 0x9E3779B97F4A7C15ull;
  x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27; x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (uint32_t)(x & 1);
}

template<class T> static inline T f16r(T v)
{ // round to IEEE binary16, round to nearest even, and back
  if(std::isnan(v)) return v;
  if(g_perturb)
  { // stochastic rounding between the neighbouring f16 values (normal range; see g_perturb)
    const T a = std::fabs(v);
    if(a >= T(6.103515625e-05) && a < T(65504.0))
    {
      int e;
      const T f = std::frexp(a, &e);
      const T x = std::ldexp(f, 11), lo = std::floor(x);
      const T m = (x == lo) ? lo : lo + T(perturb_bit((double)v));
      return std::copysign(std::ldexp(m, e - 11), v);
    }
  }
  T a = std::fabs(v);
  if(std::isinf(a)) return v;
  if(a >= T(65520.0)) return std::copysign(T(INFINITY), v);
  if(a < T(6.103515625e-05))
  { // subnormal half: integer multiples of 2^-24
    T m = std::nearbyint(std::ldexp(a, 24));
    return std::copysign(std::ldexp(m, -24), v);
  }
  int e;
  T f = std::frexp(a, &e);           // a = f * 2^e, f in [0.5, 1)
  T m = std::nearbyint(std::ldexp(f, 11)); // 11 significant bits
  return std::copysign(std::ldexp(m, e - 11), v);
}

template<class T> static inline T gmax(T a, T b) { return std::fmax(a, b); }
template<class T> static inline T gmin(T a, T b) { return std::fmin(a, b); }
template<class T> static inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template<class T> static inline T gmix(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template<class T> static inline T gsign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }
template<class T> static inline T smoothstep(T e0, T e1, T x)
{
  T t = gclamp((x - e0) / (e1 - e0), T(0), T(1));
  return t * t * (T(3) - T(2) * t);
}
template<class T> static inline T lum2020(T r, T g, T b)
{ // shared.glsl:150-154 luminance_rec2020
  return T(2.62700212e-01) * r + T(6.77998072e-01) * g + T(5.93017165e-02) * b;
}

static inline int mirror(int i, int n)
{ // VK_SAMPLER_ADDRESS_MODE_MIRRORED_REPEAT
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  return t < n ? t : m - 1 - t;
}

template<class T> struct img_t
{
  int w = 0, h = 0, c = 0;
  std::vector<T> d;
  img_t() {}
  img_t(int w_, int h_, int c_) : w(w_), h(h_), c(c_), d((size_t)w_ * h_ * c_, T(0)) {}
  T *px(int x, int y) { return d.data() + ((size_t)y * w + x) * c; }
  const T *px(int x, int y) const { return d.data() + ((size_t)y * w + x) * c; }
  T ch(int x, int y, int k) const
  { // channel read with the (r,0,0,1) rule of one-channel formats
    if(k < c) return px(x, y)[k];
    return k == 3 ? T(1) : T(0);
  }
  void store(int x, int y, const T *v, int n)
  { // imageStore into an f16 image
    T *p = px(x, y);
    for(int k = 0; k < c && k < n; k++) p[k] = f16r(v[k]);
  }
};

// texelFetch: no wrap, undefined out of range -> 0
template<class T> static inline T fetch_z(const img_t<T> &im, int x, int y, int k)
{
  if(x < 0 || y < 0 || x >= im.w || y >= im.h) return T(0);
  return im.ch(x, y, k);
}
// texture() at a texel centre: mirrored texel
template<class T> static inline T fetch_m(const img_t<T> &im, int x, int y, int k)
{
  return im.ch(mirror(x, im.w), mirror(y, im.h), k);
}
// texture() anywhere: x,y are texel-space coordinates (normalised * size).
// Vulkan samplers on the GPUs the reference runs on resolve the sample
// position to 8 sub-texel bits (VkPhysicalDeviceLimits::subTexelPrecisionBits)
// before the bilinear weights are formed, so the position is rounded to 1/256.
template<class T> static inline T subtexel(T v) { return std::floor(v * T(256) + T(0.5)) / T(256); }
template<class T> static inline void tex_bilinear(const img_t<T> &im, T x, T y, T out[4])
{
  const T xs = subtexel(x - T(0.5)), ys = subtexel(y - T(0.5));
  const T fx = std::floor(xs), fy = std::floor(ys);
  const int x0 = (int)fx, y0 = (int)fy;
  const T ax = xs - fx, ay = ys - fy;
  const int X0 = mirror(x0, im.w), X1 = mirror(x0 + 1, im.w);
  const int Y0 = mirror(y0, im.h), Y1 = mirror(y0 + 1, im.h);
  for(int k = 0; k < 4; k++)
  {
    const T t00 = im.ch(X0, Y0, k), t10 = im.ch(X1, Y0, k);
    const T t01 = im.ch(X0, Y1, k), t11 = im.ch(X1, Y1, k);
    out[k] = (t00 * (T(1) - ax) + t10 * ax) * (T(1) - ay) + (t01 * (T(1) - ax) + t11 * ax) * ay;
  }
}

// CFA colour index (0 r, 1 g, 2 b) of an absolute mosaic position.
// bayer: demosaic/splat.comp:197-222 (rggb at 0,0); x-trans: splat.comp:167-195.
static inline int cfa_bayer(int x, int y)
{
  const int ox = x & 1, oy = y & 1;
  if((ox == 0 && oy == 1) || (ox == 1 && oy == 0)) return 1;
  if(ox == 0 && oy == 0) return 0;
  return 2;
}
static inline int cfa_xtrans(int x, int y)
{ // expects non-negative coordinates (callers add the 6 px margin)
  const bool blue_top = ((x / 3 + y / 3) & 1) > 0;
  const int px = x - (x / 3) * 3, py = y - (y / 3) * 3;
  if(((px + py) & 1) == 0) return 1;
  if(blue_top ^ (py == 1)) return 2;
  return 0;
}

// shared.glsl:244-293 evd2x2 (after christoph peters). M = (m00, m10, m11)
template<class T> static inline void evd2x2(T eval[2], T evec0[2], T evec1[2], T a, T b, T c)
{
  const T pHalf = T(-0.5) * (a + c);
  const T q = a * c - b * b;
  const T dr = std::sqrt(pHalf * pHalf - q);
  eval[0] = -pHalf + dr;
  eval[1] = -pHalf - dr;
  const T a0 = a - eval[0], b0 = b, c0 = c - eval[0];
  const T sl0 = a0 * a0 + b0 * b0;
  const T sl1 = b0 * b0 + c0 * c0;
  T sl;
  if(sl0 > sl1) { evec1[0] = a0; evec1[1] = b0; sl = sl0; }
  else          { evec1[0] = b0; evec1[1] = c0; sl = sl1; }
  evec1[0] = (sl == T(0)) ? T(1) : evec1[0];
  sl = (sl == T(0)) ? T(1) : sl;
  const T inv = T(1) / std::sqrt(sl);
  evec1[0] *= inv;
  evec1[1] *= inv;
  evec0[0] = evec1[1];
  evec0[1] = -evec1[0];
}

// ------------------------------------------------------------------ colour matrices (src/pipe/modules/matrices.h, row major)
static const double M_cat16_Mi[9] = { 1.86206786, -1.01125463,  0.14918677, 0.38752654,  0.62144744, -0.00897398, -0.01584150, -0.03412294,  1.04996444 };
static const double M_cat16_M[9]  = { 0.401288, 0.650173, -0.051461, -0.250268, 1.204414,  0.045854, -0.002079, 0.048952,  0.953127 };
static const double M_rec2020_to_xyz[9] = { 0.636958048301290991, 0.144616903586208406, 0.168880975164172054, 0.26270021201126692, 0.677998071518871148, 0.0593017164698619384, 4.9999999999999999e-17, 0.0280726930490874452, 1.06098505771079066 };
static const double M_xyz_to_rec2020[9] = { 1.71665119, -0.35567078, -0.25336628, -0.66668435,  1.61648124,  0.01576855, 0.01763986, -0.04277061, 0.94210312 };
static const double M_rec709_to_rec2020[9] = { 0.62750375, 0.32927542, 0.04330266, 0.06910828, 0.91951916, 0.0113596, 0.01639406, 0.08801125, 0.89538035 };
static const double M_rec2020_to_rec709[9] = { 1.66022677, -0.58754761, -0.07283825, -0.12455334,  1.13292605, -0.00834963, -0.01815514, -0.10060303,  1.11899817 };
static const double M_rec709_to_yuv[9] = { 0.299, 0.587, 0.114, -0.147, -0.289, 0.436, 0.615, -0.515, -0.100 };
static const double M_yuv_to_rec709[9] = { 1.0, -3.94570707e-05, 1.13982797, 1.0, -3.94610164e-01, -5.80500316e-01, 1.0, 2.03199968, -4.81376263e-04 };

template<class T> struct m3 { T m[9]; };
template<class T> static m3<T> m3_load(const double *a) { m3<T> r; for(int i = 0; i < 9; i++) r.m[i] = T(a[i]); return r; }
template<class T> static m3<T> m3_mul(const m3<T> &A, const m3<T> &B)
{ // glsl A*B with column-major storage evaluates the same sums as row-major A*B
  m3<T> r;
  for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)
    r.m[3 * i + j] = A.m[3 * i + 0] * B.m[0 + j] + A.m[3 * i + 1] * B.m[3 + j] + A.m[3 * i + 2] * B.m[6 + j];
  return r;
}
template<class T> static inline void m3_apply(const m3<T> &A, const T v[3], T o[3])
{ // glsl mat3*vec3: col0*v.x + col1*v.y + col2*v.z
  T r[3];
  for(int i = 0; i < 3; i++) r[i] = A.m[3 * i + 0] * v[0] + A.m[3 * i + 1] * v[1] + A.m[3 * i + 2] * v[2];
  o[0] = r[0]; o[1] = r[1]; o[2] = r[2];
}

// ------------------------------------------------------------------ decisions
// the decision record/force context of the current develop call (one at a time)
static oracle_decisions_t *g_dec = nullptr;

template<class T> static inline float rel_gap(T a, T b)
{
  const T m = gmax(std::fabs(a), std::fabs(b));
  return m > T(0) ? (float)(std::fabs(a - b) / m) : 0.0f;
}

// the stage a develop call starts from, with the given input image (node-wise
// checks: a stage of the path on another implementation's input). 0: the mosaic.
static struct { int start; const float *img; } g_inj = { 0, nullptr };

template<class T> static img_t<T> from_float(const float *src, int w, int h, int c)
{ // values already stored by an f16 image: taken as they are
  img_t<T> im(w, h, c);
  for(size_t i = 0; i < im.d.size(); i++) im.d[i] = T(src[i]);
  return im;
}

// ------------------------------------------------------------------ denoise

// denoise/noop.comp:36-57 (gain map absent on the synthetic input)
template<class T> static img_t<T> denoise_noop(const img_t<T> &in, int wd, int ht,
    const int crop[4], const T black[4], const T white[4])
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T col[4];
    for(int k = 0; k < 3; k++)
      col[k] = gmax(T(0), (fetch_z(in, x + crop[0], y + crop[1], k) - black[k]) / (white[k] - black[k]));
    col[3] = T(1);
    out.store(x, y, col, 4);
  }
  return out;
}

// denoise/noise.glsl:1-11 (edges applied per channel)
template<class T> static inline void noise_sigma(T out[3], T na, T nb, T black, T white, const T edges[4], T val)
{
  const T s = std::sqrt(na + gmax(T(0), (val - black) / (white - black)) * nb);
  for(int k = 0; k < 3; k++)
    out[k] = gclamp(std::exp2(T(12) * edges[k] + edges[3]) * s, T(1e-3), T(1e3));
}

// denoise/half.comp:24-74
template<class T> static img_t<T> denoise_half(const img_t<T> &in, int wd, int ht,
    const int crop[4], T white_g, uint32_t filters)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgba[4];
    if(filters == 9)
    {
      const int bx = crop[0] + 3 * x, by = crop[1] + 3 * y;
      T c[9];
      for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) c[3 * i + j] = fetch_z(in, bx + i, by + j, 0);
      const T c0 = (c[1] + c[7]) * T(0.5), c1 = (c[3] + c[5]) * T(0.5);
      if(((x + y + crop[0] + crop[1]) & 1) > 0) { rgba[0] = c0; rgba[2] = c1; }
      else                                      { rgba[2] = c0; rgba[0] = c1; }
      rgba[1] = (c[0] + c[2] + c[4] + c[6] + c[8]) * T(1.0) / T(5.0);
      rgba[3] = T(1);
    }
    else
    {
      const int i0 = crop[0] + 2 * x, j0 = crop[1] + 2 * y;
      T cx = fetch_m(in, i0, j0 + 1, 0), cy = fetch_m(in, i0 + 1, j0 + 1, 0);
      T cz = fetch_m(in, i0 + 1, j0, 0), cw = fetch_m(in, i0, j0, 0);
      if(cx >= white_g) cx = cz;
      if(cz >= white_g) cz = cx;
      rgba[0] = cw; rgba[1] = (cx + cz) / T(2); rgba[2] = cy; rgba[3] = T(1);
    }
    out.store(x, y, rgba, 4);
  }
  return out;
}

// denoise/cov.glsl:159-276 response(). p in texel coordinates of img.
template<class T> static void denoise_response(const img_t<T> &img, int px_, int py_, T res_out[3], T cov[4], size_t idx)
{
  T mw[2] = {0, 0}, mb[2] = {0, 0}, smw = 0, smb = 0, mean_b = 0;
  T Sw00 = 0, Sw01 = 0, Sw10 = 0, Sw11 = 0, Sb00 = 0, Sb01 = 0, Sb10 = 0, Sb11 = 0, sw = 0, sb = 0;
  const T w = T(1);
  for(int j = -2; j <= 2; j++) for(int i = -2; i <= 2; i++)
  {
    const T px = lum2020(fetch_m(img, px_ + i, py_ + j, 0), fetch_m(img, px_ + i, py_ + j, 1), fetch_m(img, px_ + i, py_ + j, 2));
    const T p[2] = { T(i), T(j) };
    mw[0] += p[0] * px * w; mw[1] += p[1] * px * w;
    smw += px * w;
    mb[0] += p[0] / px * w; mb[1] += p[1] / px * w;
    smb += T(1) / px * w;
  }
  mw[0] /= smw; mw[1] /= smw;
  mb[0] /= smb; mb[1] /= smb;
  for(int j = -2; j <= 2; j++) for(int i = -2; i <= 2; i++)
  {
    const T px = lum2020(fetch_m(img, px_ + i, py_ + j, 0), fetch_m(img, px_ + i, py_ + j, 1), fetch_m(img, px_ + i, py_ + j, 2));
    mean_b += px / T(25);
    T p2 = px * px * w;
    T p[2] = { T(i) - mw[0], T(j) - mw[1] };
    Sw00 += p2 * p[0] * p[0]; Sw01 += p2 * p[0] * p[1]; Sw10 += p2 * p[1] * p[0]; Sw11 += p2 * p[1] * p[1];
    sw += p2;
    p[0] = T(i) - mb[0]; p[1] = T(j) - mb[1];
    p2 = T(1) / (px * px) * w;
    Sb00 += p2 * p[0] * p[0]; Sb01 += p2 * p[0] * p[1]; Sb10 += p2 * p[1] * p[0]; Sb11 += p2 * p[1] * p[1];
    sb += p2;
  }
  Sw00 /= sw; Sw01 /= sw; Sw10 /= sw; Sw11 /= sw;
  Sb00 /= sb; Sb01 /= sb; Sb10 /= sb; Sb11 /= sb;
  const T detw = Sw00 * Sw11 - Sw10 * Sw01, detb = Sb00 * Sb11 - Sb10 * Sb01;
  bool usew = detw < detb;
  // the hot pixel skips this texel takes (decision record, oracle_decisions_t)
  uint32_t skip = 0;
  float hot_gap = 1e30f;
  for(int j = -2; j <= 2; j++) for(int i = -2; i <= 2; i++)
  {
    const T pr = fetch_m(img, px_ + i, py_ + j, 0);
    if(pr > T(2) * mean_b) skip |= 1u << ((i + 2) + 5 * (j + 2));
    hot_gap = std::min(hot_gap, rel_gap(pr, T(2) * mean_b));
  }
  if(g_dec && g_dec->dn_cov) g_dec->dn_cov[idx] = skip | (usew ? 1u << 25 : 0u);
  if(g_dec && g_dec->dn_cov_margin) { g_dec->dn_cov_margin[2 * idx] = rel_gap(detw, detb); g_dec->dn_cov_margin[2 * idx + 1] = hot_gap; }
  if(g_dec && g_dec->dn_cov_force) { usew = (g_dec->dn_cov_force[idx] >> 25) & 1; skip = g_dec->dn_cov_force[idx] & 0x1ffffffu; }
  T eval[2], evec0[2], evec1[2];
  if(usew) evd2x2(eval, evec0, evec1, Sw00, Sw10, Sw11);
  else     evd2x2(eval, evec0, evec1, Sb00, Sb10, Sb11);
  eval[0] *= T(1.0); eval[1] *= T(0.05);
  eval[0] = gclamp(eval[0], T(0.01), T(25)); eval[1] = gclamp(eval[1], T(0.01), T(25));
  cov[0] = eval[0]; cov[1] = eval[1]; cov[2] = evec0[0]; cov[3] = evec0[1];
  T res[3] = {0, 0, 0}, wt = 0;
  for(int j = -2; j <= 2; j++) for(int i = -2; i <= 2; i++)
  {
    const T pr = fetch_m(img, px_ + i, py_ + j, 0), pg = fetch_m(img, px_ + i, py_ + j, 1), pb = fetch_m(img, px_ + i, py_ + j, 2);
    if((skip >> ((i + 2) + 5 * (j + 2))) & 1) continue;   // pr > 2 mean_b (or the forced skip)
    const T x0 = T(i) * evec0[0] + T(j) * evec0[1];
    const T x1 = T(i) * evec1[0] + T(j) * evec1[1];
    const T ww = gmax(T(1e-9), std::exp(T(-0.5) * (x0 / eval[0] * x0 + x1 / eval[1] * x1)));
    res[0] += ww * pr; res[1] += ww * pg; res[2] += ww * pb;
    wt += ww;
  }
  const T d = gmax(wt, T(1e-8));
  res_out[0] = res[0] / d; res_out[1] = res[1] / d; res_out[2] = res[2] / d;
}

static inline void swz(int &x, int &y, int w, int h)
{ // denoise/down.comp:102-104 decimated write position
  const int ox = (x & 1) * (w + 1) / 2, oy = (y & 1) * (h + 1) / 2;
  x = x / 2 + ox; y = y / 2 + oy;
}

// denoise/downcov.comp:41-63
template<class T> static img_t<T> denoise_downcov(const img_t<T> &in, int wd, int ht, const int crop[4])
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgb[3], cov[4];
    denoise_response(in, x + crop[0], y + crop[1], rgb, cov, (size_t)y * wd + x);
    T edge = gclamp(T(75) * gmax(T(0), cov[1] - T(0.09)), T(0), T(1));
    edge = smoothstep(T(0.4), T(0.75), edge);
    edge = gclamp(T(0.02) + edge, T(0), T(1));
    int X = x, Y = y;
    swz(X, Y, wd, ht);
    const T v[4] = { rgb[0], rgb[1], rgb[2], edge };
    out.store(X, Y, v, 4);
  }
  return out;
}

// denoise/down.comp:59-108 (level >= 0 branch)
template<class T> static img_t<T> denoise_down(const img_t<T> &in, int wd, int ht, const int crop[4],
    T black_g, T white_g, T na, T nb, const T edges[4], int level, int block_i)
{
  img_t<T> out(wd, ht, 4);
  const T t = T(0.2);
  const T block = (block_i == 3) ? T(2.23607) : (block_i == 2 ? T(1.414213) : T(1.0));
  const T offs[4][2] = {
    { T(0.5) + T(1.2), T(0.5) + T(0.4) }, { T(0.5) - T(1.2), T(0.5) - T(0.4) },
    { T(0.5) + T(0.4), T(0.5) - T(1.2) }, { T(0.5) - T(0.4), T(0.5) + T(1.2) } };
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgb[3];
    for(int k = 0; k < 3; k++) rgb[k] = fetch_m(in, x + crop[0], y + crop[1], k);
    T sum[3], wgt[3];
    for(int k = 0; k < 3; k++) { sum[k] = t * rgb[k]; wgt[k] = t; }
    T ns[3];
    noise_sigma(ns, na, nb, black_g, white_g, edges, rgb[0]);
    const T pl = std::pow(T(0.7), T(level));
    T wc[3];
    for(int k = 0; k < 3; k++) { const T sigma = pl * ns[k] / block; wc[k] = T(1) / sigma; }
    for(int o = 0; o < 4; o++)
    {
      T col[4];
      tex_bilinear(in, T(x + crop[0]) + offs[o][0], T(y + crop[1]) + offs[o][1], col);
      for(int k = 0; k < 3; k++)
      {
        const T g0 = col[k] < T(0) ? col[k] : std::pow(col[k], T(0.8));
        const T g1 = rgb[k] < T(0) ? rgb[k] : std::pow(rgb[k], T(0.8));
        const T e = gclamp(T(1) - T(0.5) * (wc[k] * std::fabs(g0 - g1)), T(0), T(1));
        const T w = e * (T(1) - t) / T(4);
        sum[k] += w * col[k];
        wgt[k] += w;
      }
    }
    for(int k = 0; k < 3; k++) rgb[k] = sum[k] / wgt[k];
    int X = x, Y = y;
    swz(X, Y, wd, ht);
    const T v[4] = { rgb[0], rgb[1], rgb[2], T(1) };
    out.store(X, Y, v, 4);
  }
  return out;
}

// denoise/assemble.comp:151-273
template<class T> static img_t<T> denoise_assemble(const img_t<T> *s, int wd, int ht, const int crop[4],
    const T wb[4], const T black[4], const T white[4], T na, T nb, uint32_t filters,
    T strength, T luma, const T edges[4])
{
  img_t<T> out(wd, ht, 4);
  const m3<T> rgb_to_yuv = m3_mul(m3_load<T>(M_rec709_to_yuv), m3_load<T>(M_rec2020_to_rec709));
  const m3<T> yuv_to_rgb = m3_mul(m3_load<T>(M_rec709_to_rec2020), m3_load<T>(M_yuv_to_rec709));
  const int szx = s[1].w + 1, szy = s[1].h + 1;
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T orig[3], d[5][3];
    for(int k = 0; k < 3; k++) orig[k] = fetch_z(s[0], x + crop[0], y + crop[1], k);
    int ex = x, ey = y;
    for(int k = 0; k < 3; k++) d[0][k] = orig[k];
    T test;
    for(int l = 1; l <= 4; l++)
    {
      ex = ex / 2 + (ex & 1) * szx / 2;
      ey = ey / 2 + (ey & 1) * szy / 2;
      for(int k = 0; k < 3; k++) d[l][k] = fetch_z(s[l], ex, ey, k);
      if(l == 1) test = fetch_z(s[1], ex, ey, 3);
    }
    T sigma[3];
    noise_sigma(sigma, na, nb, black[1], white[1], edges, gmax(d[2][0], T(0)));
    const T block = filters == 0u ? T(1.0) : (filters == 9u ? T(2.23607) : T(1.414213));
    const T b[4] = { T(0.7000) / block, T(0.4900) / block, T(0.3430) / block, T(0.2401) / block };
    for(int l = 0; l < 4; l++) for(int k = 0; k < 3; k++) d[l][k] = (d[l][k] - d[l + 1][k]) / (sigma[k] * b[l]);
    T len[4];
    for(int l = 0; l < 4; l++) len[l] = std::sqrt(d[l][0] * d[l][0] + d[l][1] * d[l][1] + d[l][2] * d[l][2]);
    const T d0 = len[0], d1 = len[1], d2 = len[2], d3 = len[3];
    const T slope = ((d3 - d0) / T(3.0) + (d2 - d1) / T(1.0) + (d1 - d0) / T(1.0) + (d3 - d2) / T(1.0) + (d2 - d0) / T(2.0) + (d3 - d1) / T(2.0)) / T(6.0);
    test = gmax(T(0), -slope);
    test = gmax(T(0), T(1) - test);
    test = std::pow(test, T(16));
    test = gclamp(T(1.5) * test, T(0), T(1));
    const T thrs0 = std::pow(strength, T(4));
    const T ht_ = T(10);
    const size_t idx = (size_t)y * wd + x;
    uint32_t sw = 0;
    for(int l = 0; l < 4; l++)
    {
      if(std::fabs(d[l][0]) > ht_) sw |= 1u << l;
      if(g_dec && g_dec->dn_thr_margin) g_dec->dn_thr_margin[4 * idx + l] = rel_gap(std::fabs(d[l][0]), ht_);
    }
    if(g_dec && g_dec->dn_thr) g_dec->dn_thr[idx] = (uint8_t)sw;
    if(g_dec && g_dec->dn_thr_force) sw = g_dec->dn_thr_force[idx];
    for(int l = 3; l >= 0; l--)
    {
      const T thrs = ((sw >> l) & 1) ? T(10000) : thrs0;
      for(int k = 0; k < 3; k++)
      {
        const T a = std::fabs(d[l][k]);
        const T tt = gmin(T(1), a / (T(2) * thrs));
        d[4][k] += sigma[k] * b[l] * gsign(d[l][k]) * gmix(gmax(a - thrs, T(0)), a, tt);
      }
    }
    T v4[3], vo[3];
    for(int k = 0; k < 3; k++)
    {
      v4[k] = (d[4][k] - black[k]) / (white[k] - black[k]) * wb[k];
      vo[k] = (orig[k] - black[k]) / (white[k] - black[k]) * wb[k];
    }
    T yuv[3], yuvo[3];
    m3_apply(rgb_to_yuv, v4, yuv);
    m3_apply(rgb_to_yuv, vo, yuvo);
    yuv[0] = gmix(yuvo[0], yuv[0], luma);
    T rgb[3];
    m3_apply(yuv_to_rgb, yuv, rgb);
    T o[4];
    for(int k = 0; k < 3; k++) o[k] = rgb[k] / wb[k] * (white[k] - black[k]) + black[k];
    o[3] = test;
    out.store(x, y, o, 4);
  }
  return out;
}

// denoise/doub.comp:35-116 (gain map absent)
template<class T> static img_t<T> denoise_doub(const img_t<T> &orig, const img_t<T> &crs0, const img_t<T> &crs1,
    int wd, int ht, const int crop[4], const T black4[4], const T white4[4], uint32_t filters,
    T na, T nb, T strength, T luma, T detail, const T edges[4])
{
  img_t<T> out(wd, ht, 1);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T upsm[4], down[4];
    const T ux = (T(x) + T(0.5)) / T(wd), uy = (T(y) + T(0.5)) / T(ht);
    tex_bilinear(crs0, ux * T(crs0.w), uy * T(crs0.h), upsm);
    tex_bilinear(crs1, ux * T(crs1.w), uy * T(crs1.h), down);
    T black = black4[1], white = white4[1], crs = upsm[1], crs1v = down[1];
    T Tt = T(0.5) * strength * upsm[3], blendw = luma;
    int col;
    if(filters == 9) col = cfa_xtrans(x, y);
    else             col = cfa_bayer(x, y);
    if(col != 1)
    {
      black = black4[col]; white = white4[col];
      crs = upsm[col]; crs1v = down[col]; blendw = T(1);
      if(filters == 9) Tt /= gmax(T(1e-4), upsm[3]);
    }
    T sigma[3];
    noise_sigma(sigma, na, nb, black, white, edges, crs);
    T val = fetch_m(orig, x + crop[0], y + crop[1], 0);
    blendw = T(0.5) * (blendw + T(1));
    if(val < white)
    {
      const T wav = (val - crs1v) / gmax(sigma[0] + sigma[2], T(1e-8));
      const T tt = gmin(T(1), wav / gmax(T(2) * Tt, T(1e-8)));
      T uw = std::pow(gmin(T(1), T(1) * upsm[3]), T(4));
      uw = T(1) - (T(1) - uw) * detail;
      const T aw = std::fabs(wav);
      val = gmix(val, gmax(T(0), crs + sigma[1] * gsign(wav) * gmix(gmax(T(0), aw - Tt), aw, tt)), uw * blendw);
    }
    val = gmax(T(0), (val - black) / (white - black));
    const T v[1] = { val };
    out.store(x, y, v, 1);
  }
  return out;
}

// ------------------------------------------------------------------ hilite

// hilite/half.comp:21-72
template<class T> static img_t<T> hilite_half(const img_t<T> &in, int wd, int ht, T white, uint32_t filters)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgba[4];
    if(filters == 9)
    {
      T c[9];
      for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) c[3 * i + j] = fetch_z(in, 3 * x + i, 3 * y + j, 0);
      if(c[1] >= white) c[1] = c[7];
      if(c[7] >= white) c[7] = c[1];
      if(c[3] >= white) c[3] = c[5];
      if(c[5] >= white) c[5] = c[3];
      const T maxg = gmax(gmax(gmax(c[0], c[2]), c[4]), gmax(c[6], c[8]));
      if(maxg >= white) c[0] = c[2] = c[4] = c[6] = c[8] = T(1);
      const T c0 = (c[1] + c[7]) * T(0.5), c1 = (c[3] + c[5]) * T(0.5);
      if(((x + y) & 1) > 0) { rgba[0] = c0; rgba[2] = c1; }
      else                  { rgba[2] = c0; rgba[0] = c1; }
      rgba[1] = (c[0] + c[2] + c[4] + c[6] + c[8]) / T(5.0);
      rgba[3] = T(1);
    }
    else
    {
      T cx = fetch_m(in, 2 * x, 2 * y + 1, 0), cy = fetch_m(in, 2 * x + 1, 2 * y + 1, 0);
      T cz = fetch_m(in, 2 * x + 1, 2 * y, 0), cw = fetch_m(in, 2 * x, 2 * y, 0);
      if(cx >= white) cx = cz;
      if(cz >= white) cz = cx;
      rgba[0] = cw; rgba[1] = (cx + cz) / T(2); rgba[2] = cy; rgba[3] = T(1);
    }
    out.store(x, y, rgba, 4);
  }
  return out;
}

// hilite/reduce.comp:21-61
template<class T> static img_t<T> hilite_reduce(const img_t<T> &in, int wd, int ht, const T wb4[4], T white_p, T desat)
{
  img_t<T> out(wd, ht, 4);
  T white = white_p;
  if(!(white > T(0))) white = T(1);
  const T w[5] = { T(1.0) / T(16.0), T(4.0) / T(16.0), T(6.0) / T(16.0), T(4.0) / T(16.0), T(1.0) / T(16.0) };
  const T sw[5] = { T(1), T(2), T(0), T(-2), T(-1) };
  T wb[3] = { wb4[0], wb4[1], wb4[2] };
  if(!(wb[0] * wb[0] + wb[1] * wb[1] + wb[2] * wb[2] > T(1e-3))) wb[0] = wb[1] = wb[2] = T(1);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T edge[2] = {0, 0}, col[3] = {0, 0, 0}, wgt = 0;
    for(int jj = -2; jj <= 2; jj++) for(int ii = -2; ii <= 2; ii++)
    {
      T rgb[3];
      for(int k = 0; k < 3; k++) rgb[k] = fetch_m(in, 2 * x + ii, 2 * y + jj, k);
      const T l = lum2020(rgb[0], rgb[1], rgb[2]);
      edge[0] += w[jj + 2] * sw[ii + 2] * l;
      edge[1] += w[ii + 2] * sw[jj + 2] * l;
      const T u = w[ii + 2] * w[jj + 2];
      const T rw = rgb[0] * wb[0], gw = rgb[1] * wb[1], bw = rgb[2] * wb[2];
      const T cmax = gmax(rw, gmax(gw, bw));
      const T cmin = gmin(rw, gmin(gw, bw));
      const T sat = (cmax - cmin) / gmax(T(1e-3), cmax);
      if(rgb[0] < white && rgb[1] < white && rgb[2] < white)
      {
        const T s = smoothstep(T(0.2), T(1.0), gmax(rgb[0], gmax(rgb[1], rgb[2])) / white);
        T t = smoothstep(T(0.15), T(0.9), sat);
        const T ds = desat * desat;
        t = gclamp(T(5) * ds * ds * s * t, T(0), T(1));
        for(int k = 0; k < 3; k++)
        {
          rgb[k] = gmix(rgb[k], (cmax + cmin) / wb[k] * T(0.5), t);
          col[k] += rgb[k] * u;
        }
        wgt += u;
      }
    }
    T o[4];
    if(wgt == T(0)) { o[0] = o[1] = o[2] = T(1); }
    else for(int k = 0; k < 3; k++) o[k] = col[k] / wgt;
    o[3] = std::sqrt(edge[0] * edge[0] + edge[1] * edge[1]);
    out.store(x, y, o, 4);
  }
  return out;
}

// hilite/assemble.comp:23-81 gauss_expand
template<class T> static void hilite_expand(const img_t<T> &im, int ox, int oy, T c[3])
{
  const T w[5] = { T(1.0) / T(16.0), T(4.0) / T(16.0), T(6.0) / T(16.0), T(4.0) / T(16.0), T(1.0) / T(16.0) };
  c[0] = c[1] = c[2] = T(0);
  T wgt = T(0);
  const int ix = ox / 2, iy = oy / 2;
  const int d = (ox & 1) + 2 * (oy & 1);
  const int i0 = (d & 1) ? 0 : -1, j0 = (d & 2) ? 0 : -1;
  for(int ii = i0; ii <= 1; ii++) for(int jj = j0; jj <= 1; jj++)
  {
    const T wy = (d & 2) ? w[2 * jj + 1] : w[2 * jj + 2];
    const T wx = (d & 1) ? w[2 * ii + 1] : w[2 * ii + 2];
    for(int k = 0; k < 3; k++) c[k] += fetch_m(im, ix + ii, iy + jj, k) * wy * wx;
    wgt += wy * wx;
  }
  if(wgt == T(0)) { c[0] = 0; c[1] = 1; c[2] = 1; return; }
  for(int k = 0; k < 3; k++) c[k] /= wgt;
}

// hilite/assemble.comp:83-119
template<class T> static img_t<T> hilite_assemble(const img_t<T> &fine, const img_t<T> &coarse, int wd, int ht, T white, T soft)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T upsm[3];
    hilite_expand(coarse, x, y, upsm);
    T f[4];
    for(int k = 0; k < 4; k++) f[k] = fetch_z(fine, x, y, k);
    const T sr = f[0] / gmax(T(0.001), upsm[0]);
    const T sg = f[1] / gmax(T(0.001), upsm[1]);
    const T sb = f[2] / gmax(T(0.001), upsm[2]);
    const T wr = std::exp(upsm[0] - gmax(upsm[1], upsm[2]));
    const T wg = std::exp(upsm[1] - gmax(upsm[0], upsm[2]));
    const T wbb = std::exp(upsm[2] - gmax(upsm[0], upsm[1]));
    const T scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
    T rec[3];
    for(int k = 0; k < 3; k++) rec[k] = gclamp(upsm[k] * scale, T(-65535.0), T(65535.0));
    T t = soft;
    if(f[0] >= white || f[1] >= white || f[2] >= white) t = T(1);
    if(std::isnan(f[3])) f[3] = T(0);
    t = gclamp(gmix(t, T(1), std::sqrt(gmax(T(0), f[3]))), T(0), T(1));
    T o[4];
    for(int k = 0; k < 3; k++) o[k] = gmix(f[k], rec[k], t);
    o[3] = T(1);
    out.store(x, y, o, 4);
  }
  return out;
}

// hilite/doub.comp:141-241. out is the full mosaic.
template<class T> static void hilite_doub(const img_t<T> &in, const img_t<T> &coarse, int wd, int ht, T white,
    uint32_t filters, img_t<T> &out)
{
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T up[3];
    for(int k = 0; k < 3; k++) up[k] = fetch_z(coarse, x, y, k);
    if(filters == 9)
    {
      if(((x + y) & 1) == 0) std::swap(up[0], up[2]);
      T c[9];
      for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) c[3 * i + j] = fetch_z(in, 3 * x + i, 3 * y + j, 0);
      const T minr = gmin(c[1], c[7]), minb = gmin(c[3], c[5]);
      const T ming = gmin(gmin(gmin(c[0], c[2]), c[4]), gmin(c[6], c[8]));
      const T sr = minr / gmax(T(0.001), up[0]);
      const T sg = ming / gmax(T(0.001), up[1]);
      const T sb = minb / gmax(T(0.001), up[2]);
      const T wr = std::exp(up[0] - gmax(up[1], up[2]));
      const T wg = std::exp(up[1] - gmax(up[0], up[2]));
      const T wbb = std::exp(up[2] - gmax(up[0], up[1]));
      const T scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
      const T maxr = gmax(c[1], c[7]), maxb = gmax(c[3], c[5]);
      const T maxg = gmax(gmax(gmax(c[0], c[2]), c[4]), gmax(c[6], c[8]));
      const T softw = T(0.97) * white;
      const T maxrgb = gmax(maxr, gmax(maxg, maxb));
      if(maxrgb > softw)
      {
        T t = smoothstep(softw, white, maxrgb);
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
      for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++)
      {
        const int X = 3 * x + i, Y = 3 * y + j;
        if(X < out.w && Y < out.h) { const T v[1] = { c[3 * i + j] }; out.store(X, Y, v, 1); }
      }
    }
    else
    {
      T cx = fetch_m(in, 2 * x, 2 * y + 1, 0), cy = fetch_m(in, 2 * x + 1, 2 * y + 1, 0);
      T cz = fetch_m(in, 2 * x + 1, 2 * y, 0), cw = fetch_m(in, 2 * x, 2 * y, 0);
      const T ming = gmin(cx, cz);
      const T sr = cw / gmax(T(0.001), up[0]);
      const T sg = ming / gmax(T(0.001), up[1]);
      const T sb = cy / gmax(T(0.001), up[2]);
      const T wr = std::exp(up[0] - gmax(up[1], up[2]));
      const T wg = std::exp(up[1] - gmax(up[0], up[2]));
      const T wbb = std::exp(up[2] - gmax(up[0], up[1]));
      const T scale = (sr * wr + sg * wg + sb * wbb) / (wr + wg + wbb);
      const T softw = T(0.97) * white;
      const T maxrgb = gmax(gmax(cx, cy), gmax(cz, cw));
      if(maxrgb > softw)
      {
        const T t = smoothstep(softw, white, maxrgb);
        cx = gmix(cx, scale * up[1], t);
        cy = gmix(cy, scale * up[2], t);
        cz = gmix(cz, scale * up[1], t);
        cw = gmix(cw, scale * up[0], t);
      }
      const T vw[1] = { cw }, vz[1] = { cz }, vx[1] = { cx }, vy[1] = { cy };
      if(2 * x < out.w && 2 * y < out.h) out.store(2 * x, 2 * y, vw, 1);
      if(2 * x + 1 < out.w && 2 * y < out.h) out.store(2 * x + 1, 2 * y, vz, 1);
      if(2 * x < out.w && 2 * y + 1 < out.h) out.store(2 * x, 2 * y + 1, vx, 1);
      if(2 * x + 1 < out.w && 2 * y + 1 < out.h) out.store(2 * x + 1, 2 * y + 1, vy, 1);
    }
  }
}

// ------------------------------------------------------------------ demosaic

// demosaic/gauss.comp:19-126
template<class T> static img_t<T> demosaic_gauss(const img_t<T> &orig, int wd, int ht, uint32_t filters)
{
  img_t<T> out(wd, ht, 4);
  const int blk = filters == 9 ? 3 : 2;
  const int j0 = filters == 9 ? 0 : -1, j1 = filters == 9 ? 3 : 3;
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T mw[2] = {0, 0}, mb[2] = {0, 0}, smw = 0, smb = 0;
    T Sw00 = 0, Sw01 = 0, Sw10 = 0, Sw11 = 0, Sb00 = 0, Sb01 = 0, Sb10 = 0, Sb11 = 0, sw = 0, sb = 0;
    auto skip = [&](int i, int j) { return filters == 9 ? (((j + i) & 1) == 1) : (((j + i) & 1) != 1); };
    for(int j = j0; j < j1; j++) for(int i = j0; i < j1; i++)
    {
      if(skip(i, j)) continue;
      const T px = fetch_m(orig, blk * x + i, blk * y + j, 0);
      mw[0] += T(i) * px; mw[1] += T(j) * px;
      smw += px;
      mb[0] += T(i) / px; mb[1] += T(j) / px;
      smb += T(1) / px;
    }
    mw[0] /= smw; mw[1] /= smw;
    mb[0] /= smb; mb[1] /= smb;
    for(int j = j0; j < j1; j++) for(int i = j0; i < j1; i++)
    {
      if(skip(i, j)) continue;
      const T px = fetch_m(orig, blk * x + i, blk * y + j, 0);
      T p2 = px * px;
      T p[2] = { T(i) - mw[0], T(j) - mw[1] };
      Sw00 += p2 * p[0] * p[0]; Sw01 += p2 * p[0] * p[1]; Sw10 += p2 * p[1] * p[0]; Sw11 += p2 * p[1] * p[1];
      sw += p2;
      p[0] = T(i) - mb[0]; p[1] = T(j) - mb[1];
      p2 = T(1) / p2;
      Sb00 += p2 * p[0] * p[0]; Sb01 += p2 * p[0] * p[1]; Sb10 += p2 * p[1] * p[0]; Sb11 += p2 * p[1] * p[1];
      sb += p2;
    }
    Sw00 /= sw; Sw01 /= sw; Sw10 /= sw; Sw11 /= sw;
    Sb00 /= sb; Sb01 /= sb; Sb10 /= sb; Sb11 /= sb;
    const T detw = Sw00 * Sw11 - Sw10 * Sw01, detb = Sb00 * Sb11 - Sb10 * Sb01;
    // the form and the snapped direction (own decision, recorded with its margins;
    // a forced decision replaces both)
    auto snap_of = [&](const T e[2], float *gap) {
      const T ax = std::fabs(e[0]), ay = std::fabs(e[1]);
      if(filters != 9)
      {
        if(gap) *gap = (float)std::fabs(ax - ay);
        return ax > ay ? 0 : 1;
      }
      if(gap) *gap = (float)std::min(std::fabs(ax - T(2) * ay), std::fabs(ay - T(2) * ax));
      return ax > T(2) * ay ? 0 : (ay > T(2) * ax ? 1 : 2);
    };
    bool usew = detw < detb;
    T eval[2], evec0[2], evec1[2];
    if(usew) evd2x2(eval, evec0, evec1, Sw00, Sw10, Sw11);
    else     evd2x2(eval, evec0, evec1, Sb00, Sb10, Sb11);
    float snap_gap;
    int snap = snap_of(evec0, &snap_gap);
    const size_t idx = (size_t)y * wd + x;
    if(g_dec && g_dec->gauss) g_dec->gauss[idx] = (uint8_t)((usew ? 1 : 0) | (snap << 1));
    if(g_dec && g_dec->gauss_margin) { g_dec->gauss_margin[2 * idx] = rel_gap(detw, detb); g_dec->gauss_margin[2 * idx + 1] = snap_gap; }
    if(g_dec && g_dec->gauss_force)
    {
      const bool fw = g_dec->gauss_force[idx] & 1;
      if(fw != usew)
      {
        usew = fw;
        if(usew) evd2x2(eval, evec0, evec1, Sw00, Sw10, Sw11);
        else     evd2x2(eval, evec0, evec1, Sb00, Sb10, Sb11);
      }
      snap = (g_dec->gauss_force[idx] >> 1) & 3;
    }
    if(filters != 9)
    {
      eval[0] *= T(0.2); eval[1] *= T(0.2);
      if(snap == 0) { evec0[0] = 1; evec0[1] = 0; }
      else          { evec0[0] = 0; evec0[1] = 1; }
    }
    else
    {
      eval[0] *= T(0.4); eval[1] *= T(0.4);
      if(snap == 0)      { evec0[0] = 1; evec0[1] = 0; }
      else if(snap == 1) { evec0[0] = 0; evec0[1] = 1; }
      else { eval[0] = T(0.1); eval[1] = T(0.1); }
    }
    const T v[4] = { eval[0], eval[1], evec0[0], evec0[1] };
    out.store(x, y, v, 4);
  }
  return out;
}

// demosaic/splat.comp:142-266
template<class T> static img_t<T> demosaic_splat(const img_t<T> &in, const img_t<T> &gauss, int wd, int ht, uint32_t filters)
{
  img_t<T> out(wd, ht, 1);
  const int r = filters == 9 ? 2 : 1;
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T cov[4];
    for(int k = 0; k < 4; k++)
      cov[k] = filters == 9 ? fetch_z(gauss, x / 3, y / 3, k) : fetch_z(gauss, (x + 1) / 2, (y + 1) / 2, k);
    T rgb[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    for(int j = -r; j <= r; j++) for(int i = -r; i <= r; i++)
    {
      int px = x + i, py = y + j;
      if(px < 0) px += 6;
      if(py < 0) py += 6;
      if(px >= in.w) px -= 6;
      if(py >= in.h) py -= 6;
      const T col = fetch_z(in, px, py, 0);
      const T e0 = gclamp(cov[0], T(0.01), T(25)), e1 = gclamp(cov[1], T(0.01), T(25));
      const T of0 = cov[2] * T(i) + cov[3] * T(j);
      const T of1 = -cov[3] * T(i) + cov[2] * T(j);
      T weight = gclamp(std::exp(T(-0.5) * (of0 / e0 * of0 + of1 / e1 * of1)), T(1e-4), T(1.0));
      if(i == 0 && j == 0) weight = T(666.0);
      int c;
      if(filters == 9) c = cfa_xtrans(x + i + 6, y + j + 6);
      else             c = cfa_bayer(x + i, y + j);
      if(filters == 9) rgb[c] += col * weight;
      else             rgb[c] += col * weight;
      w[c] += weight;
    }
    const T g = rgb[1] / gmax(T(1e-8), w[1]);
    const T v[1] = { g };
    out.store(x, y, v, 1);
  }
  return out;
}

// demosaic/fix.comp:21-135
template<class T> static img_t<T> demosaic_fix(const img_t<T> &in, const img_t<T> &g, const img_t<T> &cov_img,
    int wd, int ht, uint32_t filters, int fixup)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgb[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    const T gc = fetch_m(g, x, y, 0);
    T cov[4];
    int r;
    T scale;
    if(filters == 9)
    {
      for(int k = 0; k < 4; k++) cov[k] = fetch_z(cov_img, (x + 1) / 3, (y + 1) / 3, k);
      cov[0] = gclamp(cov[0], T(1.), T(10.)); cov[1] = gclamp(cov[1], T(1.), T(10.));
      r = std::min(std::max(fixup + 2, 2), 3);
      scale = T(3);
    }
    else
    {
      for(int k = 0; k < 4; k++) cov[k] = fetch_z(cov_img, (x + 1) / 2, (y + 1) / 2, k);
      cov[0] = gclamp(cov[0], T(1.0), T(49)); cov[1] = gclamp(cov[1], T(1.0), T(49));
      r = std::min(std::max(fixup + 1, 1), 2);
      scale = T(2);
    }
    for(int j = -r; j <= r; j++) for(int i = -r; i <= r; i++)
    {
      const T gh = fetch_m(g, x + i, y + j, 0);
      const T col = fetch_m(in, x + i, y + j, 0);
      int c;
      if(filters == 9)
      { // write_xtrans2: the pattern is evaluated on the unshifted position
        const int px = x + i, py = y + j;
        const bool blue_top = ((px / 3 + py / 3) & 1) > 0;
        const int qx = px - (px / 3) * 3, qy = py - (py / 3) * 3;
        if(((qx + qy) & 1) == 0) c = 1;
        else if(blue_top ^ (qy == 1)) c = 2;
        else c = 0;
      }
      else c = cfa_bayer(x + i, y + j);
      if(c == 1) { rgb[1] = gc; w[1] = T(1); continue; }
      // eval_gauss(vec4(scale*cov.xy, cov.zw), (i,j))
      const T e0 = scale * cov[0], e1 = scale * cov[1];
      const T of0 = cov[2] * T(i) + cov[3] * T(j);
      const T of1 = -cov[3] * T(i) + cov[2] * T(j);
      const T weight = gclamp(std::exp(T(-0.5) * (of0 / e0 * of0 + of1 / e1 * of1)), T(1e-3), T(1.0));
      if(filters == 9)
      {
        const T corr = (T(1e-4) + gc) / (T(1e-4) + gh);
        rgb[c] += col * corr * weight;
      }
      else rgb[c] += col * (T(1e-4) + gc) / (T(1e-4) + gh) * weight;
      w[c] += weight;
    }
    T o[4];
    for(int k = 0; k < 3; k++) o[k] = rgb[k] / gmax(T(1e-8), w[k]);
    o[3] = T(1);
    out.store(x, y, o, 4);
  }
  return out;
}

// demosaic/halfsize.comp:155-187
template<class T> static img_t<T> demosaic_halfsize(const img_t<T> &in, int wd, int ht, uint32_t filters)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T rgba[4];
    if(filters == 9)
    {
      T c[9];
      for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) c[3 * i + j] = fetch_z(in, 3 * x + i, 3 * y + j, 0);
      rgba[1] = (c[0] + c[2] + c[4] + c[6] + c[8]) * T(1.0) / T(5.0);
      const T c0 = (c[1] + c[7]) * T(0.5), c1 = (c[3] + c[5]) * T(.5);
      if(((x + y) & 1) > 0) { rgba[0] = c0; rgba[2] = c1; }
      else                  { rgba[2] = c0; rgba[0] = c1; }
      rgba[3] = T(1); // not written by the shader: the f16 target holds whatever, use 1
    }
    else
    {
      const T cx = fetch_m(in, 2 * x, 2 * y + 1, 0), cy = fetch_m(in, 2 * x + 1, 2 * y + 1, 0);
      const T cz = fetch_m(in, 2 * x + 1, 2 * y, 0), cw = fetch_m(in, 2 * x, 2 * y, 0);
      rgba[0] = cw; rgba[1] = (cx + cz) / T(2); rgba[2] = cy; rgba[3] = T(1);
    }
    out.store(x, y, rgba, 4);
  }
  return out;
}

// shared/resample.comp:213-224 with shared.glsl:47-96 sample_catmull_rom
template<class T> static img_t<T> shared_resample(const img_t<T> &in, int wd, int ht)
{
  img_t<T> out(wd, ht, 4);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    const T sp[2] = { (T(x) + T(0.5)) / T(wd) * T(in.w), (T(y) + T(0.5)) / T(ht) * T(in.h) };
    T t0[2], t12[2], t3[2], w0[2], w12[2], w3[2];
    for(int k = 0; k < 2; k++)
    {
      const T tp1 = std::floor(sp[k] - T(0.5)) + T(0.5);
      const T f = sp[k] - tp1;
      w0[k] = f * (T(-0.5) + f * (T(1.0) - T(0.5) * f));
      const T w1 = T(1.0) + f * f * (T(-2.5) + T(1.5) * f);
      const T w2 = f * (T(0.5) + f * (T(2.0) - T(1.5) * f));
      w3[k] = f * f * (T(-0.5) + T(0.5) * f);
      w12[k] = w1 + w2;
      const T off12 = w2 / (w1 + w2);
      t0[k] = tp1 - T(1.0); t3[k] = tp1 + T(2.0); t12[k] = tp1 + off12;
    }
    const T *tx[3] = { &t0[0], &t12[0], &t3[0] }, *ty[3] = { &t0[1], &t12[1], &t3[1] };
    const T wx[3] = { w0[0], w12[0], w3[0] }, wy[3] = { w0[1], w12[1], w3[1] };
    T res[4] = {0, 0, 0, 0};
    for(int j = 0; j < 3; j++) for(int i = 0; i < 3; i++)
    {
      T v[4];
      tex_bilinear(in, *tx[i], *ty[j], v);
      for(int k = 0; k < 4; k++) res[k] += v[k] * wx[i] * wy[j];
    }
    out.store(x, y, res, 4);
  }
  return out;
}

// shared.glsl:47-96 sample_catmull_rom at normalised uv: nine bilinear taps,
// the positions divided back to normalised coordinates as the shader does
template<class T> static void catmull_rom_uv(const img_t<T> &in, T u, T v, T res[4])
{
  const T ts[2] = { T(in.w), T(in.h) };
  const T uv[2] = { u, v };
  T tp[3][2], w[3][2];
  for(int k = 0; k < 2; k++)
  {
    const T sp = uv[k] * ts[k];
    const T tp1 = std::floor(sp - T(0.5)) + T(0.5);
    const T f = sp - tp1;
    const T w0 = f * (T(-0.5) + f * (T(1.0) - T(0.5) * f));
    const T w1 = T(1.0) + f * f * (T(-2.5) + T(1.5) * f);
    const T w2 = f * (T(0.5) + f * (T(2.0) - T(1.5) * f));
    const T w3 = f * f * (T(-0.5) + T(0.5) * f);
    w[0][k] = w0; w[1][k] = w1 + w2; w[2][k] = w3;
    tp[0][k] = (tp1 - T(1.0)) / ts[k];
    tp[1][k] = (tp1 + w2 / (w1 + w2)) / ts[k];
    tp[2][k] = (tp1 + T(2.0)) / ts[k];
  }
  for(int c = 0; c < 4; c++) res[c] = T(0);
  for(int j = 0; j < 3; j++) for(int i = 0; i < 3; i++)
  {
    T t[4];
    tex_bilinear(in, tp[i][0] * ts[0], tp[j][1] * ts[1], t);
    for(int c = 0; c < 4; c++) res[c] += t[c] * w[i][0] * w[j][1];
  }
}

// ------------------------------------------------------------------ crop

// crop/main.comp:19-55. b is the committed block (crop/main.c:276-343): the
// homography H as three columns padded to four floats (b[0..11]), the
// rotation mat2(r0, r1, r2, r3) (b[12..15]) and the window x X y Y
// (b[16..19]). Per output pixel the input position is found by undoing the
// operations in reverse: the window's top left corner, the rotation about the
// input's centre, then H with the homogeneous divide. Matrix products sum
// their terms column by column, as GLSL's mat * vec. Outside [0,1)^2 the
// output is 0; without rotation (r0 == 1) the nearest texel is fetched,
// otherwise the Catmull-Rom filter samples. Alpha is stored as 1.
template<class T> static img_t<T> crop_main(const img_t<T> &in, const float *b, int wd, int ht)
{
  img_t<T> out(wd, ht, 4);
  const T tsx = T(in.w), tsy = T(in.h);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T px = T(x) + T(0.5), py = T(y) + T(0.5);
    px = px + T(b[16]) * tsx;
    py = py + T(b[18]) * tsy;
    const T vx = px - tsx * T(0.5), vy = py - tsy * T(0.5);
    px = (T(b[12]) * vx + T(b[14]) * vy) + tsx * T(0.5);
    py = (T(b[13]) * vx + T(b[15]) * vy) + tsy * T(0.5);
    const T hx = (T(b[0]) * px + T(b[4]) * py) + T(b[8]);
    const T hy = (T(b[1]) * px + T(b[5]) * py) + T(b[9]);
    const T hz = (T(b[2]) * px + T(b[6]) * py) + T(b[10]);
    const T rx = hx / hz / tsx, ry = hy / hz / tsy;
    T rgba[4] = { T(0), T(0), T(0), T(0) };
    // a position without value (hz = 0) is left undefined by the shader: 0 here
    if(!(rx >= T(0) && ry >= T(0) && rx < T(1) && ry < T(1))) {}
    else if(b[12] != 1.0f) catmull_rom_uv(in, rx, ry, rgba);
    else
    {
      const int ix = (int)(rx * tsx), iy = (int)(ry * tsy);
      for(int c = 0; c < 4; c++) rgba[c] = fetch_z(in, ix, iy, c);
    }
    rgba[3] = T(1);
    out.store(x, y, rgba, 4);
  }
  return out;
}

// core/gaussian_elimination.h:40-109 (gauss_solve, after H. Spaeth,
// "Numerik", 1994): Gaussian elimination with partial pivoting in the form of
// LINPACK's dgefa/dgesl. A is n x n row major. Column k's pivot is the first
// row of largest magnitude; the pivot row is swapped only right of column k,
// the multipliers (negated) stay where they were formed, and the right hand
// side is permuted step by step while it is reduced. The operations and their
// order are the reference's, so the solution is the same to the last bit.
// Returns false for a singular matrix (b untouched).
static bool solve_pivoted(double *A, double *b, int n)
{
  auto a = [&](int r, int c) -> double & { return A[r * n + c]; };
  int piv[16];
  for(int k = 0; k < n; k++)
  {
    int m = k;
    for(int r = k + 1; r < n; r++) if(std::fabs(a(r, k)) > std::fabs(a(m, k))) m = r;
    piv[k] = m;
    const double t = a(m, k);
    a(m, k) = a(k, k);
    a(k, k) = t;
    if(t == 0.0) return false;
    for(int r = k + 1; r < n; r++) a(r, k) /= -t;
    if(m != k) for(int c = k + 1; c < n; c++) std::swap(a(m, c), a(k, c));
    for(int r = k + 1; r < n; r++) for(int c = k + 1; c < n; c++) a(r, c) += a(r, k) * a(k, c);
  }
  for(int k = 0; k + 1 < n; k++)
  {
    std::swap(b[piv[k]], b[k]);
    const double t = b[k];
    for(int r = k + 1; r < n; r++) b[r] += a(r, k) * t;
  }
  for(int k = n - 1; k > 0; k--)
  {
    b[k] /= a(k, k);
    const double t = b[k];
    for(int r = 0; r < k; r++) b[r] -= a(r, k) * t;
  }
  b[0] /= a(0, 0);
  return true;
}

// crop/main.c:175-226 get_crop_rot: rotation 1337 takes the exif orientation
// (3: 180, 8: 90, 6: 270 degrees, else 0); the window 1,3,3,7 becomes a 3 px
// margin (none at 400 px or less), transposed for the quarter turns
static void crop_rot(uint32_t orient, double wd, double ht, const float pcrop[4], float prot, float crop[4], float *rot)
{
  *rot = prot;
  for(int k = 0; k < 4; k++) crop[k] = pcrop[k];
  if(prot == 1337.0f) *rot = orient == 3 ? 180.0f : orient == 8 ? 90.0f : orient == 6 ? 270.0f : 0.0f;
  if(crop[0] == 1.0 && crop[1] == 3.0 && crop[2] == 3.0 && crop[3] == 7.0)
  {
    const double mw = wd > 400 ? 3.0 / wd : 0.0, mh = ht > 400 ? 3.0 / ht : 0.0;
    const float r = *rot;
    const bool quarter = (r >= 45 && r < 135) || (r >= 225 && r < 315);
    if(quarter)
    {
      crop[0] = 0.5 - (.5 - mh) * ht / wd;
      crop[2] = 0.5 - (.5 - mw) * wd / ht;
      crop[1] = 0.5 + (.5 - mh) * ht / wd;
      crop[3] = 0.5 + (.5 - mw) * wd / ht;
    }
    else
    {
      crop[0] = mw; crop[2] = mh;
      crop[1] = 1.0 - mw; crop[3] = 1.0 - mh;
    }
  }
}

// ------------------------------------------------------------------ demosaic RCD (method 1)

// demosaic/rcd_conv.comp:8-49: per pixel the vertical/horizontal
// discriminator (vh, full size), per red/blue pixel the diagonal one (pq) and
// per green pixel the low pass of its red/blue neighbour (lp); pq and lp are
// half width images indexed by x/2. The mosaic is read through the sampler
// at texel centres (mirrored outside).
template<class T> static void rcd_conv(const img_t<T> &cfa, img_t<T> &vh, img_t<T> &pq, img_t<T> &lp)
{
  const int wd = cfa.w, ht = cfa.h;
  vh = img_t<T>(wd, ht, 1); pq = img_t<T>(wd / 2, ht, 1); lp = img_t<T>(wd / 2, ht, 1);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    auto c = [&](int i, int j) { return fetch_m(cfa, x + i, y + j, 0); };
    T s0 = T(0), s1 = T(0);
    for(int i = -1; i <= 1; i++)
    {
      s0 = s0 + (c(i, -3) - T(3) * c(i, -2) - c(i, -1) + T(6) * c(i, 0) - c(i, 1) - T(3) * c(i, 2) + c(i, 3));
      s1 = s1 + (c(-3, i) - T(3) * c(-2, i) - c(-1, i) + T(6) * c(0, i) - c(1, i) - T(3) * c(2, i) + c(3, i));
    }
    s0 = s0 * s0; s1 = s1 * s1;
    const T v = s0 / (T(1e-5f) + s0 + s1);
    vh.store(x, y, &v, 1);
    if(((x + y) & 1) == 0)
    { // red/blue pixel: diagonal discriminator
      T p0 = T(1e-5f), p1 = T(1e-5f);
      for(int i = -1; i <= 1; i++)
      {
        p0 = p0 + (c(-3 + i, -3 + i) - c(1 + i, -1 + i) - c(1 + i, 1 + i) + c(3 + i, 3 + i)
            - T(3) * (c(-2 + i, -2 + i) + c(2 + i, 2 + i)) + T(6) * c(i, i));
        p1 = p1 + (c(3 + i, -3 - i) - c(1 + i, -1 - i) - c(-1 + i, 1 - i) + c(-3 + i, 3 - i)
            - T(3) * (c(2 + i, -2 - i) + c(-2 + i, 2 - i)) + T(6) * c(i, -i));
      }
      p0 = p0 * p0; p1 = p1 * p1;
      const T q = p0 / (p0 + p1);
      pq.store(x / 2, y, &q, 1);
    }
    else
    { // green pixel: 3x3 low pass around the adjacent red/blue pixel of its row
      const int off = (x & 1) == 1 ? -1 : 1;
      const T w[3] = { T(0.5), T(1.0), T(0.5) };
      T l = T(0);
      for(int j = -1; j <= 1; j++) for(int i = -1; i <= 1; i++)
        l = l + w[j + 1] * w[i + 1] * c(i + off, j);
      l = gmax(T(1e-6f), l);
      lp.store(x / 2, y, &l, 1);
    }
  }
}

// demosaic/rcd_fill.comp:20-162 with the tile geometry of demosaic/config.h:
// one workgroup of 32x32 invocations per 64x32 tile, each invocation owns a
// horizontal pixel pair; tiles step by 58x26 (border 3) and only the inner
// 58x26 pixels are written. The tile lives in three f16 arrays indexed
// linearly (64 * row + column), so a neighbour offset past a tile edge wraps
// into the adjacent row; the reference's later two stages each read three
// pixels out while the border is three, so the invocations of tile rows 0-2
// and 29-31 index up to three rows outside the arrays. Those reads are
// undefined in the reference; here they read 0 (as does the CUDA kernel).
// The results that reach the written pixels never depend on the order of
// invocations within a stage.
static inline int rcd_col(int x, int y) { return ((x + y) & 1) == 1 ? 1 : ((y & 1) == 0 ? 0 : 2); }
template<class T> static img_t<T> rcd_fill(const img_t<T> &cfa, const img_t<T> &vh, const img_t<T> &pq,
    const img_t<T> &lp, const T wb[3])
{
  const int wd = cfa.w, ht = cfa.h;
  const int TX = 64, TY = 32, BD = 3, SX = TX - 2 * BD, SY = TY - 2 * BD, N = TX * TY;
  const int ntx = (wd + SX - 1) / SX, nty = (ht + SY - 1) / SY;
  const T eps = T(1e-5f);
  img_t<T> out(wd, ht, 4);
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
  for(int ty = 0; ty < nty; ty++) for(int tx = 0; tx < ntx; tx++)
  {
    std::vector<T> sh(3 * N);   // shm_r, shm_g, shm_b
    auto S = [&](int c, int i) -> T { return (i < 0 || i >= N) ? T(0) : sh[(size_t)c * N + i]; };
    auto Sw = [&](int c, int i, T v) { if(i >= 0 && i < N) sh[(size_t)c * N + i] = v; };
    auto hsub = [](T a, T b) { return f16r(a - b); };   // float16_t - float16_t
    for(int stage = 0; stage < 5; stage++)
      for(int ly = 0; ly < 32; ly++) for(int lx = 0; lx < 32; lx++)
      {
        const int ix = tx * SX + 2 * lx - BD, iy = ty * SY + ly - BD;   // ipos
        const int lidx = 2 * lx, lidy = ly;
        if(stage == 0)
        { // fill the tile from the mosaic (texelFetch: 0 outside), white balanced
          for(int k = 0; k < 2; k++)
          {
            const int c = rcd_col(ix + k, iy);
            const T v = gclamp(fetch_z(cfa, ix + k, iy, 0), T(0), T(65535));
            for(int ch = 0; ch < 3; ch++) Sw(ch, TX * lidy + lidx + k, c == ch ? f16r(wb[ch] * v) : T(0));
          }
          continue;
        }
        if(stage == 4)
        { // write the inner pixels
          for(int k = 0; k < 2; k++)
          {
            const int gx = ix + k, lxx = lidx + k;
            if(lxx >= BD && lidy >= BD && gx < wd && iy < ht && lxx < TX - BD && lidy < TY - BD)
            {
              const int i = TX * lidy + lxx;
              T o[4] = { S(0, i) / wb[0], S(1, i) / wb[1], S(2, i) / wb[2], T(1) };
              out.store(gx, iy, o, 4);
            }
          }
          continue;
        }
        // the pixel of the pair this stage works on: red/blue for stages 1, 2; green for 3
        const int rbk = rcd_col(ix, iy) == 1 ? 1 : 0;
        const int k = stage == 3 ? 1 - rbk : rbk;
        const int tcx = ix + k, tcy = iy;
        auto ind = [&](int dx, int dy) { return TX * (lidy + dy) + lidx + dx + k; };
        auto cf = [&](int dx, int dy) { return fetch_z(cfa, tcx + dx, tcy + dy, 0); };
        auto vhf = [&](int dx, int dy) { return fetch_m(vh, tcx + dx, tcy + dy, 0); };
        auto half_idx = [&](int dx, int dy) { return (tcx + dx + (((tcy + dy) & 1) == 1 ? 0 : 1)) / 2; };
        auto pqf = [&](int dx, int dy) { return fetch_m(pq, half_idx(dx, dy), tcy + dy, 0); };
        auto lpf = [&](int dx, int dy) { return fetch_m(lp, half_idx(dx, dy), tcy + dy, 0); };
        auto sg = [&](int dx, int dy) { return S(1, ind(dx, dy)); };
        if(stage == 1)
        { // green at red/blue pixels
          const T vhc = vhf(0, 0);
          const T vhn = T(0.25) * (vhf(-1, -1) + vhf(1, -1) + vhf(-1, 1) + vhf(1, 1));
          const T vhd = std::fabs(T(0.5) - vhc) < std::fabs(T(0.5) - vhn) ? vhn : vhc;
          const T Ng = eps + std::fabs(cf(0, -1) - cf(0, 1)) + std::fabs(cf(0, 0) - cf(0, -2))
                     + std::fabs(cf(0, -1) - cf(0, -3)) + std::fabs(cf(0, -2) - cf(0, -4));
          const T Sg = eps + std::fabs(cf(0, -1) - cf(0, 1)) + std::fabs(cf(0, 0) - cf(0, 2))
                     + std::fabs(cf(0, 1) - cf(0, 3)) + std::fabs(cf(0, 2) - cf(0, 4));
          const T Wg = eps + std::fabs(cf(-1, 0) - cf(1, 0)) + std::fabs(cf(0, 0) - cf(-2, 0))
                     + std::fabs(cf(-1, 0) - cf(-3, 0)) + std::fabs(cf(-2, 0) - cf(-4, 0));
          const T Eg = eps + std::fabs(cf(-1, 0) - cf(1, 0)) + std::fabs(cf(0, 0) - cf(2, 0))
                     + std::fabs(cf(1, 0) - cf(3, 0)) + std::fabs(cf(2, 0) - cf(4, 0));
          const T l0 = lpf(0, 0);
          const T Ne = cf(0, -1) * T(2) * l0 / (eps + l0 + lpf(0, -2));
          const T Se = cf(0, 1) * T(2) * l0 / (eps + l0 + lpf(0, 2));
          const T We = cf(-1, 0) * T(2) * l0 / (eps + l0 + lpf(-2, 0));
          const T Ee = cf(1, 0) * T(2) * l0 / (eps + l0 + lpf(2, 0));
          const T ve = gclamp((Sg * Ne + Ng * Se) / (Ng + Sg), T(0), T(65534));
          const T he = gclamp((Wg * Ee + Eg * We) / (Eg + Wg), T(0), T(65534));
          Sw(1, ind(0, 0), f16r(gmix(ve, he, vhd)));
        }
        else if(stage == 2)
        { // blue at red and red at blue pixels, along the diagonals
          const bool red = rcd_col(tcx, tcy) == 0;
          const int oc = red ? 2 : 0;
          auto sc = [&](int dx, int dy) { return S(oc, ind(dx, dy)); };
          const T pqc = pqf(0, 0);
          const T pqn = T(0.25) * (pqf(-1, -1) + pqf(1, -1) + pqf(-1, 1) + pqf(1, 1));
          const T pqd = std::fabs(T(0.5) - pqc) < std::fabs(T(0.5) - pqn) ? pqn : pqc;
          const T NWg = eps + std::fabs(hsub(sc(-1, -1), sc(1, 1))) + std::fabs(hsub(sc(-1, -1), sc(-3, -3))) + std::fabs(hsub(sg(0, 0), sg(-2, -2)));
          const T NEg = eps + std::fabs(hsub(sc(1, -1), sc(-1, 1))) + std::fabs(hsub(sc(1, -1), sc(3, -3))) + std::fabs(hsub(sg(0, 0), sg(2, -2)));
          const T SWg = eps + std::fabs(hsub(sc(1, -1), sc(-1, 1))) + std::fabs(hsub(sc(-1, 1), sc(-3, 3))) + std::fabs(hsub(sg(0, 0), sg(-2, 2)));
          const T SEg = eps + std::fabs(hsub(sc(-1, -1), sc(1, 1))) + std::fabs(hsub(sc(1, 1), sc(3, 3))) + std::fabs(hsub(sg(0, 0), sg(2, 2)));
          const T NWe = hsub(sc(-1, -1), sg(-1, -1)), NEe = hsub(sc(1, -1), sg(1, -1));
          const T SWe = hsub(sc(-1, 1), sg(-1, 1)), SEe = hsub(sc(1, 1), sg(1, 1));
          const T pe = (NWg * SEe + SEg * NWe) / (NWg + SEg);
          const T qe = (NEg * SWe + SWg * NEe) / (NEg + SWg);
          Sw(oc, ind(0, 0), f16r(gclamp(sg(0, 0) + gmix(pe, qe, pqd), T(0), T(65535))));
        }
        else
        { // red and blue at green pixels
          const T vhc = vhf(0, 0);
          const T vhn = T(0.25) * (vhf(-1, -1) + vhf(1, -1) + vhf(-1, 1) + vhf(1, 1));
          const T vhd = std::fabs(T(0.5) - vhc) < std::fabs(T(0.5) - vhn) ? vhn : vhc;
          const T N1 = eps + std::fabs(hsub(sg(0, 0), sg(0, -2)));
          const T S1 = eps + std::fabs(hsub(sg(0, 0), sg(0, 2)));
          const T W1 = eps + std::fabs(hsub(sg(0, 0), sg(-2, 0)));
          const T E1 = eps + std::fabs(hsub(sg(0, 0), sg(2, 0)));
          for(int c = 0; c < 2; c++)
          {
            const int oc = c == 0 ? 0 : 2;
            auto sc = [&](int dx, int dy) { return S(oc, ind(dx, dy)); };
            const T SN = std::fabs(hsub(sc(0, -1), sc(0, 1)));
            const T EW = std::fabs(hsub(sc(-1, 0), sc(1, 0)));
            const T Ng = N1 + SN + std::fabs(hsub(sc(0, -1), sc(0, -3)));
            const T Sg = S1 + SN + std::fabs(hsub(sc(0, 1), sc(0, 3)));
            const T Wg = W1 + EW + std::fabs(hsub(sc(-1, 0), sc(-3, 0)));
            const T Eg = E1 + EW + std::fabs(hsub(sc(1, 0), sc(3, 0)));
            const T Ne = hsub(sc(0, -1), sg(0, -1)), Se = hsub(sc(0, 1), sg(0, 1));
            const T We = hsub(sc(-1, 0), sg(-1, 0)), Ee = hsub(sc(1, 0), sg(1, 0));
            const T ve = (Ng * Se + Sg * Ne) / (Ng + Sg);
            const T he = (Eg * We + Wg * Ee) / (Eg + Wg);
            Sw(oc, ind(0, 0), f16r(gclamp(sg(0, 0) + gmix(ve, he, vhd), T(0), T(65535))));
          }
        }
      }
  }
  return out;
}

// ------------------------------------------------------------------ colour

// colour/main.c:219-292 commit_params (matrix path) + main-impl.glsl:200-341
template<class T> static img_t<T> colour_main(const img_t<T> &in, const oracle_img_param_t *ip, const oracle_params_t *p)
{
  // host side: p_wb from the camera coefficients when white = 0 (main.c:241-253)
  float p_wb[3] = { p->co_white[0], p->co_white[1], p->co_white[2] };
  if(p_wb[0] == 0.0f && p_wb[1] == 0.0f && p_wb[2] == 0.0f)
  {
    float w0[3] = {0}, w[] = { ip->whitebalance[0], ip->whitebalance[1], ip->whitebalance[2] };
    for(int j = 0; j < 3; j++) for(int i = 0; i < 3; i++) w0[j] += ip->cam_to_rec2020[3 * j + i] / w[i];
    w0[0] /= w0[1]; w0[2] /= w0[1]; w0[1] = 1.0f;
    p_wb[0] = 1 / w0[0]; p_wb[1] = 1; p_wb[2] = 1 / w0[2];
  }
  if(!(p_wb[0] == p_wb[0]) || p_wb[0] == 0.0f || p_wb[1] == 0.0f || p_wb[2] == 0.0f)
    p_wb[0] = p_wb[1] = p_wb[2] = 1.0f;
  const float mulf[4] = { p_wb[0] / p_wb[1], 1.0f, p_wb[2] / p_wb[1], powf(2.0f, p->co_exposure) };
  m3<T> cam;
  if(p->co_matrix == 1) for(int i = 0; i < 9; i++) cam.m[i] = T(ip->cam_to_rec2020[i]);
  else for(int i = 0; i < 9; i++) cam.m[i] = T(i % 4 == 0 ? 1 : 0);
  // cat16(rgb, vec3(1), mul.rgb): the matrix products fold at compile time
  const m3<T> P = m3_mul(m3_load<T>(M_cat16_M), m3_load<T>(M_rec2020_to_xyz));
  const m3<T> Q = m3_mul(m3_load<T>(M_xyz_to_rec2020), m3_load<T>(M_cat16_Mi));
  const T one[3] = { 1, 1, 1 }, mul3[3] = { T(mulf[0]), T(mulf[1]), T(mulf[2]) };
  T cl_src[3], cl_dst[3];
  m3_apply(P, one, cl_src);
  m3_apply(P, mul3, cl_dst);
  img_t<T> out(in.w, in.h, 4);
  OMP_FOR
  for(int y = 0; y < in.h; y++) for(int x = 0; x < in.w; x++)
  {
    T rgb[3];
    for(int k = 0; k < 3; k++) rgb[k] = fetch_m(in, x, y, k);
    m3_apply(cam, rgb, rgb);           // decode_colour: primaries custom, trc linear
    T cl[3];
    m3_apply(P, rgb, cl);
    for(int k = 0; k < 3; k++) cl[k] *= cl_dst[k] / cl_src[k];
    m3_apply(Q, cl, rgb);
    T o[4];
    for(int k = 0; k < 3; k++) o[k] = gclamp(rgb[k] * T(mulf[3]), T(-65535.0), T(65535.0));
    o[3] = T(1);
    out.store(x, y, o, 4);
  }
  return out;
}

// ------------------------------------------------------------------ filmcurv

template<class T> static inline T weibull_cdf(T x, T il, T k)
{ // filmcurv/params.glsl:15-34
  return T(1.0) - std::exp(-std::pow(gmax(x, T(1e-7)) * il, k));
}

// shared.glsl:371-387 adjust_colour_dng
template<class T> static void adjust_colour_dng(T c0[3], T c1[3])
{
  bool fx = false, fy = false, fz = false;
  if(c0[2] > c0[1]) { std::swap(c0[2], c0[1]); std::swap(c1[2], c1[1]); fx = true; }
  if(c0[1] > c0[0]) { std::swap(c0[0], c0[1]); std::swap(c1[0], c1[1]); fy = true; }
  if(c0[2] > c0[1]) { std::swap(c0[2], c0[1]); std::swap(c1[2], c1[1]); fz = true; }
  c1[1] = gmix(c1[2], c1[0], (c0[1] - c0[2] + T(1e-6)) / (c0[0] - c0[2] + T(1e-6)));
  if(fz) std::swap(c1[2], c1[1]);
  if(fy) std::swap(c1[0], c1[1]);
  if(fx) std::swap(c1[2], c1[1]);
}

// filmcurv/main.comp:106-205 (colour modes 1 and 3)
template<class T> static img_t<T> filmcurv_main(const img_t<T> &in, const oracle_params_t *p)
{
  img_t<T> out(in.w, in.h, 4);
  const T il = gmax(T(5e-3), T(p->fc_light));
  const T k = gmax(T(1e-4), T(p->fc_contrast));
  OMP_FOR
  for(int y = 0; y < in.h; y++) for(int x = 0; x < in.w; x++)
  {
    T c0[3], c1[3];
    for(int j = 0; j < 3; j++) c0[j] = fetch_z(in, x, y, j) + T(p->fc_bias);
    for(int j = 0; j < 3; j++) c1[j] = weibull_cdf(c0[j], il, k);
    if(p->fc_colour == 3) adjust_colour_dng(c0, c1);  // mode 1: per channel curve
    const T o[4] = { c1[0], c1[1], c1[2], T(1) };
    out.store(x, y, o, 4);
  }
  return out;
}

// ------------------------------------------------------------------ histogram

// natural logarithm used by the histogram bin index. the reference calls the
// GPU's log(); bin counts are integer results and must agree bit for bit
// between this oracle and the kernel, so both evaluate the same published
// method with the same operation order and no contraction:
// x = 2^e * m with m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
// log(m) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ... + s^13/13) (series of the
// inverse hyperbolic tangent, cf. Cody & Waite, "Software manual for the
// elementary functions", 1980, ch. 5), log(x) = e ln2 + log(m).
static float hist_log(float x)
{
  if(!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
  if(x == INFINITY) return INFINITY;
  uint32_t u; memcpy(&u, &x, 4);
  int e = (int)((u >> 23) & 0xff);
  if(e == 0) { x *= 8388608.0f; memcpy(&u, &x, 4); e = (int)((u >> 23) & 0xff) - 23; }
  e -= 127;
  u = (u & 0x007fffffu) | 0x3f800000u;
  float m; memcpy(&m, &u, 4);
  if(m > 1.41421356f) { m *= 0.5f; e += 1; }
  volatile float num = m - 1.0f, den = m + 1.0f;
  const float s = num / den;
  const float s2 = s * s;
  float poly = 1.0f / 13.0f;
  poly = poly * s2; poly = poly + 1.0f / 11.0f;
  poly = poly * s2; poly = poly + 1.0f / 9.0f;
  poly = poly * s2; poly = poly + 1.0f / 7.0f;
  poly = poly * s2; poly = poly + 1.0f / 5.0f;
  poly = poly * s2; poly = poly + 1.0f / 3.0f;
  poly = poly * s2; poly = poly + 1.0f;
  const float lm = 2.0f * s * poly;
  const float fe = (float)e;
  const float hi = fe * 0.693145752f;       // ln2 split: hi part exact in 16 bits
  const float lo = fe * 1.42860677e-06f;    // ln2 - hi
  return (hi + (lo + lm));
}

} // namespace

// rawhist/collect.comp:22-66 (test infrastructure). The sums are 64-bit fixed
// point (value * 2^36, rounded to nearest) and the bin uses hist_log / ln 2,
// like the kernel, so counts and sums reproduce exactly; out: 3*bins doubles.
extern "C" void oracle_rawhist(const uint16_t *mosaic, int wd, int ht, uint32_t filters, float black_dn,
    float white_dn, int bins, double *out)
{
  const uint32_t bi = (uint32_t)std::max(1.0f, black_dn), wi = (uint32_t)white_dn;   // rawhist/main.c:17-28
  const float black = (float)bi / 65536.0f, white = (float)wi / 65536.0f;
  std::vector<uint64_t> c(bins, 0), sm(bins, 0), s2(bins, 0);
  auto val = [&](int x, int y) {
    const float v = (x < wd && y < ht) ? (float)mosaic[(size_t)y * wd + x] / 65535.0f : 0.0f;
    const float t = (v - black) / (white - black);
    return std::fmin(std::fmax(t, 0.0f), 1.0f);
  };
  const int block = filters == 9u ? 3 : 2;
  for(int by = 0; by < ht / block; by++) for(int bx = 0; bx < wd / block; bx++)
  {
    float mean, mom2;
    if(filters == 9u)
    {
      const int x = 3 * bx, y = 3 * by;
      const float v0 = val(x, y), v1 = val(x + 2, y), v2 = val(x + 1, y + 1), v3 = val(x, y + 2), v4 = val(x + 2, y + 2);
      mean = ((((v0 + v1) + v2) + v3) + v4) / 5.0f;
      const float q0 = v0 * v0, q1 = v1 * v1, q2 = v2 * v2, q3 = v3 * v3, q4 = v4 * v4;
      mom2 = ((((q0 + q1) + q2) + q3) + q4) / 5.0f;
    }
    else
    {
      const int x = 2 * bx, y = 2 * by;
      const float v0 = val(x + 1, y), v1 = val(x, y + 1);
      mean = (v0 + v1) * 0.5f;
      const float q0 = v0 * v0, q1 = v1 * v1;
      mom2 = (q0 + q1) * 0.5f;
    }
    const float l = hist_log(mean + 1.0f) * 1.44269504f;
    const float xb = (float)bins * l;
    const int bin = (int)xb;
    if(bin < 0 || bin >= bins) continue;
    c[bin]++;
    sm[bin] += (uint64_t)std::nearbyint((double)mean * 68719476736.0);
    s2[bin] += (uint64_t)std::nearbyint((double)mom2 * 68719476736.0);
  }
  for(int i = 0; i < bins; i++)
  {
    out[i] = (double)c[i];
    out[bins + i] = (double)sm[i] / 68719476736.0;
    out[2 * bins + i] = (double)s2[i] / 68719476736.0;
  }
}

// i-mlv/video_mlv.c:254-274: an uncompressed magic lantern frame. Pixel i
// is read as the 32-bit little-endian word of the 16-bit words (i*bpp)/16
// and (i*bpp)/16 + 1, rotated right by 16 + (32 - bpp) - (i*bpp)%16 and
// masked to bpp bits. The rotation amount reaches 38; the shift pair the
// reference writes compiles to a rotate, whose amount counts modulo 32.
static inline uint32_t mlv_word(const uint8_t *p, size_t bytes, size_t w)
{
  return 2 * w + 1 < bytes ? (uint32_t)p[2 * w] | ((uint32_t)p[2 * w + 1] << 8) : 0u;
}
extern "C" void oracle_unpack_mlv(const uint8_t *packed, size_t bytes, int bpp, size_t npix, uint16_t *out)
{
  const uint32_t mask = bpp >= 32 ? 0xffffffffu : (1u << bpp) - 1u;
  for(size_t i = 0; i < npix; i++)
  {
    const uint64_t off = (uint64_t)i * (uint64_t)bpp;
    const size_t a = (size_t)(off / 16);
    const uint32_t sh = (uint32_t)(off % 16);
    const uint32_t r = (16u + (32u - (uint32_t)bpp) - sh) & 31u;
    const uint32_t u = mlv_word(packed, bytes, a) | (mlv_word(packed, bytes, a + 1) << 16);
    const uint32_t d = r ? (u >> r) | (u << (32 - r)) : u;
    out[i] = (uint16_t)(d & mask);
  }
}
// the inverse (test data): the bits unpack_mlv reads for each pixel, set from its value
extern "C" void oracle_pack_mlv(const uint16_t *in, size_t npix, int bpp, uint8_t *packed, size_t bytes)
{
  memset(packed, 0, bytes);
  for(size_t i = 0; i < npix; i++)
  {
    const uint64_t off = (uint64_t)i * (uint64_t)bpp;
    const size_t a = (size_t)(off / 16);
    const uint32_t r = (16u + (32u - (uint32_t)bpp) - (uint32_t)(off % 16)) & 31u;
    for(int k = 0; k < bpp; k++)
    {
      if(!((in[i] >> k) & 1)) continue;
      const uint32_t pos = (r + (uint32_t)k) & 31u;
      const size_t w = pos < 16 ? a : a + 1;
      const size_t byte = 2 * w + ((pos & 15) >> 3);
      if(byte < bytes) packed[byte] |= (uint8_t)(1u << (pos & 7));
    }
  }
}

// i-mcraw (motioncam raw video): blocks of 64 samples, each a reference
// value plus deltas of a bit width given by a 4-bit count per block.
// i-mcraw/prefix.comp:46-63: the bytes of a block by its bit count
static inline uint32_t mc_block_bytes(uint32_t cnt)
{
  switch(cnt)
  {
    case 0: return 0;
    case 1: return 8;
    case 2: return 16;
    case 3: return 24;
    case 4: return 32;
    case 5: return 40;
    case 6: return 48;
    case 7: case 8: return 64;
    case 9: case 10: return 80;
    default: return 128;
  }
}
static inline uint32_t mc_bits(uint32_t v, int off, int n) { return (v >> off) & ((1u << n) - 1u); }
// i-mcraw/decode.comp:31-282: the two deltas invocation si (0..31) of a block
// extracts from the block's bytes d, for each bit count
static void mc_decode_pair(uint32_t cnt, const uint8_t *d, int si, uint32_t r[2])
{
  auto pr = [&](int reg, uint32_t p[2]) { p[0] = d[reg]; p[1] = d[reg + 1]; };
  uint32_t p[2], q[2], t[2];
  switch(cnt)
  {
    case 0: r[0] = r[1] = 0; return;
    case 1:
      pr(2 * (si % 4), p);
      for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], si / 4, 1);
      return;
    case 2:
      pr(2 * (si % 8), p);
      for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 2 * (si / 8), 2);
      return;
    case 3:
    {
      int reg, off;
      if(si < 4)       { reg = 0 + si * 2; off = 0; }
      else if(si < 8)  { reg = 0 + (si - 4) * 2; off = 3; }
      else if(si < 12) { reg = 0 + (si - 8) * 2; off = 6; }
      else if(si < 16) { reg = 8 + (si - 12) * 2; off = 0; }
      else if(si < 20) { reg = 8 + (si - 16) * 2; off = 3; }
      else if(si < 24) { reg = 8 + (si - 20) * 2; off = 6; }
      else if(si < 28) { reg = 16 + (si - 24) * 2; off = 0; }
      else             { reg = 16 + (si - 28) * 2; off = 3; }
      pr(reg, p);
      for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], off, 3);
      if(si >= 8 && si < 12)
      {
        pr(16 + (si - 8) * 2, q);
        for(int c = 0; c < 2; c++) r[c] |= mc_bits(q[c], 6, 1) << 2;
      }
      else if(si >= 20 && si < 24)
      {
        pr(16 + (si - 20) * 2, q);
        for(int c = 0; c < 2; c++) r[c] |= mc_bits(q[c], 7, 1) << 2;
      }
      return;
    }
    case 4:
      pr((2 * si / 16) * 8 + (2 * si) % 8, p);
      for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], ((2 * si / 8) & 1) == 0 ? 0 : 4, 4);
      return;
    case 5:
      if(si < 20) { pr(2 * si, p); for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 0, 5); return; }
      if(si < 28)
      {
        pr(si < 24 ? 0 + (si - 20) * 2 : 8 + (si - 24) * 2, p);
        pr(si < 24 ? 24 + (si - 20) * 2 : 32 + (si - 24) * 2, q);
        for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 5, 3) | (mc_bits(q[c], 5, 2) << 3);
        return;
      }
      pr(16 + (si - 28) * 2, p); pr(24 + (si - 28) * 2, q); pr(32 + (si - 28) * 2, t);
      for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 5, 3) | (mc_bits(q[c], 7, 1) << 3) | (mc_bits(t[c], 7, 1) << 4);
      return;
    case 6:
      if(si < 24) { pr(2 * si, p); for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 0, 6); return; }
      {
        const int b = si < 28 ? 0 : 24, k = si < 28 ? si - 24 : si - 28;
        pr(b + k * 2, p); pr(b + 8 + k * 2, q); pr(b + 16 + k * 2, t);
        for(int c = 0; c < 2; c++) r[c] = mc_bits(p[c], 6, 2) | (mc_bits(q[c], 6, 2) << 2) | (mc_bits(t[c], 6, 2) << 4);
      }
      return;
    case 7: case 8:
      r[0] = d[2 * si]; r[1] = d[2 * si + 1];
      return;
    case 9: case 10:
    {
      pr(si < 16 ? 2 * si : 40 + (si - 16) * 2, p);
      pr(si < 16 ? 32 + (si % 4) * 2 : 72 + (si % 4) * 2, q);
      const int off = 2 * ((si & 15) / 4);
      for(int c = 0; c < 2; c++) r[c] = p[c] | (mc_bits(q[c], off, 2) << 8);
      return;
    }
    default:
      r[0] = (uint32_t)d[4 * si] | ((uint32_t)d[4 * si + 1] << 8);
      r[1] = (uint32_t)d[4 * si + 2] | ((uint32_t)d[4 * si + 3] << 8);
      return;
  }
}
// image position of sample c (0, 1) of invocation si of block idx (decode.comp:290-326):
// four consecutive blocks cover 64x4 pixels, each one CFA phase in steps of two
static inline void mc_position(uint32_t idx, int si, int c, int rwd, int &x, int &y)
{
  const uint32_t k = idx / 4, bpr = (uint32_t)rwd / 64;
  x = 64 * (int)(k % bpr); y = 4 * (int)(k / bpr);
  if(si >= 16) { x -= 64; y += 2; }
  if((idx & 3) == 1) x += 1;
  if((idx & 3) == 2) y += 1;
  if((idx & 3) == 3) { x += 1; y += 1; }
  x += 4 * si + 2 * c;
}
// the R16_UNORM store of res / 65536
static inline uint16_t mc_store(uint32_t res)
{
  const float v = std::fmin(std::fmax((float)res / 65536.0f, 0.0f), 1.0f);
  return (uint16_t)std::nearbyint(v * 65535.0f);
}
extern "C" void oracle_mcraw_decode(const uint8_t *bitcnt, const uint16_t *refval, const uint8_t *data, size_t data_bytes,
    int rwd, int ht, int ox, int oy, int wd_out, int ht_out, uint16_t *out)
{
  const uint32_t blocks = (uint32_t)rwd * (uint32_t)ht / 64;
  uint64_t off = 0;   // the exclusive prefix of the block sizes (prefix.comp, inclusive, read one block back)
  for(uint32_t idx = 0; idx < blocks; idx++)
  {
    uint32_t cnt = bitcnt[idx / 2];
    if(idx & 1) cnt >>= 4;
    cnt &= 0xf;
    uint8_t d[128];
    for(int b = 0; b < 128; b++) d[b] = off + b < data_bytes ? data[off + b] : 0;
    for(int si = 0; si < 32; si++)
    {
      uint32_t r[2];
      mc_decode_pair(cnt, d, si, r);
      for(int c = 0; c < 2; c++)
      {
        int x, y;
        mc_position(idx, si, c, rwd, x, y);
        x -= ox; y -= oy;
        if(x >= 0 && y >= 0 && x < wd_out && y < ht_out) out[(size_t)y * wd_out + x] = mc_store(r[c] + refval[idx]);
      }
    }
    off += mc_block_bytes(cnt);
  }
}
// test data: a frame encoded so that the decoder above gives it back. The bit
// layout of each count is found by decoding single set bits (the decoder only
// moves bits), the reference is the block's minimum and the count the width of
// its largest delta (counts 7 and 9 are stored as given, 11..16 as 15).
extern "C" size_t oracle_mcraw_encode(const uint16_t *img, int rwd, int ht, int force_cnt,
    uint8_t *bitcnt, uint16_t *refval, uint8_t *data, size_t cap)
{
  static int map[16][64][16];   // [cnt][sample][bit] -> byte * 8 + bit
  static bool ready = false;
  if(!ready)
  {
    for(int cnt = 1; cnt < 16; cnt++)
    {
      for(int j = 0; j < 64; j++) for(int q = 0; q < 16; q++) map[cnt][j][q] = -1;
      for(uint32_t b = 0; b < mc_block_bytes((uint32_t)cnt); b++) for(int t = 0; t < 8; t++)
      {
        uint8_t d[128] = { 0 };
        d[b] = (uint8_t)(1u << t);
        for(int si = 0; si < 32; si++)
        {
          uint32_t r[2];
          mc_decode_pair((uint32_t)cnt, d, si, r);
          for(int c = 0; c < 2; c++) for(int q = 0; q < 16; q++)
            if((r[c] >> q) & 1) map[cnt][2 * si + c][q] = (int)(8 * b + t);
        }
      }
    }
    ready = true;
  }
  const uint32_t blocks = (uint32_t)rwd * (uint32_t)ht / 64;
  memset(bitcnt, 0, (blocks + 1) / 2);
  size_t off = 0;
  for(uint32_t idx = 0; idx < blocks; idx++)
  {
    uint32_t v[64], mn = 0xffff, mx = 0;
    for(int si = 0; si < 32; si++) for(int c = 0; c < 2; c++)
    {
      int x, y;
      mc_position(idx, si, c, rwd, x, y);
      v[2 * si + c] = img[(size_t)y * rwd + x];
      mn = std::min(mn, v[2 * si + c]);
      mx = std::max(mx, v[2 * si + c]);
    }
    int bits = 0;
    while(bits < 16 && ((mx - mn) >> bits)) bits++;
    int cnt = force_cnt >= 0 ? std::max(force_cnt, bits) : bits;
    if(cnt > 10) cnt = 15;
    const int width = cnt == 7 ? 8 : cnt == 9 ? 10 : cnt == 15 ? 16 : cnt;
    bitcnt[idx / 2] |= (uint8_t)(cnt << ((idx & 1) ? 4 : 0));
    refval[idx] = (uint16_t)mn;
    const uint32_t nb = mc_block_bytes((uint32_t)cnt);
    if(off + nb > cap) return 0;
    memset(data + off, 0, nb);
    for(int j = 0; j < 64; j++) for(int q = 0; q < width; q++)
      if(((v[j] - mn) >> q) & 1)
      {
        const int pos = map[cnt][j][q];
        if(pos < 0) return 0;
        data[off + pos / 8] |= (uint8_t)(1u << (pos % 8));
      }
    off += nb;
  }
  return off;
}

// ------------------------------------------------------------------ output encode: BC1 (o-bc1)
// o-bc1/main.c:21-47 compresses every 4x4 block of the rgba u8 thumbnail with
// the vendored stb_dxt (o-bc1/stb_dxt.h v1.08b: stb_compress_dxt_block, no
// alpha, normal mode: no dither, one refinement). Restated step by step:
// endpoints from the principal axis (four power iterations on the colour
// covariance), indices by projection onto the endpoint line, one least
// squares refinement of the endpoints, the optimal single colour tables for
// constant blocks. Integer work as there; the float and double steps in the
// same order (the oracle builds without contraction).
namespace bc1 {
struct tables_t { uint8_t om5[256][2], om6[256][2]; };
static inline int e5(int i) { return (i << 3) | (i >> 2); }
static inline int e6(int i) { return (i << 2) | (i >> 4); }
static inline int mul8(int a, int b) { const int t = a * b + 128; return (t + (t >> 8)) >> 8; }   // a*b/255, rounded
static inline int lerp13(int a, int b) { return (2 * a + b) / 3; }
static void opt_table(uint8_t tab[256][2], int size, int (*ex)(int))
{ // the endpoint pair whose 1/3 point reproduces a constant best (DX10's 3% rule as a penalty)
  for(int i = 0; i < 256; i++)
  {
    int best = 256;
    for(int mn = 0; mn < size; mn++) for(int mx = 0; mx < size; mx++)
    {
      const int err = std::abs(lerp13(ex(mx), ex(mn)) - i) + std::abs(ex(mx) - ex(mn)) * 3 / 100;
      if(err < best) { tab[i][0] = (uint8_t)mx; tab[i][1] = (uint8_t)mn; best = err; }
    }
  }
}
static const tables_t &tables()
{
  static tables_t t;
  static bool done = false;
  if(!done) { opt_table(t.om5, 32, e5); opt_table(t.om6, 64, e6); done = true; }
  return t;
}
static inline uint16_t to565(int r, int g, int b) { return (uint16_t)((mul8(r, 31) << 11) + (mul8(g, 63) << 5) + mul8(b, 31)); }
static void palette(uint16_t c0, uint16_t c1, int col[4][3])
{
  col[0][0] = e5(c0 >> 11); col[0][1] = e6((c0 >> 5) & 63); col[0][2] = e5(c0 & 31);
  col[1][0] = e5(c1 >> 11); col[1][1] = e6((c1 >> 5) & 63); col[1][2] = e5(c1 & 31);
  for(int k = 0; k < 3; k++) { col[2][k] = lerp13(col[0][k], col[1][k]); col[3][k] = lerp13(col[1][k], col[0][k]); }
}
static uint32_t match(const uint8_t *px, const int col[4][3])
{ // indices from the projection onto the endpoint line (stops: the midpoints between palette entries)
  const int dr = col[0][0] - col[1][0], dg = col[0][1] - col[1][1], db = col[0][2] - col[1][2];
  int stops[4];
  for(int k = 0; k < 4; k++) stops[k] = col[k][0] * dr + col[k][1] * dg + col[k][2] * db;
  const int c0p = (stops[1] + stops[3]) >> 1, half = (stops[3] + stops[2]) >> 1, c3p = (stops[2] + stops[0]) >> 1;
  uint32_t mask = 0;
  for(int i = 15; i >= 0; i--)
  {
    const int dot = px[4 * i] * dr + px[4 * i + 1] * dg + px[4 * i + 2] * db;
    mask <<= 2;
    if(dot < half) mask |= dot < c0p ? 1u : 3u;
    else           mask |= dot < c3p ? 2u : 0u;
  }
  return mask;
}
static void pca(const uint8_t *px, uint16_t &mx16, uint16_t &mn16)
{
  int mu[3], lo[3], hi[3];
  for(int c = 0; c < 3; c++)
  {
    int sum = px[c];
    lo[c] = hi[c] = px[c];
    for(int i = 1; i < 16; i++)
    {
      const int v = px[4 * i + c];
      sum += v;
      lo[c] = std::min(lo[c], v);
      hi[c] = std::max(hi[c], v);
    }
    mu[c] = (sum + 8) >> 4;
  }
  int cov[6] = { 0, 0, 0, 0, 0, 0 };
  for(int i = 0; i < 16; i++)
  {
    const int r = px[4 * i] - mu[0], g = px[4 * i + 1] - mu[1], b = px[4 * i + 2] - mu[2];
    cov[0] += r * r; cov[1] += r * g; cov[2] += r * b; cov[3] += g * g; cov[4] += g * b; cov[5] += b * b;
  }
  float cf[6];
  for(int i = 0; i < 6; i++) cf[i] = (float)cov[i] / 255.0f;
  float vr = (float)(hi[0] - lo[0]), vg = (float)(hi[1] - lo[1]), vb = (float)(hi[2] - lo[2]);
  for(int it = 0; it < 4; it++)
  {
    const float r = vr * cf[0] + vg * cf[1] + vb * cf[2];
    const float g = vr * cf[1] + vg * cf[3] + vb * cf[4];
    const float b = vr * cf[2] + vg * cf[4] + vb * cf[5];
    vr = r; vg = g; vb = b;
  }
  double magn = std::fabs((double)vr);
  if(std::fabs((double)vg) > magn) magn = std::fabs((double)vg);
  if(std::fabs((double)vb) > magn) magn = std::fabs((double)vb);
  int wr, wg, wb;
  if(magn < 4.0) { wr = 299; wg = 587; wb = 114; }   // too small: luminance
  else
  {
    magn = 512.0 / magn;
    wr = (int)((double)vr * magn); wg = (int)((double)vg * magn); wb = (int)((double)vb * magn);
  }
  int mind = 0x7fffffff, maxd = -0x7fffffff, imin = 0, imax = 0;
  for(int i = 0; i < 16; i++)
  {
    const int dot = px[4 * i] * wr + px[4 * i + 1] * wg + px[4 * i + 2] * wb;
    if(dot < mind) { mind = dot; imin = i; }
    if(dot > maxd) { maxd = dot; imax = i; }
  }
  mx16 = to565(px[4 * imax], px[4 * imax + 1], px[4 * imax + 2]);
  mn16 = to565(px[4 * imin], px[4 * imin + 1], px[4 * imin + 2]);
}
static inline int sclamp(float y, int lo, int hi) { const int x = (int)y; return x < lo ? lo : (x > hi ? hi : x); }
static bool refine(const uint8_t *px, uint16_t &mx16, uint16_t &mn16, uint32_t mask)
{ // least squares endpoints for the given indices (normal equations, Cramer's rule)
  const uint16_t omn = mn16, omx = mx16;
  uint16_t a16, b16;
  if((mask ^ (mask << 2)) < 4)
  { // one index for all pixels: the optimal single colour of the average
    const tables_t &t = tables();
    int r = 8, g = 8, b = 8;
    for(int i = 0; i < 16; i++) { r += px[4 * i]; g += px[4 * i + 1]; b += px[4 * i + 2]; }
    r >>= 4; g >>= 4; b >>= 4;
    a16 = (uint16_t)((t.om5[r][0] << 11) | (t.om6[g][0] << 5) | t.om5[b][0]);
    b16 = (uint16_t)((t.om5[r][1] << 11) | (t.om6[g][1] << 5) | t.om5[b][1]);
  }
  else
  {
    static const int w1[4] = { 3, 0, 2, 1 };
    int xx = 0, yy = 0, xy = 0, a1[3] = { 0, 0, 0 }, a2[3] = { 0, 0, 0 };
    uint32_t cm = mask;
    for(int i = 0; i < 16; i++, cm >>= 2)
    {
      const int w = w1[cm & 3];
      xx += w * w; yy += (3 - w) * (3 - w); xy += w * (3 - w);
      for(int c = 0; c < 3; c++) { a1[c] += w * px[4 * i + c]; a2[c] += px[4 * i + c]; }
    }
    for(int c = 0; c < 3; c++) a2[c] = 3 * a2[c] - a1[c];
    const float frb = 3.0f * 31.0f / 255.0f / (float)(xx * yy - xy * xy);
    const float fg = frb * 63.0f / 31.0f;
    a16 = (uint16_t)((sclamp((float)(a1[0] * yy - a2[0] * xy) * frb + 0.5f, 0, 31) << 11)
        | (sclamp((float)(a1[1] * yy - a2[1] * xy) * fg + 0.5f, 0, 63) << 5)
        | sclamp((float)(a1[2] * yy - a2[2] * xy) * frb + 0.5f, 0, 31));
    b16 = (uint16_t)((sclamp((float)(a2[0] * xx - a1[0] * xy) * frb + 0.5f, 0, 31) << 11)
        | (sclamp((float)(a2[1] * xx - a1[1] * xy) * fg + 0.5f, 0, 63) << 5)
        | sclamp((float)(a2[2] * xx - a1[2] * xy) * frb + 0.5f, 0, 31));
  }
  mn16 = b16; mx16 = a16;
  return omn != mn16 || omx != mx16;
}
static void block(const uint8_t *px, uint8_t *out)
{
  uint32_t mask;
  uint16_t mx16, mn16;
  bool constant = true;
  for(int i = 1; i < 16 && constant; i++) constant = memcmp(px + 4 * i, px, 4) == 0;
  if(constant)
  {
    const tables_t &t = tables();
    const int r = px[0], g = px[1], b = px[2];
    mask = 0xaaaaaaaau;
    mx16 = (uint16_t)((t.om5[r][0] << 11) | (t.om6[g][0] << 5) | t.om5[b][0]);
    mn16 = (uint16_t)((t.om5[r][1] << 11) | (t.om6[g][1] << 5) | t.om5[b][1]);
  }
  else
  {
    int col[4][3];
    pca(px, mx16, mn16);
    if(mx16 != mn16) { palette(mx16, mn16, col); mask = match(px, col); }
    else mask = 0;
    const uint32_t last = mask;
    if(refine(px, mx16, mn16, mask))
    {
      if(mx16 != mn16) { palette(mx16, mn16, col); mask = match(px, col); }
      else mask = 0;
    }
    (void)last;
  }
  if(mx16 < mn16) { const uint16_t t = mn16; mn16 = mx16; mx16 = t; mask ^= 0x55555555u; }
  out[0] = (uint8_t)mx16; out[1] = (uint8_t)(mx16 >> 8); out[2] = (uint8_t)mn16; out[3] = (uint8_t)(mn16 >> 8);
  for(int k = 0; k < 4; k++) out[4 + k] = (uint8_t)(mask >> (8 * k));
}
} // namespace bc1

// lens/main.comp:22-57, the double sphere camera model (V. Usenko, N. Demmel, D.
// Cremers, "The Double Sphere Camera Model", 2018): the output position, centred
// and scaled by the output's aspect, is unprojected with the two sphere radii
// r = (squish0, squish1), projected back to a pinhole, moved by the centre and
// sampled with the Catmull-Rom filter; with chromatic aberration factors other
// than (1, 1) red and blue sample at positions scaled about the image centre.
// par is the uniform block: centre (2), scale (2), squish0, squish1, ca red, ca
// blue. GLSL's component-wise operations in the shader's order; out stores f16.
template<class T> static img_t<T> lens_main(const img_t<T> &in, const float *par, int wd, int ht)
{
  img_t<T> out(wd, ht, 4);
  const T aspx = T(wd) / T(ht);
  const T cx = par[0], cy = par[1], fx = par[2], fy = par[3], r0 = par[4], r1 = par[5];
  const T cax = par[6], cay = par[7];
  const bool plain = par[6] == 1.0f && par[7] == 1.0f;
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    const T px = ((T(x) + T(0.5)) / T(wd) - T(0.5)) * aspx;
    const T py = ((T(y) + T(0.5)) / T(ht) - T(0.5)) * T(1);
    const T mx = px / fx, my = py / fy;
    const T r2 = T(0) + mx * mx + my * my;                       // dot(m, m)
    const T mz = (T(1) - r0 * r0 * r2) / (r0 * std::sqrt(T(1) - (T(2) * r0 - T(1)) * r2) + T(1) - r0);
    const T s = (mz * r1 + std::sqrt(mz * mz + (T(1) - r1 * r1))) / (mz * mz + r2);
    const T X = s * mx - T(0), Y = s * my - T(0), Z = s * mz - r1;
    const T ux = X / Z / aspx + T(0.5) + cx;
    const T uy = Y / Z / T(1) + T(0.5) + cy;
    T rgba[4], t[4];
    catmull_rom_uv(in, ux, uy, t);
    rgba[0] = t[0]; rgba[1] = t[1]; rgba[2] = t[2];
    if(!plain)
    {
      catmull_rom_uv(in, (ux - T(0.5)) * cax + T(0.5), (uy - T(0.5)) * cax + T(0.5), t);
      rgba[0] = t[0];
      catmull_rom_uv(in, (ux - T(0.5)) * cay + T(0.5), (uy - T(0.5)) * cay + T(0.5), t);
      rgba[2] = t[2];
    }
    rgba[3] = T(1);
    out.store(x, y, rgba, 4);
  }
  return out;
}

extern "C" void oracle_lens(const float *rgba, int wd, int ht, int owd, int oht, const float *par, float *out)
{
  img_t<float> in(wd, ht, 4);
  std::copy(rgba, rgba + (size_t)wd * ht * 4, in.d.begin());
  const img_t<float> o = lens_main(in, par, owd, oht);
  std::copy(o.d.begin(), o.d.end(), out);
}

// colenc/main.comp:15-80: rec2020 linear rgb to the output primaries
// (matrices.h, row major) and transfer curve; out: rgba with alpha 1, as FP32
// values (the f16 store rounds them; an 8-bit sink rounds them to 1/255)
// grade/main.comp:23-64: lift / gamma / gain / offset per channel (each with its
// fourth component added, grade/main.comp:32-35), or in mode != 0 their zoned
// form weighted by a log luminance. par: lift, gamma, gain, offset (4 each).
extern "C" void oracle_grade(const float *rgba, int wd, int ht, const float *par, int mode, float sh_pivot,
    float hi_pivot, float *out)
{
  float lift[3], gamma[3], gain[3], off[3];
  for(int k = 0; k < 3; k++)
  {
    lift[k] = par[k] + par[3];
    gamma[k] = gmax(par[4 + k] + par[7], 1e-6f);
    gain[k] = gmax(par[8 + k] + par[11], 0.0f);
    off[k] = par[12 + k] + par[15];
  }
  OMP_FOR
  for(int64_t i = 0; i < (int64_t)wd * ht; i++)
  {
    float rgb[3] = { rgba[4 * i + 0], rgba[4 * i + 1], rgba[4 * i + 2] };
    float ge[3] = { gain[0], gain[1], gain[2] }, le[3] = { lift[0], lift[1], lift[2] };
    float ye[3] = { gamma[0], gamma[1], gamma[2] };
    if(mode != 0)
    { // dot(max(rgb, 0), (0.2126, 0.7152, 0.0722)) summed in order
      float L = 0.0f;
      L = L + gmax(rgb[0], 0.0f) * 0.2126f;
      L = L + gmax(rgb[1], 0.0f) * 0.7152f;
      L = L + gmax(rgb[2], 0.0f) * 0.0722f;
      L = gclamp(0.67f + std::log2(gmax(L, 1e-6f)) * 0.11f, 0.0f, 1.0f);
      const float sp = gclamp(sh_pivot, 1e-3f, 1.0f - 1e-3f);
      const float hp = gclamp(hi_pivot, sp + 1e-3f, 1.0f);
      const float ws = 1.0f - smoothstep(0.0f, sp, L);
      const float wh = smoothstep(hp, 1.0f, L);
      const float wm = 1.0f - ws - wh;
      for(int k = 0; k < 3; k++)
      {
        ge[k] = gmix(1.0f, gain[k], wh);
        le[k] = lift[k] * ws;
        ye[k] = gmix(1.0f, gamma[k], wm);
      }
    }
    for(int k = 0; k < 3; k++)
    {
      float v = ge[k] * rgb[k];
      v = v * (1.0f - le[k]) + le[k];
      v = std::pow(gmax(v, 0.0f), 1.0f / ye[k]);
      out[4 * i + k] = v + off[k];
    }
    out[4 * i + 3] = 1.0f;
  }
}

extern "C" void oracle_colenc(const float *rgba, int wd, int ht, int prim, int trc, float *out)
{
  static const double Mp[8][9] = {
    { 1.66022677, -0.58754761, -0.07283825, -0.12455334, 1.13292605, -0.00834963, -0.01815514, -0.10060303, 1.11899817 },  // rec709
    { 1.15194302, -0.09753232, -0.05448118, -0.12454585, 1.13290963, -0.00837122, -0.02253539, -0.04979918, 1.07275365 },  // adobergb
    { 1.34353337, -0.28218904, -0.06142427, -0.06530851, 1.07578268, -0.01048453, 0.00282971, -0.01961215, 1.01717851 },  // p3d65
    { 0.636958048301290991, 0.144616903586208406, 0.168880975164172054, 0.26270021201126692, 0.677998071518871148,
      0.0593017164698619384, 4.9999999999999999e-17, 0.0280726930490874452, 1.06098505771079066 },                   // xyz
    { 6.68685575e-01, 1.51817679e-01, 1.77189677e-01, 4.49002044e-02, 8.62145497e-01, 1.01922441e-01, -2.66851927e-09,
      2.78271109e-02, 1.05170358 },                                                                                  // ap0
    { 9.62918591e-01, 1.16137050e-02, 2.55863361e-02, 4.16800770e-04, 9.99378426e-01, -8.82457347e-05, 5.31123331e-03,
      2.18655328e-02, 9.75907920e-01 },                                                                              // ap1
    { 0.853263, 0.079695, 0.067042, 0.029375, 0.809195, 0.161430, 0.051575, 0.208097, 0.740329 },                     // redwg
  };
  const int mi = prim == 1 ? 0 : prim == 3 ? 1 : prim == 4 ? 2 : prim == 5 ? 3 : prim == 6 ? 4 : prim == 7 ? 5 : prim == 10 ? 6 : -1;
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    const float *p = rgba + 4 * ((size_t)y * wd + x);
    float c[3] = { p[0], p[1], p[2] };
    if(mi >= 0)
    {
      float o[3];
      for(int j = 0; j < 3; j++)
      {
        float a = 0.0f;
        for(int i = 0; i < 3; i++) a = a + (float)Mp[mi][3 * j + i] * c[i];
        o[j] = a;
      }
      for(int j = 0; j < 3; j++) c[j] = o[j];
    }
    for(int k = 0; k < 3; k++)
    {
      float v = c[k];
      if(trc == 1)
      {
        const float a = 1.09929682680944f, b = 0.018053968510807f;
        v = v > b ? std::pow(v, 1.0f / 2.2f) * a - (a - 1.0f) : v * 4.5f;
      }
      else if(trc == 2) v = v > 0.0031308f ? std::pow(v, 1.0f / 2.4f) * 1.055f - 0.055f : v * 12.92f;
      else if(trc == 3)
      {
        const float c3 = 2392.0f / 128.0f, c2 = 2413.0f / 128.0f, c1 = c3 - c2 + 1.0f, m1 = 1305.0f / 8192.0f, m2 = 2523.0f / 32.0f;
        const float q = std::pow(std::fmax(0.0f, v), m1);
        const float num = (c1 - 1.0f) + (c2 - c3) * q, den = 1.0f + c3 * q;
        v = std::pow(1.0f + num / den, m2);
      }
      else if(trc == 4) v = std::pow(v, 1.0f / 2.6f);
      else if(trc == 5)
      {
        const float a = 0.17883277f, b = 1.0f - 4.0f * a, cc = 0.5f - a * std::log(4.0f * a);
        v = v > 1.0f / 12.0f ? a * std::log(12.0f * v - b) + cc : std::sqrt(3.0f * v);
      }
      else if(trc == 6) v = std::pow(v, 1.0f / 2.2f);
      c[k] = v;
    }
    float *o = out + 4 * ((size_t)y * wd + x);
    o[0] = c[0]; o[1] = c[1]; o[2] = c[2]; o[3] = 1.0f;
  }
}

// the blocks of an rgba u8 image, wd/4 x ht/4 of 8 bytes (o-bc1/main.c:30-47: partial blocks are dropped)
extern "C" void oracle_bc1_encode(const uint8_t *rgba, int wd, int ht, uint8_t *out)
{
  const int bx = wd / 4, by = ht / 4;
  for(int j = 0; j < by; j++) for(int i = 0; i < bx; i++)
  {
    uint8_t blk[64];
    for(int jj = 0; jj < 4; jj++) for(int ii = 0; ii < 4; ii++) for(int c = 0; c < 4; c++)
      blk[4 * (4 * jj + ii) + c] = rgba[4 * ((size_t)wd * (4 * j + jj) + (4 * i + ii)) + c];
    bc1::block(blk, out + 8 * ((size_t)bx * j + i));
  }
}

extern "C" void oracle_rcd(const float *cfa, int wd, int ht, const float wb[3], float *out)
{ // demosaic/rcd_conv.comp + rcd_fill.comp on an f16 mosaic (FP32 build)
  img_t<float> in(wd, ht, 1);
  for(size_t i = 0; i < (size_t)wd * ht; i++) in.d[i] = cfa[i];
  img_t<float> vh, pq, lp;
  rcd_conv(in, vh, pq, lp);
  const float w[3] = { wb[0], wb[1], wb[2] };
  img_t<float> o = rcd_fill(in, vh, pq, lp, w);
  std::memcpy(out, o.d.data(), sizeof(float) * o.d.size());
}

extern "C" uint32_t oracle_hist_bin(float r, float g, float b)
{ // OpenDRT/hist.comp:15-20 get_bin, shared/oetf.glsl:13-15 eotf_filmlight_tlog
  const float p0 = 2.62700212e-01f * r, p1 = 6.77998072e-01f * g, p2 = 5.93017165e-02f * b;
  const float v = (p0 + p1) + p2;
  float l;
  if(v < 0.0f) { const float t = v * 16.184376489665897f; l = t + 0.075f; }
  else
  {
    const float a = v + 0.0057048244042473785f;
    const float t = hist_log(a) * 0.09232902596577353f;
    l = t + 0.5520126568606655f;
  }
  const float f = 256.0f * l;
  const float fb = f + 0.5f;
  uint32_t bin;
  if(!(fb > 0.0f)) bin = 0;                 // negative and NaN saturate to 0
  else if(fb >= 4294967295.0f) bin = 0xffffffffu;
  else bin = (uint32_t)fb;
  return bin > 255u ? 255u : bin;
}

namespace {

template<class T> static void hist(const img_t<T> &in, uint32_t *h)
{
  for(int i = 0; i < 257; i++) h[i] = 0;
  for(int y = 0; y < in.h; y++) for(int x = 0; x < in.w; x++)
  {
    const uint32_t bin = oracle_hist_bin((float)fetch_z(in, x, y, 0), (float)fetch_z(in, x, y, 1), (float)fetch_z(in, x, y, 2));
    if(bin > 0) { h[bin]++; h[256]++; }
  }
}

// ------------------------------------------------------------------ llap

static const int NUM_GAMMA = 10; // llap/config.h:2

template<class T> static inline T gamma_from_i(int i)
{ // llap/llap.glsl:3-14
  return T(i) / (T(NUM_GAMMA) - T(1.0));
}
template<class T> static inline int gamma_hi_from_v(T v)
{ // llap/llap.glsl:16-21
  int hi = 1;
  for(; hi < NUM_GAMMA - 1 && gamma_from_i<T>(hi) <= v; hi++);
  return hi;
}

// llap/curve.comp:39-63
template<class T> static inline T llap_curve_fn(T x, T g, T sigma, T shadows, T highlights, T clarity)
{
  const T c = x - g;
  T val;
  const T ssigma = c > T(0) ? sigma : -sigma;
  const T shadhi = c > T(0) ? shadows : highlights;
  if(std::fabs(c) > T(2) * sigma) val = g + ssigma + shadhi * (c - ssigma);
  else
  {
    const T t = gclamp(c / (T(2.0) * ssigma), T(0.0), T(1.0));
    const T t2 = t * t;
    const T mt = T(1.0) - t;
    val = g + ssigma * T(2.0) * mt * t + t2 * (ssigma + ssigma * shadhi);
  }
  val += clarity * c * std::exp(-c * c / (T(2.0) * sigma * sigma / T(3.0)));
  return val;
}

// llap/curve.comp:65-79: 11 planes (NUM_GAMMA curves + grey)
template<class T> static std::vector<img_t<T>> llap_curve(const img_t<T> &in, const oracle_params_t *p)
{
  std::vector<img_t<T>> out(NUM_GAMMA + 1, img_t<T>(in.w, in.h, 1));
  OMP_FOR
  for(int y = 0; y < in.h; y++) for(int x = 0; x < in.w; x++)
  {
    T rgb[3];
    for(int k = 0; k < 3; k++) rgb[k] = gclamp(fetch_z(in, x, y, k), T(-1000.0), T(1000.0));
    const T yv = lum2020(rgb[0], rgb[1], rgb[2]);
    for(int i = 0; i < NUM_GAMMA; i++)
    {
      const T v[1] = { llap_curve_fn(yv, gamma_from_i<T>(i), T(p->ll_sigma), T(p->ll_shadows), T(p->ll_hilights), T(p->ll_clarity)) };
      out[i].store(x, y, v, 1);
    }
    const T v[1] = { yv };
    out[NUM_GAMMA].store(x, y, v, 1);
  }
  return out;
}

// one bilinear tap at half-texel offsets (texel-space coordinate x of the sampler)
template<class T> static inline T tap(const img_t<T> &im, T x, T y)
{
  T v[4];
  tex_bilinear(im, x, y, v);
  return v[0];
}

// llap/reduce.comp:17-35 with shared.glsl:130-148 sample_semisoft
template<class T> static img_t<T> llap_reduce(const img_t<T> &in, int wd, int ht)
{
  img_t<T> out(wd, ht, 1);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    const T cx = T(2 * x) + T(0.5), cy = T(2 * y) + T(0.5);
    T r = T(0);
    r += tap(in, cx - T(.5), cy - T(.5));
    r += tap(in, cx + T(.5), cy - T(.5));
    r += tap(in, cx - T(.5), cy + T(.5));
    r += tap(in, cx + T(.5), cy + T(.5));
    const T v[1] = { r / T(4.0) };
    out.store(x, y, v, 1);
  }
  return out;
}

// llap/assemble.comp:54-58 gauss_expand via shared.glsl:99-127 sample_soft
template<class T> static inline T llap_expand(const img_t<T> &im, int ox, int oy)
{
  const T sx = T(ox) * T(0.5) + T(0.5), sy = T(oy) * T(0.5) + T(0.5);
  const T tx[3] = { sx - T(1.5), sx, sx + T(1.5) }, ty[3] = { sy - T(1.5), sy, sy + T(1.5) };
  T r = T(0);
  for(int j = 0; j < 3; j++) for(int i = 0; i < 3; i++) r += tap(im, tx[i], ty[j]);
  return r / T(9.0);
}

// llap/assemble.comp:89-123
template<class T> static img_t<T> llap_assemble(const img_t<T> &coarse, const std::vector<img_t<T>> &l0,
    const std::vector<img_t<T>> &l1, int first, int wd, int ht)
{
  img_t<T> out(wd, ht, 1);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    T res;
    if(first > 0) res = llap_expand(l1[NUM_GAMMA], x, y);
    else          res = llap_expand(coarse, x, y);
    const T v = fetch_z(l0[NUM_GAMMA], x, y, 0);
    const int hi = gamma_hi_from_v(v);
    const int lo = hi - 1;
    const T glo = gamma_from_i<T>(lo), ghi = gamma_from_i<T>(hi);
    const T a = gclamp((v - glo) / (ghi - glo), T(0.0), T(1.0));
    const T la = fetch_z(l0[hi - 1], x, y, 0) - llap_expand(l1[hi - 1], x, y);
    const T lb = fetch_z(l0[hi], x, y, 0) - llap_expand(l1[hi], x, y);
    const T o[1] = { res + la * (T(1.0) - a) + lb * a };
    out.store(x, y, o, 1);
  }
  return out;
}

// llap/colour.comp:141-160
template<class T> static img_t<T> llap_colour(const img_t<T> &yimg, const img_t<T> &org)
{
  img_t<T> out(org.w, org.h, 4);
  OMP_FOR
  for(int y = 0; y < org.h; y++) for(int x = 0; x < org.w; x++)
  {
    T yv = fetch_z(yimg, x, y, 0);
    T rgb[3];
    for(int k = 0; k < 3; k++) rgb[k] = fetch_z(org, x, y, k);
    const T yo = gmax(lum2020(rgb[0], rgb[1], rgb[2]), T(1e-8));
    const T c = T(1.0);
    if(yv < yo) yv = yo * std::exp(c * (yv - yo));
    T o[4];
    for(int k = 0; k < 3; k++) o[k] = gmax(T(0), rgb[k] * yv / yo);
    o[3] = T(1);
    out.store(x, y, o, 4);
  }
  return out;
}

// ------------------------------------------------------------------ graph

template<class T> static void to_float(const img_t<T> &im, float *dst)
{
  if(!dst) return;
  for(size_t i = 0; i < im.d.size(); i++) dst[i] = (float)im.d[i];
}
template<class T> static void to_float_ch(const img_t<T> &im, int ch, float *dst)
{ // first ch channels of every pixel
  if(!dst) return;
  OMP_FOR
  for(int y = 0; y < im.h; y++) for(int x = 0; x < im.w; x++)
    for(int k = 0; k < ch; k++) dst[((size_t)y * im.w + x) * ch + k] = (float)im.ch(x, y, k);
}

template<class T> static int develop(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *st)
{
  if(wd <= 0 || ht <= 0 || !mosaic || !ip || !p) return 1;
  const uint32_t filters = ip->filters;
  if(filters == 0) return 2; // the path starts on a mosaic
  // i-raw output: R16_UNORM
  img_t<T> raw(wd, ht, 1);
  for(size_t i = 0; i < (size_t)wd * ht; i++) raw.d[i] = T(mosaic[i]) / T(65535);

  // ---- denoise (denoise/main.c:133-333). crop window and black/white in unorm units
  T black[4], white[4], wb[4];
  for(int k = 0; k < 4; k++)
  {
    black[k] = T(ip->black[k] / 65535.0f);
    white[k] = T(ip->white[k] / 65535.0f);
    wb[k] = T(ip->whitebalance[k]);
  }
  const int cw = (int)(ip->crop_aabb[2] - ip->crop_aabb[0]), ch = (int)(ip->crop_aabb[3] - ip->crop_aabb[1]);
  if(cw <= 0 || ch <= 0 || (int)ip->crop_aabb[2] > wd || (int)ip->crop_aabb[3] > ht) return 3;
  const int crop[4] = { (int)ip->crop_aabb[0], (int)ip->crop_aabb[1], (int)ip->crop_aabb[2], (int)ip->crop_aabb[3] };
  const int W = cw, H = ch; // module output roi
  const T edges[4] = { T(p->dn_edges[0]), T(p->dn_edges[1]), T(p->dn_edges[2]), T(p->dn_edges[3]) };
  img_t<T> dn;
  if(p->dn_strength <= 0.0f)
  {
    dn = denoise_noop(raw, W, H, crop, black, white);
  }
  else
  {
    const int block = filters == 9u ? 3 : 2;
    const int hw = W / block, hh = H / block;
    img_t<T> half = denoise_half(raw, hw, hh, crop, white[1], filters);
    const int zc[4] = { 0, 0, 0, 0 };
    img_t<T> s[5];
    s[0] = half;
    s[1] = denoise_downcov(half, hw, hh, zc);
    for(int i = 1; i < 4; i++)
      s[i + 1] = denoise_down(s[i], hw, hh, zc, black[1], white[1], T(ip->noise_a), T(ip->noise_b), edges, i, block);
    img_t<T> as = denoise_assemble(s, hw, hh, zc, wb, black, white, T(ip->noise_a), T(ip->noise_b), filters,
        T(p->dn_strength), T(p->dn_luma), edges);
    dn = denoise_doub(raw, as, half, W, H, crop, black, white, filters, T(ip->noise_a), T(ip->noise_b),
        T(p->dn_strength), T(p->dn_luma), T(p->dn_detail), edges);
  }
  if(g_inj.start >= 1) dn = from_float<T>(g_inj.img, W, H, 1);   // (the start stage replaces it)
  if(st) to_float_ch(dn, 1, st->denoise);

  // ---- hilite (hilite/main.c:5-90)
  const int block = filters == 9u ? 3 : 2;
  img_t<T> hl(W, H, 1);
  {
    const T hwhite = T(p->hl_white);
    const int hw = W / block, hh = H / block;
    img_t<T> h0 = hilite_half(dn, hw, hh, hwhite, filters);
    std::vector<img_t<T>> red;   // reduce outputs r_1..r_n
    std::vector<int> rw, rh;
    int cwd = (hw - 1) / 2 + 1, cht = (hh - 1) / 2 + 1;
    const int max_nl = 15;
    const img_t<T> *fine = &h0;
    red.reserve(max_nl);
    for(int l = 1; l < max_nl; l++)
    {
      red.push_back(hilite_reduce(*fine, cwd, cht, wb, hwhite, T(p->hl_desat)));
      fine = &red.back();
      const int nwd = (cwd - 1) / 2 + 1, nht = (cht - 1) / 2 + 1;
      cwd = nwd; cht = nht;
      if(cwd <= 1 || cht <= 1 || l + 1 == max_nl) break;
    }
    if(st) st->hilite_levels = (int)red.size();
    // assemble from the coarsest: the last assemble takes the last reduce as coarse
    img_t<T> up = red.back();
    for(int l = (int)red.size() - 1; l >= 0; l--)
    {
      const img_t<T> &f = l == 0 ? h0 : red[l - 1];
      up = hilite_assemble(f, up, f.w, f.h, hwhite, T(p->hl_soft));
    }
    hilite_doub(dn, up, hw, hh, hwhite, filters, hl);
  }
  if(g_inj.start >= 2) hl = from_float<T>(g_inj.img, W, H, 1);
  if(st) to_float_ch(hl, 1, st->hilite);

  // ---- demosaic (demosaic/main.c:18-203)
  // demosaic/main.c:18-41: method 2 halves the module's output size
  const int fw = p->dm_method == 2 ? (W + 1) / 2 : W, fh = p->dm_method == 2 ? (H + 1) / 2 : H;
  const int ow = p->out_wd > 0 ? p->out_wd : fw, oh = p->out_ht > 0 ? p->out_ht : fh;
  const float scale = (float)W / (float)ow;
  const int halfsize = (scale >= 1.5 * block) || (p->dm_method == 2);
  img_t<T> rgb;
  if(halfsize)
  {
    img_t<T> hs = demosaic_halfsize(hl, W / block, H / block, filters);
    if(block != scale) rgb = shared_resample(hs, ow, oh);
    else rgb = hs;
  }
  else
  {
    if(ow != W || oh != H) return 4; // resample after full-size demosaic not covered
  }
  if(!halfsize && p->dm_method == 1)
  { // demosaic/main.c:113-155: RCD (the module runs it whatever the pattern)
    img_t<T> vh, pq, lp;
    rcd_conv(hl, vh, pq, lp);
    rgb = rcd_fill(hl, vh, pq, lp, wb);
  }
  else if(!halfsize)
  {
    img_t<T> cov = demosaic_gauss(hl, W / block, H / block, filters);
    img_t<T> g = demosaic_splat(hl, cov, W, H, filters);
    rgb = demosaic_fix(hl, g, cov, W, H, filters, p->dm_colour);
  }
  if(g_inj.start == 3 || (g_inj.start > 3 && !p->cr_on)) rgb = from_float<T>(g_inj.img, rgb.w, rgb.h, 4);
  if(st) to_float(rgb, st->demosaic);

  // ---- crop (crop/main.comp) when connected between demosaic and colour
  if(p->cr_on && g_inj.start >= 4) rgb = from_float<T>(g_inj.img, p->cr_wd, p->cr_ht, 4);
  else if(p->cr_on) rgb = crop_main(rgb, p->cr_block, p->cr_wd, p->cr_ht);
  if(st) { if(p->cr_on) to_float(rgb, st->crop); st->out_wd = rgb.w; st->out_ht = rgb.h; }

  // ---- colour, filmcurv (+ histogram of its input), llap
  if(p->fc_colour != 1 && p->fc_colour != 3) return 5; // filmcurv colour modes restated: 1, 3
  if(p->co_sat != 1.0f) return 6;                       // colour saturation path not restated
  img_t<T> col = colour_main(rgb, ip, p);
  if(g_inj.start >= 5) col = from_float<T>(g_inj.img, col.w, col.h, 4);
  if(st) to_float(col, st->colour);
  if(st && st->hist) hist(col, st->hist);
  img_t<T> fc = filmcurv_main(col, p);
  if(g_inj.start >= 6) fc = from_float<T>(g_inj.img, fc.w, fc.h, 4);
  if(st) to_float(fc, st->filmcurv);

  // llap (llap/main.c:6-106)
  std::vector<std::vector<img_t<T>>> lev;
  lev.push_back(llap_curve(fc, p));
  int rcw = (fc.w - 1) / 2 + 1, rch = (fc.h - 1) / 2 + 1;
  int nl = 12;
  for(int l = 1; l < nl; l++)
  {
    std::vector<img_t<T>> r;
    for(int i = 0; i <= NUM_GAMMA; i++) r.push_back(llap_reduce(lev[l - 1][i], rcw, rch));
    lev.push_back(r);
    rcw = (rcw - 1) / 2 + 1; rch = (rch - 1) / 2 + 1;
    if(rcw <= 1 || rch <= 1) { nl = l + 1; break; }
    if(p->ll_levels > 0 && l + 1 == p->ll_levels) { nl = l + 1; break; }
  }
  if(st) st->llap_levels = nl;
  img_t<T> up;
  for(int l = nl - 1; l >= 1; l--)
    up = llap_assemble(up, lev[l - 1], lev[l], l == nl - 1, lev[l - 1][0].w, lev[l - 1][0].h);
  img_t<T> outimg = llap_colour(up, fc);
  if(st) to_float(outimg, st->llap);
  return 0;
}

} // namespace

extern "C" {

void oracle_default_params(oracle_params_t *p)
{
  memset(p, 0, sizeof(*p));
  p->dn_strength = 0.0f; p->dn_luma = 0.6f; p->dn_detail = 1.0f; p->dn_gainmap = 1;   // denoise/params:1-6
  p->hl_white = 0.985f; p->hl_desat = 0.3f; p->hl_soft = 0.6f;                        // hilite/params:1-3
  p->dm_colour = 0; p->dm_method = 0;                                                  // demosaic/params:1-2
  p->co_exposure = 0.0f; p->co_sat = 1.0f; p->co_matrix = 1;                           // colour/params:1-9
  p->fc_light = 3.0f; p->fc_contrast = 1.2f; p->fc_bias = 0.0f; p->fc_colour = 3;      // filmcurv/params:1-10
  p->fc_chroma = 1.0f;
  p->ll_sigma = 0.12f; p->ll_shadows = 1.0f; p->ll_hilights = 1.0f; p->ll_clarity = 0.2f; // default-darkroom.i-raw:29-32
}

int oracle_develop_f32(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out)
{ return develop<float>(mosaic, wd, ht, ip, p, out); }

int oracle_develop_f64(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out)
{ return develop<double>(mosaic, wd, ht, ip, p, out); }

int oracle_develop_dec_f32(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec)
{
  g_dec = dec;
  const int r = develop<float>(mosaic, wd, ht, ip, p, out);
  g_dec = nullptr;
  return r;
}

void oracle_set_perturb(uint32_t seed) { g_perturb = seed; }

// the wavelet denoise node by node, each node on the given inputs (another
// implementation's half image, levels and assemble output, hw x hh rgba
// each): out = half (from the mosaic), downcov(in half), down l (in level
// l-1), assemble (in half, in levels), doub (mosaic, in assemble, in half)
int oracle_denoise_nodes(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip,
    const oracle_params_t *p, const float *const in[6], float *const out[7], oracle_decisions_t *dec)
{
  if(!mosaic || !ip || !p || p->dn_strength <= 0.0f || ip->filters == 0) return 1;
  img_t<float> raw(wd, ht, 1);
  for(size_t i = 0; i < (size_t)wd * ht; i++) raw.d[i] = float(mosaic[i]) / 65535.0f;
  float black[4], white[4], wb[4];
  for(int k = 0; k < 4; k++)
  {
    black[k] = ip->black[k] / 65535.0f; white[k] = ip->white[k] / 65535.0f; wb[k] = ip->whitebalance[k];
  }
  const int crop[4] = { (int)ip->crop_aabb[0], (int)ip->crop_aabb[1], (int)ip->crop_aabb[2], (int)ip->crop_aabb[3] };
  const int W = crop[2] - crop[0], H = crop[3] - crop[1];
  const int block = ip->filters == 9u ? 3 : 2;
  const int hw = W / block, hh = H / block;
  const float edges[4] = { p->dn_edges[0], p->dn_edges[1], p->dn_edges[2], p->dn_edges[3] };
  const int zc[4] = { 0, 0, 0, 0 };
  g_dec = dec;
  img_t<float> s[5];
  for(int i = 0; i < 5; i++) s[i] = from_float<float>(in[i], hw, hh, 4);
  const img_t<float> as_in = from_float<float>(in[5], hw, hh, 4);
  img_t<float> o = denoise_half(raw, hw, hh, crop, white[1], ip->filters);
  to_float(o, out[0]);
  o = denoise_downcov(s[0], hw, hh, zc);
  to_float(o, out[1]);
  for(int l = 1; l < 4; l++)
  {
    o = denoise_down(s[l], hw, hh, zc, black[1], white[1], ip->noise_a, ip->noise_b, edges, l, block);
    to_float(o, out[l + 1]);
  }
  o = denoise_assemble(s, hw, hh, zc, wb, black, white, ip->noise_a, ip->noise_b, ip->filters, p->dn_strength,
      p->dn_luma, edges);
  to_float(o, out[5]);
  o = denoise_doub(raw, as_in, s[0], W, H, crop, black, white, ip->filters, ip->noise_a, ip->noise_b,
      p->dn_strength, p->dn_luma, p->dn_detail, edges);
  to_float_ch(o, 1, out[6]);
  g_dec = nullptr;
  return 0;
}

int oracle_develop_from_f32(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip,
    const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec, int start, const float *input)
{
  g_dec = dec;
  g_inj.start = start; g_inj.img = input;
  const int r = develop<float>(mosaic, wd, ht, ip, p, out);
  g_inj.start = 0; g_inj.img = nullptr;
  g_dec = nullptr;
  return r;
}

int oracle_develop_dec_f64(const uint16_t *mosaic, int wd, int ht,
    const oracle_img_param_t *ip, const oracle_params_t *p, oracle_stages_t *out, oracle_decisions_t *dec)
{
  g_dec = dec;
  const int r = develop<double>(mosaic, wd, ht, ip, p, out);
  g_dec = nullptr;
  return r;
}

void oracle_gauss_decisions(const float *mosaic, int wd, int ht, uint32_t filters, uint8_t *dec, float *margin)
{ // demosaic/gauss.comp on a given (hilite output) mosaic, the decisions only
  img_t<float> in(wd, ht, 1);
  for(size_t i = 0; i < (size_t)wd * ht; i++) in.d[i] = mosaic[i];
  oracle_decisions_t d;
  memset(&d, 0, sizeof(d));
  d.gauss = dec; d.gauss_margin = margin;
  g_dec = &d;
  const int block = filters == 9u ? 3 : 2;
  demosaic_gauss(in, wd / block, ht / block, filters);
  g_dec = nullptr;
}

void oracle_scene(int wd, int ht, uint32_t seed, uint32_t image_id, uint32_t filters, float black, float white,
    float noise_a, float noise_b, const float wb[3], float pan_x, float pan_y, uint16_t *out)
{ // the benchmark's seeded scene, from the recipe the library also generates on the device
  scene_layout_t s;
  scene_layout_make(&s, wd, ht, seed, image_id, filters, black, white, noise_a, noise_b, wb, pan_x, pan_y);
  OMP_FOR
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++) out[(size_t)y * wd + x] = scene_pixel(&s, x, y);
}

void oracle_crop_commit(int wd, int ht, const float perspect[8], const float pcrop[4], float rotate,
    uint32_t orientation, float block[20], int *out_wd, int *out_ht)
{ // crop/main.c:228-275 (modify_roi_in/out at full resolution) and :276-343 (commit_params)
  float crop[4], rot;
  crop_rot(orientation, (float)wd, (float)ht, pcrop, rotate, crop, &rot);
  const float cw = crop[1] - crop[0], ch = crop[3] - crop[2];
  *out_wd = (int)(uint32_t)std::min(32768.0f, (float)(uint32_t)wd * cw);
  *out_ht = (int)(uint32_t)std::min(32768.0f, (float)(uint32_t)ht * ch);
  // the homography taking the axis aligned quad (a,b) (A,b) (A,B) (a,B) to the given one
  // (P. Heckbert, "Fundamentals of Texture Mapping and Image Warping", 1989, pp. 17-21)
  float q[8];
  for(int k = 0; k < 4; k++) { q[2 * k] = (float)(uint32_t)wd * perspect[2 * k]; q[2 * k + 1] = (float)(uint32_t)ht * perspect[2 * k + 1]; }
  const float u[8] = { q[0], q[1], q[2], q[1], q[2], q[7], q[0], q[7] };
  double M[64], r[9];
  for(int k = 0; k < 4; k++)
  {
    double *ex = M + 8 * k, *ey = M + 8 * (k + 4);
    const float ux = u[2 * k], uy = u[2 * k + 1];
    ex[0] = ux; ex[1] = uy; ex[2] = 1; ex[3] = 0; ex[4] = 0; ex[5] = 0;
    ex[6] = -q[2 * k] * ux; ex[7] = -q[2 * k] * uy;             // float products, as the reference
    ey[0] = 0; ey[1] = 0; ey[2] = 0; ey[3] = ux; ey[4] = uy; ey[5] = 1;
    ey[6] = -q[2 * k + 1] * ux; ey[7] = -q[2 * k + 1] * uy;
    r[k] = q[2 * k]; r[k + 4] = q[2 * k + 1];
  }
  r[8] = 1.0;
  solve_pivoted(M, r, 8);
  const int col[12] = { 0, 3, 6, -1, 1, 4, 7, -1, 2, 5, 8, -1 };   // padded column major
  for(int k = 0; k < 12; k++) block[k] = col[k] < 0 ? 0.0f : (float)r[col[k]];
  const float rad = rot * 3.1415629 / 180.0f;
  block[12] = cosf(rad); block[13] = sinf(rad);
  block[14] = -sinf(rad); block[15] = cosf(rad);
  for(int k = 0; k < 4; k++) block[16 + k] = crop[k];
}

void oracle_noop(const uint16_t *mosaic, int wd, int ht, const oracle_img_param_t *ip, float *out)
{
  img_t<float> raw(wd, ht, 1);
  for(size_t i = 0; i < (size_t)wd * ht; i++) raw.d[i] = float(mosaic[i]) / 65535.0f;
  float black[4], white[4];
  for(int k = 0; k < 4; k++) { black[k] = ip->black[k] / 65535.0f; white[k] = ip->white[k] / 65535.0f; }
  const int crop[4] = { (int)ip->crop_aabb[0], (int)ip->crop_aabb[1], (int)ip->crop_aabb[2], (int)ip->crop_aabb[3] };
  img_t<float> o = denoise_noop(raw, (int)(crop[2] - crop[0]), (int)(crop[3] - crop[1]), crop, black, white);
  to_float_ch(o, 1, out);
}

void oracle_hist(const float *rgba, int wd, int ht, uint32_t *h)
{
  img_t<float> im(wd, ht, 4);
  memcpy(im.d.data(), rgba, sizeof(float) * 4 * (size_t)wd * ht);
  hist(im, h);
}

// hist/collect.comp:13-26, the rgb waveform (its arithmetic without contraction;
// float to unsigned saturates: negative and NaN to 0, as GPUs convert)
void oracle_waveform(const float *rgba, int wd, int ht, int wo, int ho, uint32_t *out)
{
  memset(out, 0, sizeof(uint32_t) * (size_t)wo * ho);
  const float scale = (float)wo / (float)wd;
  auto row = [&](float v) -> uint32_t {
    const float t = (1.0f - v) * (float)ho + 0.5f;
    const uint32_t u = t >= 4294967296.0f ? 0xffffffffu : (t > 0.0f ? (uint32_t)t : 0u);
    return std::min(u, (uint32_t)(ho - 1));
  };
  for(int y = 0; y < ht; y++) for(int x = 0; x < wd; x++)
  {
    const float *p = rgba + 4 * ((size_t)y * wd + x);
    const int c = std::min(std::max((int)(scale * (float)x), 0), wo - 1);
    out[(size_t)row(p[0]) * wo + c] += 1u;
    out[(size_t)row(p[1]) * wo + c] += 1024u;
    out[(size_t)row(p[2]) * wo + c] += 1048576u;
  }
}

int oracle_cfa_colour(uint32_t filters, int x, int y)
{
  if(filters == 9) return cfa_xtrans(x + 6, y + 6);
  return cfa_bayer(x, y);
}

float oracle_f16(float v) { return f16r(v); }

} // extern "C"
