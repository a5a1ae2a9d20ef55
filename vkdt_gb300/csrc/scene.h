// Seeded synthetic raw scene: smooth colour gradients, 64 hard-edged
// rectangles and 32 sine gratings in camera-linear space, sampled on the CFA,
// with Poisson-Gaussian noise in DN and 2% of the pixels clipped to white.
// The same code runs on the host (tests) and on the device (benchmarks).
#pragma once
#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define SCENE_HD __host__ __device__ __forceinline__
#else
#define SCENE_HD static inline
#endif

#define SCENE_NRECT 64
#define SCENE_NGRAT 32

typedef struct scene_layout_t
{
  int32_t  wd, ht;
  uint32_t seed, image_id, filters;
  float    black, white, noise_a, noise_b;
  float    iwb[3];                 // 1 / white balance
  float    pan_x, pan_y;
  float    grad[3][6];             // c0 + cu u + cv v + cuv u v + cuu u^2 + cvv v^2
  float    rect[SCENE_NRECT][7];   // x0 y0 x1 y1 r g b (scene pixels)
  float    grat[SCENE_NGRAT][9];   // x0 y0 x1 y1 freq cos sin phase contrast
  float    clip_thr;               // scene luminance of the brightest 10%
}
scene_layout_t;

// Philox-4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC 2011)
SCENE_HD void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1)
{
  for(int r = 0; r < 10; r++)
  {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}
SCENE_HD float u01(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

// a stream of uniforms keyed by (seed, image, purpose, index)
typedef struct scene_rng_t { uint32_t c[4]; uint32_t out[4]; int used; uint32_t k0, k1; } scene_rng_t;
SCENE_HD void rng_init(scene_rng_t *r, uint32_t seed, uint32_t image, uint32_t a, uint32_t b)
{
  r->c[0] = a; r->c[1] = b; r->c[2] = image; r->c[3] = 0;
  r->k0 = seed; r->k1 = 0x5eedu ^ image;
  r->used = 4;
}
SCENE_HD float rng_next(scene_rng_t *r)
{
  if(r->used == 4)
  {
    r->out[0] = r->c[0]; r->out[1] = r->c[1]; r->out[2] = r->c[2]; r->out[3] = r->c[3];
    philox4x32(r->out, r->k0, r->k1);
    r->c[3]++;
    r->used = 0;
  }
  return u01(r->out[r->used++]);
}

// bayer rggb at (0,0) or x-trans (the pattern demosaic/splat.comp:167-195 implies)
SCENE_HD int scene_cfa(uint32_t filters, int x, int y)
{
  if(filters == 9)
  {
    const int X = x + 6, Y = y + 6;
    const int bt = ((X / 3 + Y / 3) & 1);
    const int px = X % 3, py = Y % 3;
    if(((px + py) & 1) == 0) return 1;
    if(bt ^ (py == 1)) return 2;
    return 0;
  }
  const int ox = x & 1, oy = y & 1;
  if(ox != oy) return 1;
  return ox ? 2 : 0;
}

// noise-free scene colour at scene coordinates (x, y), channel c
SCENE_HD float scene_colour(const scene_layout_t *s, float x, float y, int c)
{
  const float u = x / (float)(s->wd > 1 ? s->wd - 1 : 1), v = y / (float)(s->ht > 1 ? s->ht - 1 : 1);
  const float *g = s->grad[c];
  float val = g[0] + g[1] * u + g[2] * v + g[3] * u * v + g[4] * u * u + g[5] * v * v;
  val = fminf(fmaxf(val, 0.05f), 0.6f);
  for(int i = 0; i < SCENE_NRECT; i++)
  {
    const float *r = s->rect[i];
    if(x >= r[0] && x < r[2] && y >= r[1] && y < r[3]) val = r[4 + c];
  }
  for(int i = 0; i < SCENE_NGRAT; i++)
  {
    const float *q = s->grat[i];
    if(x >= q[0] && x < q[2] && y >= q[1] && y < q[3])
    {
      const float ph = 6.28318530718f * q[4] * (x * q[5] + y * q[6]) + q[7];
      val *= 1.0f + q[8] * sinf(ph);
    }
  }
  // keep the scene below the sensor's white so the clipped pixels are the
  // seeded 2% only
  return fminf(fmaxf(val, 0.0f), 0.92f);
}

SCENE_HD float scene_luma(const scene_layout_t *s, float x, float y)
{
  return 0.25f * scene_colour(s, x, y, 0) + 0.5f * scene_colour(s, x, y, 1) + 0.25f * scene_colour(s, x, y, 2);
}

// Poisson sample: inversion for small means, PTRS (W. Hoermann, "The
// transformed rejection method for generating Poisson random variables",
// Insurance: Mathematics and Economics 12, 1993) for lam >= 10.
SCENE_HD float scene_poisson(scene_rng_t *r, float lam)
{
  if(!(lam > 0.0f)) return 0.0f;
  if(lam < 10.0f)
  {
    const float L = expf(-lam);
    float p = 1.0f;
    int k = 0;
    for(int it = 0; it < 200; it++)
    {
      p *= rng_next(r);
      if(p <= L) break;
      k++;
    }
    return (float)k;
  }
  const float slam = sqrtf(lam), loglam = logf(lam);
  const float b = 0.931f + 2.53f * slam;
  const float a = -0.059f + 0.02483f * b;
  const float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
  const float vr = 0.9277f - 3.6224f / (b - 2.0f);
  for(int it = 0; it < 64; it++)
  {
    const float U = rng_next(r) - 0.5f;
    const float V = rng_next(r);
    const float us = 0.5f - fabsf(U);
    const float k = floorf((2.0f * a / us + b) * U + lam + 0.43f);
    if(us >= 0.07f && V <= vr) return k;
    if(k < 0.0f || (us < 0.013f && V > us)) continue;
    if(logf(V) + logf(invalpha) - logf(a / (us * us) + b) <= -lam + k * loglam - lgammaf(k + 1.0f)) return k;
  }
  return floorf(lam + 0.5f); // not reached in practice; bounded loop
}

SCENE_HD float scene_gauss(scene_rng_t *r)
{ // Box-Muller
  const float u1 = rng_next(r), u2 = rng_next(r);
  return sqrtf(-2.0f * logf(1.0f - u1)) * cosf(6.28318530718f * u2);
}

// one raw DN value of the mosaic at pixel (x, y)
SCENE_HD uint16_t scene_pixel(const scene_layout_t *s, int x, int y)
{
  const float sx = (float)x + s->pan_x, sy = (float)y + s->pan_y;
  const int c = scene_cfa(s->filters, x, y);
  const float cam = scene_colour(s, sx, sy, c) * s->iwb[c];
  const float range = s->white - s->black;
  const float sig = fmaxf(0.0f, cam) * range;
  scene_rng_t r;
  rng_init(&r, s->seed, s->image_id, (uint32_t)x, (uint32_t)y);
  const float pois = s->noise_b > 0.0f ? s->noise_b * scene_poisson(&r, sig / s->noise_b) : sig;
  float dn = s->black + pois + sqrtf(fmaxf(s->noise_a, 0.0f)) * scene_gauss(&r);
  const float hv = rng_next(&r);
  if(hv < 0.2f && scene_luma(s, sx, sy) >= s->clip_thr) dn = s->white;
  dn = fminf(fmaxf(dn, 0.0f), s->white);
  return (uint16_t)(dn + 0.5f);
}

#if defined(__cplusplus) && !defined(__CUDA_ARCH__)
#include <algorithm>
// the scene of a seed (host): gradients, rectangles, gratings and the clip
// threshold (the brightest 10% of the scene luminance on a 96x96 sample)
static inline void scene_layout_make(scene_layout_t *s, int32_t wd, int32_t ht, uint32_t seed, uint32_t image_id,
    uint32_t filters, float black, float white, float noise_a, float noise_b, const float wb[3], float pan_x, float pan_y)
{
  *s = scene_layout_t();
  s->wd = wd; s->ht = ht; s->seed = seed; s->image_id = image_id; s->filters = filters;
  s->black = black; s->white = white; s->noise_a = noise_a; s->noise_b = noise_b;
  for(int k = 0; k < 3; k++) s->iwb[k] = 1.0f / wb[k];
  s->pan_x = pan_x; s->pan_y = pan_y;
  scene_rng_t r;
  rng_init(&r, seed, image_id, 0xA11CEu, 0x5CE4Eu);
  const float W = (float)wd, H = (float)ht;
  for(int c = 0; c < 3; c++)
  {
    s->grad[c][0] = 0.05f + 0.55f * rng_next(&r);
    for(int k = 1; k < 6; k++) s->grad[c][k] = 0.4f * (rng_next(&r) - 0.5f);
  }
  for(int i = 0; i < SCENE_NRECT; i++)
  {
    const float w = (0.02f + 0.23f * rng_next(&r)) * W, h = (0.02f + 0.23f * rng_next(&r)) * W;
    const float x0 = rng_next(&r) * (W - w), y0 = rng_next(&r) * fmaxf(H - h, 1.0f);
    float *q = s->rect[i];
    q[0] = x0; q[1] = y0; q[2] = x0 + w; q[3] = y0 + h;
    for(int c = 0; c < 3; c++) q[4 + c] = 0.02f + 0.93f * rng_next(&r);
  }
  for(int i = 0; i < SCENE_NGRAT; i++)
  {
    const float w = (0.05f + 0.2f * rng_next(&r)) * W, h = (0.05f + 0.2f * rng_next(&r)) * H;
    const float x0 = rng_next(&r) * (W - w), y0 = rng_next(&r) * (H - h);
    float *q = s->grat[i];
    q[0] = x0; q[1] = y0; q[2] = x0 + w; q[3] = y0 + h;
    q[4] = 0.05f + 0.4f * rng_next(&r);
    const float th = 6.28318530718f * rng_next(&r);
    q[5] = cosf(th); q[6] = sinf(th);
    q[7] = 6.28318530718f * rng_next(&r);
    q[8] = 0.1f + 0.4f * rng_next(&r);
  }
  static const int NS = 96;
  float lum[NS * NS];
  for(int j = 0; j < NS; j++) for(int i = 0; i < NS; i++)
    lum[j * NS + i] = scene_luma(s, (i + 0.5f) / NS * W + s->pan_x, (j + 0.5f) / NS * H + s->pan_y);
  std::sort(lum, lum + NS * NS);
  s->clip_thr = lum[(size_t)(0.9 * NS * NS)];
}
#endif
