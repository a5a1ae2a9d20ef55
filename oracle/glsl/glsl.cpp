#include <cstring>
// Sampler, image and storage model of glsl.hpp (test infrastructure only).
#include "glsl.hpp"
#include <ucontext.h>
#include <vector>

namespace glsl {

thread_local uvec3 gl_GlobalInvocationID;
thread_local uvec3 gl_LocalInvocationID;
thread_local uvec3 gl_WorkGroupID;
thread_local uint gl_LocalInvocationIndex;
thread_local int glsl_bar_, glsl_phase_;

float half_to_float(uint16_t h)
{
  const uint32_t s = (h >> 15) & 1, e = (h >> 10) & 0x1f, m = h & 0x3ff;
  float v;
  if(e == 0) v = std::ldexp((float)m, -24);
  else if(e == 31) v = m ? NAN : INFINITY;
  else v = std::ldexp((float)(m | 0x400), (int)e - 25);
  return s ? -v : v;
}

float f16_round(float v)
{ // IEEE binary16 round to nearest even
  if(std::isnan(v) || std::isinf(v)) return v;
  const float a = std::fabs(v);
  if(a >= 65520.0f) return std::copysign(INFINITY, v);
  if(a < 6.103515625e-05f) return std::copysign(std::ldexp(std::nearbyint(std::ldexp(a, 24)), -24), v);
  int e;
  const float f = std::frexp(a, &e);
  return std::copysign(std::ldexp(std::nearbyint(std::ldexp(f, 11)), e - 11), v);
}

uint16_t float_to_half(float f)
{
  const float r = f16_round(f);
  uint16_t s = std::signbit(r) ? 0x8000 : 0;
  const float a = std::fabs(r);
  if(std::isnan(r)) return 0x7e00;
  if(std::isinf(a)) return s | 0x7c00;
  if(a < 6.103515625e-05f) return s | (uint16_t)std::ldexp(a, 24);
  int e;
  const float m = std::frexp(a, &e); // a = m 2^e, m in [0.5,1)
  return s | (uint16_t)(((e + 14) << 10) | ((uint16_t)std::ldexp(m, 11) & 0x3ff));
}

int mirror(int i, int n)
{
  const int m = 2 * n;
  int t = i % m;
  if(t < 0) t += m;
  return t < n ? t : m - 1 - t;
}

vec4 texel(const image_t *im, int x, int y)
{
  const float *p = im->data + ((size_t)y * im->w + x) * im->c;
  vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
  for(int k = 0; k < im->c && k < 4; k++) r.d[k] = p[k];
  return r;
}

vec4 texelFetch(const sampler2D &s, const ivec2 &p, int)
{
  if(!s.im || p.x < 0 || p.y < 0 || p.x >= s.im->w || p.y >= s.im->h) return vec4(0.0f);
  return texel(s.im, p.x, p.y);
}
uvec4 texelFetch(const usampler2D &s, const ivec2 &p, int)
{
  if(!s.im || p.x < 0 || p.y < 0 || p.x >= s.im->w || p.y >= s.im->h) return uvec4(0u);
  const vec4 v = texel(s.im, p.x, p.y);
  uvec4 r;
  for(int k = 0; k < 4; k++) r.d[k] = floatBitsToUint(v.d[k]);
  return r;
}

// sample position in texel space, snapped to 1/256 texel
static inline float snap(float x) { return std::floor(x * 256.0f + 0.5f) / 256.0f; }

vec4 texture(const sampler2D &s, const vec2 &uv)
{
  const image_t *im = s.im;
  if(!im || im->w <= 0 || im->h <= 0) return vec4(0.0f);
  const float x = snap(uv.x * (float)im->w - 0.5f), y = snap(uv.y * (float)im->h - 0.5f);
  const float fx = std::floor(x), fy = std::floor(y);
  const float ax = x - fx, ay = y - fy;
  const int x0 = (int)fx, y0 = (int)fy;
  const int X0 = mirror(x0, im->w), X1 = mirror(x0 + 1, im->w), Y0 = mirror(y0, im->h), Y1 = mirror(y0 + 1, im->h);
  const vec4 t00 = texel(im, X0, Y0), t10 = texel(im, X1, Y0), t01 = texel(im, X0, Y1), t11 = texel(im, X1, Y1);
  vec4 r;
  for(int k = 0; k < 4; k++)
    r.d[k] = (t00.d[k] * (1.0f - ax) + t10.d[k] * ax) * (1.0f - ay) + (t01.d[k] * (1.0f - ax) + t11.d[k] * ax) * ay;
  return r;
}
vec4 textureLod(const sampler2D &s, const vec2 &uv, float) { return texture(s, uv); }

vec4 textureGather(const sampler2D &s, const vec2 &uv, int comp)
{
  const image_t *im = s.im;
  const float x = snap(uv.x * (float)im->w - 0.5f), y = snap(uv.y * (float)im->h - 0.5f);
  const int x0 = (int)std::floor(x), y0 = (int)std::floor(y);
  const int X0 = mirror(x0, im->w), X1 = mirror(x0 + 1, im->w), Y0 = mirror(y0, im->h), Y1 = mirror(y0 + 1, im->h);
  return vec4(texel(im, X0, Y1).d[comp], texel(im, X1, Y1).d[comp], texel(im, X1, Y0).d[comp], texel(im, X0, Y0).d[comp]);
}

ivec2 textureSize(const sampler2D &s, int) { return s.im ? ivec2(s.im->w, s.im->h) : ivec2(0); }
ivec2 textureSize(const usampler2D &s, int) { return s.im ? ivec2(s.im->w, s.im->h) : ivec2(0); }
ivec2 imageSize(const image2D &i) { return i.im ? ivec2(i.im->w, i.im->h) : ivec2(0); }
ivec2 imageSize(const uimage2D &i) { return i.im ? ivec2(i.im->w, i.im->h) : ivec2(0); }

uint imageAtomicAdd(const uimage2D &i, const ivec2 &p, uint v)
{ // r32ui: the u32 stored in the float slot's bits
  image_t *im = i.im;
  if(!im || p.x < 0 || p.y < 0 || p.x >= im->w || p.y >= im->h) return 0;
  float *d = im->data + ((size_t)p.y * im->w + p.x) * im->c;
  return __atomic_fetch_add(reinterpret_cast<uint32_t *>(d), v, __ATOMIC_RELAXED);
}

float imageAtomicAdd(const image2D &i, const ivec2 &p, float v)
{ // r32f
  image_t *im = i.im;
  if(!im || p.x < 0 || p.y < 0 || p.x >= im->w || p.y >= im->h) return 0.0f;
  float *d = im->data + ((size_t)p.y * im->w + p.x) * im->c;
  uint32_t *u = reinterpret_cast<uint32_t *>(d);
  uint32_t cur = __atomic_load_n(u, __ATOMIC_RELAXED), nxt;
  float f;
  do
  { // compare and swap of the sum
    memcpy(&f, &cur, 4);
    const float s = f + v;
    memcpy(&nxt, &s, 4);
  }
  while(!__atomic_compare_exchange_n(u, &cur, nxt, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
  return f;
}

void imageStore(const image2D &i, const ivec2 &p, const vec4 &v)
{
  image_t *im = i.im;
  if(!im || p.x < 0 || p.y < 0 || p.x >= im->w || p.y >= im->h) return;
  float *d = im->data + ((size_t)p.y * im->w + p.x) * im->c;
  for(int k = 0; k < im->c && k < 4; k++)
  {
    float x = v.d[k];
    if(im->fmt == 0) x = f16_round(x);
    else if(im->fmt == 2) x = std::nearbyint(std::fmin(std::fmax(x, 0.0f), 1.0f) * 65535.0f) / 65535.0f;
    d[k] = x;
  }
}

vec4 imageLoad(const image2D &i, const ivec2 &p)
{
  image_t *im = i.im;
  if(!im || p.x < 0 || p.y < 0 || p.x >= im->w || p.y >= im->h) return vec4(0.0f);
  return texel(im, p.x, p.y);
}

// cooperative workgroups: one ucontext per invocation
namespace {
struct coop_t
{
  ucontext_t sched;
  std::vector<ucontext_t> inv;
  std::vector<std::vector<char>> stack;
  std::vector<char> done;
  int cur = -1;
  void (*fn)() = nullptr;
};
thread_local coop_t *g_coop = nullptr;
void coop_entry()
{
  g_coop->fn();
  g_coop->done[g_coop->cur] = 1;
}   // returns to uc_link: the scheduler
} // namespace

void barrier()
{
  if(g_coop) swapcontext(&g_coop->inv[g_coop->cur], &g_coop->sched);
}
void memoryBarrierShared() {}

void run_workgroups_coop(int GX, int GY, int GZ, int LX, int LY, void (*fn)())
{
  const int N = LX * LY;
#pragma omp parallel
  {
    coop_t c;
    c.inv.resize(N);
    c.stack.assign(N, std::vector<char>(256 * 1024));
    c.done.assign(N, 0);
    c.fn = fn;
    g_coop = &c;
#pragma omp for collapse(3) schedule(static)
    for(int z = 0; z < GZ; z++) for(int wy = 0; wy < GY; wy++) for(int wx = 0; wx < GX; wx++)
    {
      for(int k = 0; k < N; k++)
      {
        getcontext(&c.inv[k]);
        c.inv[k].uc_stack.ss_sp = c.stack[k].data();
        c.inv[k].uc_stack.ss_size = c.stack[k].size();
        c.inv[k].uc_link = &c.sched;
        makecontext(&c.inv[k], coop_entry, 0);
        c.done[k] = 0;
      }
      for(bool any = true; any;)
      { // one barrier phase: resume every invocation until it waits or returns
        any = false;
        for(int k = 0; k < N; k++)
        {
          if(c.done[k]) continue;
          const int lx = k % LX, ly = k / LX;
          gl_GlobalInvocationID = uvec3((uint)(wx * LX + lx), (uint)(wy * LY + ly), (uint)z);
          gl_LocalInvocationID = uvec3((uint)lx, (uint)ly, 0u);
          gl_WorkGroupID = uvec3((uint)wx, (uint)wy, (uint)z);
          gl_LocalInvocationIndex = (uint)k;
          c.cur = k;
          swapcontext(&c.sched, &c.inv[k]);
          any = true;
        }
      }
    }
    g_coop = nullptr;
  }
}

} // namespace glsl
