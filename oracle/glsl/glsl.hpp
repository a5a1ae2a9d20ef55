// A C++ emulation of the GLSL used by the vkdt compute shaders, so the
// reference's own shader sources (translated mechanically by translate.py)
// compile and run on the CPU. TEST INFRASTRUCTURE ONLY: it is the build of
// the reference that pins the oracle restatement (oracle/oracle.cpp).
//
// Semantics modelled after a GPU running the shaders under vkdt's Vulkan
// setup (src/qvk/qvk.c:596-611, src/pipe/graph-run-nodes-allocate.h):
//  - texture()/textureLod(): LINEAR filtering, MIRRORED_REPEAT wrap,
//    normalised coordinates; the sample position is snapped to 8 bits of
//    sub-texel precision before the weights are taken (subTexelPrecisionBits
//    of current GPUs), weights and blend in FP32.
//  - textureGather(.., 0): component 0 of the 2x2 quad, order (i0,j1) (i1,j1)
//    (i1,j0) (i0,j0).
//  - texelFetch(): out of range reads return 0 (undefined in the reference).
//  - one-channel images read as (r, 0, 0, 1).
//  - imageStore(): f16 images round to nearest even, unorm16 images clamp and
//    round; out of range stores are dropped.
//  - min/max/clamp: IEEE minNum/maxNum (a NaN operand yields the other), as
//    GPU min/max instructions do.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace glsl {

typedef unsigned int uint;

template<class T, int N> struct V;

// swizzle proxy over the storage of a vector of N components of type T
template<class T, int N, int... I> struct swz
{
  T d[N];
  static constexpr int M = sizeof...(I);
  using vt = V<T, M>;
  operator vt() const { return vt(d[I]...); }
  swz &operator=(const vt &v)
  {
    const int idx[] = { I... };
    for(int k = 0; k < M; k++) d[idx[k]] = v.d[k];
    return *this;
  }
  swz &operator=(const swz &o) { return *this = vt(o); }
  template<int N2, int... J> swz &operator=(const swz<T, N2, J...> &o) { return *this = vt(o); }
  T operator[](int k) const { const int idx[] = { I... }; return d[idx[k]]; }
  template<class U> swz &operator+=(const U &u);
  template<class U> swz &operator-=(const U &u);
  template<class U> swz &operator*=(const U &u);
  template<class U> swz &operator/=(const U &u);
};

#include "glsl_swizzle.inc"   // generated: the swizzle members of V<T,2..4>

template<class T> struct V<T, 2>
{
  union { T d[2]; struct { T x, y; }; struct { T r, g; }; struct { T s, t; }; GLSL_SWIZZLES_2 };
  V() : d{ T(0), T(0) } {}
  V(const V &o) { d[0] = o.d[0]; d[1] = o.d[1]; }
  V &operator=(const V &o) { T a = o.d[0], b = o.d[1]; d[0] = a; d[1] = b; return *this; }
  template<class... A> explicit V(const A &...a);
  template<class U> V(const V<U, 2> &o) { d[0] = T(o.d[0]); d[1] = T(o.d[1]); }
  T &operator[](int k) { return d[k]; }
  const T &operator[](int k) const { return d[k]; }
};
template<class T> struct V<T, 3>
{
  union { T d[3]; struct { T x, y, z; }; struct { T r, g, b; }; struct { T s, t, p; }; GLSL_SWIZZLES_3 };
  V() : d{ T(0), T(0), T(0) } {}
  V(const V &o) { for(int k = 0; k < 3; k++) d[k] = o.d[k]; }
  V &operator=(const V &o) { T a[3] = { o.d[0], o.d[1], o.d[2] }; for(int k = 0; k < 3; k++) d[k] = a[k]; return *this; }
  template<class... A> explicit V(const A &...a);
  template<class U> V(const V<U, 3> &o) { for(int k = 0; k < 3; k++) d[k] = T(o.d[k]); }
  T &operator[](int k) { return d[k]; }
  const T &operator[](int k) const { return d[k]; }
};
template<class T> struct V<T, 4>
{
  union { T d[4]; struct { T x, y, z, w; }; struct { T r, g, b, a; }; struct { T s, t, p, q; }; GLSL_SWIZZLES_4 };
  V() : d{ T(0), T(0), T(0), T(0) } {}
  V(const V &o) { for(int k = 0; k < 4; k++) d[k] = o.d[k]; }
  V &operator=(const V &o) { T a[4] = { o.d[0], o.d[1], o.d[2], o.d[3] }; for(int k = 0; k < 4; k++) d[k] = a[k]; return *this; }
  template<class... A> explicit V(const A &...a);
  template<class U> V(const V<U, 4> &o) { for(int k = 0; k < 4; k++) d[k] = T(o.d[k]); }
  T &operator[](int k) { return d[k]; }
  const T &operator[](int k) const { return d[k]; }
};

typedef V<float, 2> vec2; typedef V<float, 3> vec3; typedef V<float, 4> vec4;
typedef V<int, 2> ivec2;  typedef V<int, 3> ivec3;  typedef V<int, 4> ivec4;
typedef V<uint, 2> uvec2; typedef V<uint, 3> uvec3; typedef V<uint, 4> uvec4;
typedef V<bool, 2> bvec2; typedef V<bool, 3> bvec3; typedef V<bool, 4> bvec4;
typedef V<uint8_t, 2> u8vec2; typedef V<uint8_t, 4> u8vec4;   // GL_EXT_shader_explicit_arithmetic_types_int8

// ------------------------------------------------------------------ traits
template<class A> struct vinfo { static constexpr bool is = false; static constexpr int n = 1; using E = A; };
template<class T, int N> struct vinfo<V<T, N>> { static constexpr bool is = true; static constexpr int n = N; using E = T; };
template<class T, int N, int... I> struct vinfo<swz<T, N, I...>> { static constexpr bool is = true; static constexpr int n = sizeof...(I); using E = T; };
template<class A> struct vinfo<const A> : vinfo<A> {};
template<class A> struct vinfo<A &> : vinfo<A> {};
template<class A> using vec_of = V<typename vinfo<A>::E, vinfo<A>::n>;
template<class A> constexpr bool is_vec = vinfo<std::decay_t<A>>::is;
template<class A> inline auto tov(const A &a)
{
  if constexpr(vinfo<A>::is) return vec_of<A>(a);
  else return a;
}

// constructor: flatten scalar and vector arguments, a single scalar broadcasts
template<class T, class A> inline void push_arg(T *tmp, int &k, int n, const A &a)
{
  if constexpr(vinfo<A>::is)
  { // component access, no conversion (a swizzle converts through this constructor)
    for(int i = 0; i < vinfo<A>::n && k < n; i++) tmp[k++] = T(a[i]);
  }
  else if(k < n) tmp[k++] = T(a);
}
#define GLSL_VCTOR(N) \
  template<class T> template<class... A> V<T, N>::V(const A &...a) \
  { T tmp[N] = {}; int k = 0; (push_arg(tmp, k, N, a), ...); \
    if(k == 1) for(int i = 1; i < N; i++) tmp[i] = tmp[0]; \
    for(int i = 0; i < N; i++) d[i] = tmp[i]; }
GLSL_VCTOR(2) GLSL_VCTOR(3) GLSL_VCTOR(4)
#undef GLSL_VCTOR

// ------------------------------------------------------------------ arithmetic
template<class F, class T1, class T2, int N> inline auto vop(F f, const V<T1, N> &a, const V<T2, N> &b)
{ V<decltype(f(a.d[0], b.d[0])), N> r; for(int k = 0; k < N; k++) r.d[k] = f(a.d[k], b.d[k]); return r; }
template<class F, class T1, class S, int N> inline auto vop(F f, const V<T1, N> &a, const S &b)
{ V<decltype(f(a.d[0], b)), N> r; for(int k = 0; k < N; k++) r.d[k] = f(a.d[k], b); return r; }
template<class F, class S, class T2, int N> inline auto vop(F f, const S &a, const V<T2, N> &b)
{ V<decltype(f(a, b.d[0])), N> r; for(int k = 0; k < N; k++) r.d[k] = f(a, b.d[k]); return r; }

#define GLSL_BINOP(op) \
  template<class A, class B, class = std::enable_if_t<is_vec<A> || is_vec<B>>> \
  inline auto operator op(const A &a, const B &b) { return vop([](auto x, auto y) { return x op y; }, tov(a), tov(b)); }
GLSL_BINOP(+) GLSL_BINOP(-) GLSL_BINOP(/) GLSL_BINOP(%) GLSL_BINOP(&) GLSL_BINOP(|) GLSL_BINOP(^) GLSL_BINOP(<<) GLSL_BINOP(>>)
#undef GLSL_BINOP
// vector * vector / scalar (matrix products are overloaded below and win for matrices)
template<class A, class B, class = std::enable_if_t<is_vec<A> || is_vec<B>>>
inline auto operator*(const A &a, const B &b) { return vop([](auto x, auto y) { return x * y; }, tov(a), tov(b)); }

template<class T, int N> inline V<T, N> operator-(const V<T, N> &a) { V<T, N> r; for(int k = 0; k < N; k++) r.d[k] = -a.d[k]; return r; }
template<class T, int N, int... I> inline auto operator-(const swz<T, N, I...> &a) { return -V<T, sizeof...(I)>(a); }
template<class T, int N> inline V<T, N> operator+(const V<T, N> &a) { return a; }
template<int N> inline V<bool, N> operator!(const V<bool, N> &a) { V<bool, N> r; for(int k = 0; k < N; k++) r.d[k] = !a.d[k]; return r; }

#define GLSL_CASSIGN(op) \
  template<class T, int N, class U> inline V<T, N> &operator op##=(V<T, N> &a, const U &u) \
  { a = V<T, N>(a op u); return a; }
GLSL_CASSIGN(+) GLSL_CASSIGN(-) GLSL_CASSIGN(*) GLSL_CASSIGN(/) GLSL_CASSIGN(%) GLSL_CASSIGN(&) GLSL_CASSIGN(|)
#undef GLSL_CASSIGN
template<class T, int N, int... I> template<class U> swz<T, N, I...> &swz<T, N, I...>::operator+=(const U &u) { return *this = vt(vt(*this) + u); }
template<class T, int N, int... I> template<class U> swz<T, N, I...> &swz<T, N, I...>::operator-=(const U &u) { return *this = vt(vt(*this) - u); }
template<class T, int N, int... I> template<class U> swz<T, N, I...> &swz<T, N, I...>::operator*=(const U &u) { return *this = vt(vt(*this) * u); }
template<class T, int N, int... I> template<class U> swz<T, N, I...> &swz<T, N, I...>::operator/=(const U &u) { return *this = vt(vt(*this) / u); }

template<class A, class B, class = std::enable_if_t<is_vec<A> && is_vec<B>>>
inline bool operator==(const A &a, const B &b)
{ auto x = tov(a), y = tov(b); for(int k = 0; k < vinfo<decltype(x)>::n; k++) if(!(x.d[k] == y.d[k])) return false; return true; }
template<class A, class B, class = std::enable_if_t<is_vec<A> && is_vec<B>>>
inline bool operator!=(const A &a, const B &b) { return !(a == b); }

// ------------------------------------------------------------------ matrices (column major)
template<int N> struct M
{
  V<float, N> c[N];
  M() {}
  explicit M(float s) { for(int i = 0; i < N; i++) for(int j = 0; j < N; j++) c[i].d[j] = i == j ? s : 0.0f; }
  template<class... A, class = std::enable_if_t<(sizeof...(A) == N * N)>> M(A... a)
  { const float f[] = { float(a)... }; for(int i = 0; i < N; i++) for(int j = 0; j < N; j++) c[i].d[j] = f[N * i + j]; }
  template<class... A, class = std::enable_if_t<(sizeof...(A) == N) && (N > 1)>, class = void> M(const A &...cols)
  { const V<float, N> v[] = { V<float, N>(cols)... }; for(int i = 0; i < N; i++) c[i] = v[i]; }
  V<float, N> &operator[](int i) { return c[i]; }
  const V<float, N> &operator[](int i) const { return c[i]; }
};
typedef M<2> mat2; typedef M<3> mat3; typedef M<4> mat4;
// a mat3 member of a std140 block: three columns padded to vec4
struct mat3_std140
{
  vec4 c[3];
  operator mat3() const { mat3 m; for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) m.c[i].d[j] = c[i].d[j]; return m; }
};
template<int N> inline V<float, N> operator*(const M<N> &m, const V<float, N> &v)
{ V<float, N> r; for(int j = 0; j < N; j++) { float s = 0.0f; for(int i = 0; i < N; i++) s = s + m.c[i].d[j] * v.d[i]; r.d[j] = s; } return r; }
template<int N, class A, class = std::enable_if_t<is_vec<A> && !std::is_same_v<A, V<float, N>>>>
inline V<float, N> operator*(const M<N> &m, const A &v) { return m * V<float, N>(tov(v)); }
inline vec3 operator*(const mat3_std140 &m, const vec3 &v) { return mat3(m) * v; }
template<int N> inline V<float, N> operator*(const V<float, N> &v, const M<N> &m)
{ V<float, N> r; for(int i = 0; i < N; i++) { float s = 0.0f; for(int j = 0; j < N; j++) s = s + v.d[j] * m.c[i].d[j]; r.d[i] = s; } return r; }
template<int N> inline M<N> operator*(const M<N> &a, const M<N> &b)
{ M<N> r; for(int i = 0; i < N; i++) r.c[i] = a * b.c[i]; return r; }
template<int N> inline M<N> operator*(const M<N> &a, float s) { M<N> r; for(int i = 0; i < N; i++) r.c[i] = a.c[i] * s; return r; }
template<int N> inline M<N> operator*(float s, const M<N> &a) { return a * s; }
template<int N> inline M<N> operator/(const M<N> &a, float s) { M<N> r; for(int i = 0; i < N; i++) r.c[i] = a.c[i] / s; return r; }
template<int N> inline M<N> operator+(const M<N> &a, const M<N> &b) { M<N> r; for(int i = 0; i < N; i++) r.c[i] = a.c[i] + b.c[i]; return r; }
template<int N> inline M<N> operator-(const M<N> &a, const M<N> &b) { M<N> r; for(int i = 0; i < N; i++) r.c[i] = a.c[i] - b.c[i]; return r; }
template<int N> inline M<N> &operator/=(M<N> &a, float s) { a = a / s; return a; }
template<int N> inline M<N> &operator*=(M<N> &a, float s) { a = a * s; return a; }
inline float determinant(const mat2 &m) { return m.c[0].d[0] * m.c[1].d[1] - m.c[1].d[0] * m.c[0].d[1]; }
inline float determinant(const mat3 &m)
{
  const float a = m[0][0], b = m[1][0], c = m[2][0], d = m[0][1], e = m[1][1], f = m[2][1], g = m[0][2], h = m[1][2], i = m[2][2];
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
template<int N> inline M<N> transpose(const M<N> &m) { M<N> r; for(int i = 0; i < N; i++) for(int j = 0; j < N; j++) r.c[i].d[j] = m.c[j].d[i]; return r; }

// ------------------------------------------------------------------ built-in functions
template<class F, class A> inline auto vmap(F f, const A &a)
{
  if constexpr(vinfo<A>::is) { auto v = tov(a); V<decltype(f(v.d[0])), vinfo<A>::n> r; for(int k = 0; k < vinfo<A>::n; k++) r.d[k] = f(v.d[k]); return r; }
  else return f(a);
}
// n-ary component wise with scalar broadcast; N from the first vector argument
template<class... A> constexpr int vdim() { int n = 1; ((n = (vinfo<A>::is && n == 1) ? vinfo<A>::n : n), ...); return n; }
template<class A> inline auto comp(const A &a, int k) { if constexpr(vinfo<A>::is) return tov(a).d[k]; else return a; }
template<class F, class... A> inline auto vmapn(F f, const A &...a)
{
  constexpr int n = vdim<A...>();
  if constexpr(n == 1 && !(vinfo<A>::is || ...)) return f(a...);
  else { V<decltype(f(comp(a, 0)...)), n> r; for(int k = 0; k < n; k++) r.d[k] = f(comp(a, k)...); return r; }
}

template<class X, class Y> inline auto fmin_(X x, Y y)
{
  if constexpr(std::is_integral_v<X> && std::is_integral_v<Y>) return x < y ? x : y;
  else return std::fmin((float)x, (float)y);
}
template<class X, class Y> inline auto fmax_(X x, Y y)
{
  if constexpr(std::is_integral_v<X> && std::is_integral_v<Y>) return x > y ? x : y;
  else return std::fmax((float)x, (float)y);
}

#define GLSL_F1(name, expr) \
  inline float name(float x) { return expr; } \
  template<class A, class = std::enable_if_t<is_vec<A>>> inline auto name(const A &a) { return vmap([](float x) { return name(x); }, a); }
GLSL_F1(sqrt, std::sqrt(x)) GLSL_F1(inversesqrt, 1.0f / std::sqrt(x)) GLSL_F1(exp, std::exp(x)) GLSL_F1(exp2, std::exp2(x))
GLSL_F1(log, std::log(x)) GLSL_F1(log2, std::log2(x)) GLSL_F1(sin, std::sin(x)) GLSL_F1(cos, std::cos(x)) GLSL_F1(tan, std::tan(x))
GLSL_F1(asin, std::asin(x)) GLSL_F1(acos, std::acos(x)) GLSL_F1(sinh, std::sinh(x)) GLSL_F1(cosh, std::cosh(x)) GLSL_F1(tanh, std::tanh(x))
GLSL_F1(asinh, std::asinh(x)) GLSL_F1(floor, std::floor(x)) GLSL_F1(ceil, std::ceil(x)) GLSL_F1(fract, x - std::floor(x))
GLSL_F1(trunc, std::trunc(x)) GLSL_F1(round, std::round(x)) GLSL_F1(roundEven, std::nearbyint(x))
GLSL_F1(radians, x * 0.017453292519943295f) GLSL_F1(degrees, x * 57.29577951308232f)
#undef GLSL_F1
inline float atan(float x) { return std::atan(x); }
inline float atan(float y, float x) { return std::atan2(y, x); }
template<class A, class B, class = std::enable_if_t<is_vec<A> || is_vec<B>>> inline auto atan(const A &y, const B &x) { return vmapn([](float a, float b) { return std::atan2(a, b); }, y, x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float abs(float x) { return std::fabs(x); }
inline float abs(double x) { return std::fabs((float)x); }
template<class A, class = std::enable_if_t<is_vec<A>>> inline auto abs(const A &a) { return vmap([](auto x) { return abs(x); }, a); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline int sign(int x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }
template<class A, class = std::enable_if_t<is_vec<A>>> inline auto sign(const A &a) { return vmap([](auto x) { return sign(x); }, a); }
template<class X, class Y> inline auto pow(X x, Y y) { return vmapn([](float a, float b) { return std::pow(a, b); }, x, y); }
template<class X, class Y> inline auto mod(X x, Y y) { return vmapn([](float a, float b) { return a - b * std::floor(a / b); }, x, y); }
template<class X, class Y> inline auto min(X x, Y y) { return vmapn([](auto a, auto b) { return fmin_(a, b); }, x, y); }
template<class X, class Y> inline auto max(X x, Y y) { return vmapn([](auto a, auto b) { return fmax_(a, b); }, x, y); }
template<class X, class L, class H> inline auto clamp(X x, L lo, H hi)
{ return vmapn([](auto a, auto l, auto h) { return fmin_(fmax_(a, l), h); }, x, lo, hi); }
template<class X, class Y, class A> inline auto mix(X x, Y y, A a)
{
  if constexpr(std::is_same_v<typename vinfo<A>::E, bool>)
    return vmapn([](float p, float q, bool s) { return s ? q : p; }, x, y, a);
  else return vmapn([](float p, float q, float t) { return p * (1.0f - t) + q * t; }, x, y, a);
}
template<class E, class X> inline auto step(E e, X x) { return vmapn([](float a, float b) { return b < a ? 0.0f : 1.0f; }, e, x); }
template<class E0, class E1, class X> inline auto smoothstep(E0 e0, E1 e1, X x)
{
  return vmapn([](float a, float b, float v) { float t = fmin_(fmax_((v - a) / (b - a), 0.0f), 1.0f); return t * t * (3.0f - 2.0f * t); }, e0, e1, x);
}
template<class A, class B> inline float dot(const A &a, const B &b)
{
  const auto x = tov(a), y = tov(b);
  if constexpr(vinfo<decltype(x)>::is) { float s = 0.0f; for(int k = 0; k < vinfo<decltype(x)>::n; k++) s = s + x.d[k] * y.d[k]; return s; }
  else return x * y;
}
template<class A> inline float length(const A &a) { return sqrt(dot(a, a)); }
template<class A, class B> inline float distance(const A &a, const B &b) { return length(tov(a) - tov(b)); }
template<class A> inline auto normalize(const A &a) { return tov(a) / length(a); }
inline vec3 cross(const vec3 &a, const vec3 &b) { return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
template<class A, class = std::enable_if_t<is_vec<A>>> inline auto isnan(const A &a) { return vmap([](float x) { return (bool)std::isnan(x); }, a); }
template<class A, class = std::enable_if_t<is_vec<A>>> inline auto isinf(const A &a) { return vmap([](float x) { return (bool)std::isinf(x); }, a); }
template<class A> inline bool any(const A &a) { auto v = tov(a); for(int k = 0; k < vinfo<A>::n; k++) if(v.d[k]) return true; return false; }
template<class A> inline bool all(const A &a) { auto v = tov(a); for(int k = 0; k < vinfo<A>::n; k++) if(!v.d[k]) return false; return true; }
template<class A> inline auto not_(const A &a) { return vmap([](bool b) { return !b; }, a); }
#define GLSL_CMP(name, op) template<class A, class B> inline auto name(const A &a, const B &b) { return vmapn([](auto x, auto y) { return (bool)(x op y); }, a, b); }
GLSL_CMP(lessThan, <) GLSL_CMP(lessThanEqual, <=) GLSL_CMP(greaterThan, >) GLSL_CMP(greaterThanEqual, >=) GLSL_CMP(equal, ==) GLSL_CMP(notEqual, !=)
#undef GLSL_CMP
inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline int floatBitsToInt(float f) { int u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float intBitsToFloat(int u) { float f; std::memcpy(&f, &u, 4); return f; }
float half_to_float(uint16_t h);
uint16_t float_to_half(float f);
inline vec2 unpackHalf2x16(uint u) { return vec2(half_to_float(u & 0xffff), half_to_float(u >> 16)); }
inline uint packHalf2x16(const vec2 &v) { return (uint)float_to_half(v.x) | ((uint)float_to_half(v.y) << 16); }
template<class A> inline A nonuniformEXT(const A &a) { return a; }

// float16_t (GL_EXT_shader_explicit_arithmetic_types_float16): a value held
// exactly in binary16. Arithmetic between two float16_t rounds its result to
// binary16 (computed in FP32 and rounded once more: FP32 has more than 2*11+2
// bits, so the result is the correctly rounded binary16 one); mixed with
// float it converts to float.
float f16_round(float v);
struct float16_t
{
  float v = 0.0f;
  float16_t() {}
  explicit float16_t(float x) : v(f16_round(x)) {}
  explicit float16_t(double x) : v(f16_round((float)x)) {}
  explicit float16_t(int x) : v(f16_round((float)x)) {}
  operator float() const { return v; }
};
inline float16_t operator+(float16_t a, float16_t b) { return float16_t(a.v + b.v); }
inline float16_t operator-(float16_t a, float16_t b) { return float16_t(a.v - b.v); }
inline float16_t operator*(float16_t a, float16_t b) { return float16_t(a.v * b.v); }
inline float16_t operator/(float16_t a, float16_t b) { return float16_t(a.v / b.v); }
inline float16_t operator-(float16_t a) { float16_t r; r.v = -a.v; return r; }
inline float16_t abs(float16_t a) { float16_t r; r.v = std::fabs(a.v); return r; }

// workgroup shared array. An index outside the array is undefined in the
// reference; here a read returns 0 and a write is dropped.
template<class T, int N> struct shared_arr
{
  T e[N];
  T oob;
  T &operator[](long i)
  {
    if(i < 0 || i >= N) { oob = T(0); return oob; }
    return e[i];
  }
};
// barrier phases of the running invocation (translate.py: phases())
extern thread_local int glsl_bar_, glsl_phase_;

// barrier() anywhere in a shader: every invocation of a workgroup runs on its
// own stack and gives control back to the workgroup's scheduler at each
// barrier; the scheduler resumes all invocations once every one of them has
// reached it (or returned). Runs the workgroups of a dispatch (in parallel
// across host threads, one workgroup at a time per thread).
void barrier();
void memoryBarrierShared();
void run_workgroups_coop(int GX, int GY, int GZ, int LX, int LY, void (*fn)());

// integer built-ins of the int8/int16 extensions and GLSL 4
inline uint bitfieldExtract(uint v, int off, int bits)
{
  if(bits <= 0) return 0u;
  const uint m = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
  return (v >> off) & m;
}
template<class A, class = std::enable_if_t<is_vec<A>>> inline auto bitfieldExtract(const A &a, int off, int bits)
{ return vmap([&](auto x) { return bitfieldExtract((uint)x, off, bits); }, a); }
inline uint16_t pack16(const u8vec2 &v) { return (uint16_t)((uint)v.d[0] | ((uint)v.d[1] << 8)); }
template<class A> inline uint16_t pack16(const A &a) { return pack16(u8vec2(tov(a))); }

// ------------------------------------------------------------------ images
struct image_t
{ // row major, c channels of float (values already rounded to the storage format)
  float *data = nullptr;
  int w = 0, h = 0, c = 1;
  int fmt = 0;  // 0 f16, 1 f32, 2 unorm16, 3 u32 (stored as float bits)
};
struct sampler2D { const image_t *im = nullptr; };
struct usampler2D { const image_t *im = nullptr; };
struct image2D { image_t *im = nullptr; };
struct uimage2D { image_t *im = nullptr; };
template<class S> struct res_array
{ // unbounded arrays of sampler/image bindings (img[] in the shaders)
  S e[32];
  S &operator[](int i) { return e[i]; }
  const S &operator[](int i) const { return e[i]; }
};

int mirror(int i, int n);
vec4 texel(const image_t *im, int x, int y);         // in range read, (r,0,0,1) rule
vec4 texelFetch(const sampler2D &s, const ivec2 &p, int lod);
uvec4 texelFetch(const usampler2D &s, const ivec2 &p, int lod);
vec4 texture(const sampler2D &s, const vec2 &uv);
vec4 textureLod(const sampler2D &s, const vec2 &uv, float lod);
vec4 textureGather(const sampler2D &s, const vec2 &uv, int comp);
ivec2 textureSize(const sampler2D &s, int lod);
ivec2 textureSize(const usampler2D &s, int lod);
ivec2 imageSize(const image2D &i);
ivec2 imageSize(const uimage2D &i);
// atomic adds (workgroups run on several threads: real atomics; float sums in any order)
uint imageAtomicAdd(const uimage2D &i, const ivec2 &p, uint v);
float imageAtomicAdd(const image2D &i, const ivec2 &p, float v);
template<class V> inline uint imageAtomicAdd(const uimage2D &i, const ivec2 &p, V v) { return imageAtomicAdd(i, p, (uint)v); }
void imageStore(const image2D &i, const ivec2 &p, const vec4 &v);
vec4 imageLoad(const image2D &i, const ivec2 &p);
template<class A> inline vec4 texture(const sampler2D &s, const A &uv) { return texture(s, vec2(tov(uv))); }
template<class A> inline vec4 textureLod(const sampler2D &s, const A &uv, float l) { return textureLod(s, vec2(tov(uv)), l); }
template<class A> inline vec4 textureGather(const sampler2D &s, const A &uv, int c) { return textureGather(s, vec2(tov(uv)), c); }
template<class A, class = std::enable_if_t<is_vec<A> && !std::is_same_v<A, ivec2>>> inline vec4 texelFetch(const sampler2D &s, const A &p, int l) { return texelFetch(s, ivec2(tov(p)), l); }
template<class A, class = std::enable_if_t<is_vec<A> && !std::is_same_v<A, ivec2>>> inline void imageStore(const image2D &i, const A &p, const vec4 &v) { imageStore(i, ivec2(tov(p)), v); }
template<class A, class B, class = std::enable_if_t<!std::is_same_v<B, vec4>>> inline void imageStore(const image2D &i, const A &p, const B &v) { imageStore(i, ivec2(tov(p)), vec4(tov(v))); }

// ------------------------------------------------------------------ invocation
extern thread_local uvec3 gl_GlobalInvocationID;
extern thread_local uvec3 gl_LocalInvocationID;
extern thread_local uvec3 gl_WorkGroupID;
extern thread_local uint gl_LocalInvocationIndex;

} // namespace glsl

// the dispatch record the runner passes to every translated shader
extern "C" {
typedef struct ref_dispatch_t
{
  int wd, ht, dp;                  // invocations (rounded up to the 8x8 workgroups by the runner)
  const void *uniform;             // module parameter block (std140), may be 0
  const void *push;                // push constants (std140), may be 0
  const void *global;              // global uniform block (frame, ...), may be 0
  glsl::image_t *bind[8][32];      // bindings [binding][array element]
  void *buf[8];                    // storage buffers by binding
} ref_dispatch_t;
}
