// WGSL runtime for C++ — TEST INFRASTRUCTURE ONLY.
//
// The types, operators and builtins that WGSL compute code translated by
// oracle/wgsl_ref.py needs to compile and run as C++ on the host:
//   - f32 / u32 / i32 scalars, vec2/3/4 of each, mat3x3f (column-major, each
//     column a 16-byte vec3 so arrays of mat3x3f have WGSL's 48-byte storage
//     stride), fixed-size arrays;
//   - abstract floats (AF): WGSL evaluates literal-only expressions in at
//     least f64 and converts the result to f32 where it meets an f32 operand
//     (WGSL spec, "abstract numeric types"); AF keeps a double and follows
//     the same rule, so `sqrt(2.0 / 3.0) * x` rounds the constant once;
//     abstract integers are C++ int literals;
//   - builtins with the WGSL names (WGSL spec, "built-in functions");
//   - atomics for invocations run one at a time, and workgroup barriers for
//     the invocations of one workgroup run as coroutines, so barrier kernels
//     keep their phase semantics.
#pragma once

#include <algorithm>
#include <coroutine>
#include <exception>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

namespace wgsl {

using f32 = float;
using u32 = uint32_t;
using i32 = int32_t;

// ---------------------------------------------------------------- abstract float
struct AF {
  double v;
  constexpr explicit AF(double x) : v(x) {}
  operator float() const { return (float)v; }
};
inline AF operator-(AF a) { return AF(-a.v); }
inline AF operator+(AF a, AF b) { return AF(a.v + b.v); }
inline AF operator-(AF a, AF b) { return AF(a.v - b.v); }
inline AF operator*(AF a, AF b) { return AF(a.v * b.v); }
inline AF operator/(AF a, AF b) { return AF(a.v / b.v); }
inline AF operator+(AF a, int b) { return AF(a.v + b); }
inline AF operator-(AF a, int b) { return AF(a.v - b); }
inline AF operator*(AF a, int b) { return AF(a.v * b); }
inline AF operator/(AF a, int b) { return AF(a.v / b); }
inline AF operator+(int a, AF b) { return AF(a + b.v); }
inline AF operator-(int a, AF b) { return AF(a - b.v); }
inline AF operator*(int a, AF b) { return AF(a * b.v); }
inline AF operator/(int a, AF b) { return AF(a / b.v); }
// AF meeting f32 converts to f32 first
#define WGSL_AF_MIX(OP)                                                   \
  inline float operator OP(AF a, float b) { return (float)a OP b; }       \
  inline float operator OP(float a, AF b) { return a OP (float)b; }
WGSL_AF_MIX(+)
WGSL_AF_MIX(-)
WGSL_AF_MIX(*)
WGSL_AF_MIX(/)
#undef WGSL_AF_MIX
#define WGSL_AF_CMP(OP)                                                   \
  inline bool operator OP(AF a, AF b) { return a.v OP b.v; }              \
  inline bool operator OP(AF a, float b) { return (float)a OP b; }        \
  inline bool operator OP(float a, AF b) { return a OP (float)b; }
WGSL_AF_CMP(<)
WGSL_AF_CMP(>)
WGSL_AF_CMP(<=)
WGSL_AF_CMP(>=)
WGSL_AF_CMP(==)
WGSL_AF_CMP(!=)
#undef WGSL_AF_CMP

// ---------------------------------------------------------------- vectors
template <class T>
struct V2 {
  T x{}, y{};
  V2() = default;
  explicit V2(T s) : x(s), y(s) {}
  V2(T a, T b) : x(a), y(b) {}
  template <class U>
  explicit V2(const V2<U>& o) : x((T)o.x), y((T)o.y) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  T operator[](int i) const { return i == 0 ? x : y; }
  T& operator[](unsigned i) { return (*this)[(int)i]; }
  T operator[](unsigned i) const { return (*this)[(int)i]; }
};
template <class T>
struct alignas(16) V3 {
  T x{}, y{}, z{};
  V3() = default;
  explicit V3(T s) : x(s), y(s), z(s) {}
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
  template <class U>
  explicit V3(const V3<U>& o) : x((T)o.x), y((T)o.y), z((T)o.z) {}
  V3 xyz() const { return *this; }
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  T& operator[](unsigned i) { return (*this)[(int)i]; }
  T operator[](unsigned i) const { return (*this)[(int)i]; }
};
template <class T>
struct alignas(16) V4 {
  T x{}, y{}, z{}, w{};
  V4() = default;
  explicit V4(T s) : x(s), y(s), z(s), w(s) {}
  V4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  V4(const V3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  V3<T> xyz() const { return V3<T>(x, y, z); }
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T& operator[](unsigned i) { return (*this)[(int)i]; }
  T operator[](unsigned i) const { return (*this)[(int)i]; }
};
using vec2f = V2<float>;
using vec3f = V3<float>;
using vec4f = V4<float>;
using vec2u = V2<u32>;
using vec3u = V3<u32>;
using vec4u = V4<u32>;
using vec2i = V2<i32>;
using vec3i = V3<i32>;
using vec4i = V4<i32>;

template <class T> struct is_vec : std::false_type {};
template <class T> struct is_vec<V2<T>> : std::true_type {};
template <class T> struct is_vec<V3<T>> : std::true_type {};
template <class T> struct is_vec<V4<T>> : std::true_type {};
template <class T> struct elem { using type = T; };
template <class T> struct elem<V2<T>> { using type = T; };
template <class T> struct elem<V3<T>> { using type = T; };
template <class T> struct elem<V4<T>> { using type = T; };

// componentwise map / zip
template <class T, class F> V2<T> vmap(const V2<T>& a, F f) { return V2<T>(f(a.x), f(a.y)); }
template <class T, class F> V3<T> vmap(const V3<T>& a, F f) { return V3<T>(f(a.x), f(a.y), f(a.z)); }
template <class T, class F> V4<T> vmap(const V4<T>& a, F f) { return V4<T>(f(a.x), f(a.y), f(a.z), f(a.w)); }
template <class T, class F> V2<T> vzip(const V2<T>& a, const V2<T>& b, F f) { return V2<T>(f(a.x, b.x), f(a.y, b.y)); }
template <class T, class F> V3<T> vzip(const V3<T>& a, const V3<T>& b, F f) {
  return V3<T>(f(a.x, b.x), f(a.y, b.y), f(a.z, b.z));
}
template <class T, class F> V4<T> vzip(const V4<T>& a, const V4<T>& b, F f) {
  return V4<T>(f(a.x, b.x), f(a.y, b.y), f(a.z, b.z), f(a.w, b.w));
}

#define WGSL_VEC_BINOP(OP)                                                                               \
  template <class Vt, std::enable_if_t<is_vec<Vt>::value, int> = 0>                                      \
  Vt operator OP(const Vt& a, const Vt& b) {                                                             \
    using T = typename elem<Vt>::type;                                                                   \
    return vzip(a, b, [](T p, T q) { return (T)(p OP q); });                                             \
  }                                                                                                      \
  template <class Vt, class S,                                                                           \
            std::enable_if_t<is_vec<Vt>::value && !is_vec<S>::value, int> = 0>                           \
  Vt operator OP(const Vt& a, S s) {                                                                     \
    using T = typename elem<Vt>::type;                                                                   \
    const T t = (T)s;                                                                                    \
    return vmap(a, [t](T p) { return (T)(p OP t); });                                                    \
  }                                                                                                      \
  template <class Vt, class S,                                                                           \
            std::enable_if_t<is_vec<Vt>::value && !is_vec<S>::value, int> = 0>                           \
  Vt operator OP(S s, const Vt& a) {                                                                     \
    using T = typename elem<Vt>::type;                                                                   \
    const T t = (T)s;                                                                                    \
    return vmap(a, [t](T p) { return (T)(t OP p); });                                                    \
  }                                                                                                      \
  template <class Vt, class S, std::enable_if_t<is_vec<Vt>::value, int> = 0>                             \
  Vt& operator OP##=(Vt & a, const S & b) {                                                              \
    a = a OP b;                                                                                          \
    return a;                                                                                            \
  }
WGSL_VEC_BINOP(+)
WGSL_VEC_BINOP(-)
WGSL_VEC_BINOP(*)
WGSL_VEC_BINOP(/)
#undef WGSL_VEC_BINOP
template <class Vt, std::enable_if_t<is_vec<Vt>::value, int> = 0>
Vt operator-(const Vt& a) {
  using T = typename elem<Vt>::type;
  return vmap(a, [](T p) { return (T)(-p); });
}

// ---------------------------------------------------------------- mat3x3f
struct mat3x3f {
  vec3f c[3];
  mat3x3f() = default;
  mat3x3f(const vec3f& a, const vec3f& b, const vec3f& d) : c{a, b, d} {}
  mat3x3f(float a0, float a1, float a2, float b0, float b1, float b2, float d0, float d1, float d2)
      : c{vec3f(a0, a1, a2), vec3f(b0, b1, b2), vec3f(d0, d1, d2)} {}
  vec3f& operator[](int i) { return c[i]; }
  const vec3f& operator[](int i) const { return c[i]; }
  vec3f& operator[](unsigned i) { return c[i]; }
  const vec3f& operator[](unsigned i) const { return c[i]; }
};
static_assert(sizeof(mat3x3f) == 48, "mat3x3f keeps the 48-byte storage stride");
inline mat3x3f operator+(const mat3x3f& a, const mat3x3f& b) {
  return mat3x3f(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]);
}
inline mat3x3f operator-(const mat3x3f& a, const mat3x3f& b) {
  return mat3x3f(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]);
}
inline mat3x3f operator*(const mat3x3f& a, float s) { return mat3x3f(a.c[0] * s, a.c[1] * s, a.c[2] * s); }
inline mat3x3f operator*(float s, const mat3x3f& a) { return mat3x3f(s * a.c[0], s * a.c[1], s * a.c[2]); }
inline mat3x3f operator*(const mat3x3f& a, AF s) { return a * (float)s; }
inline mat3x3f operator*(AF s, const mat3x3f& a) { return (float)s * a; }
// M v = sum_k M[k] v[k], accumulated in column order like the WGSL definition
inline vec3f operator*(const mat3x3f& m, const vec3f& v) {
  vec3f r;
  for (int row = 0; row < 3; ++row) r[row] = m.c[0][row] * v.x + m.c[1][row] * v.y + m.c[2][row] * v.z;
  return r;
}
inline mat3x3f operator*(const mat3x3f& a, const mat3x3f& b) { return mat3x3f(a * b.c[0], a * b.c[1], a * b.c[2]); }
inline mat3x3f transpose(const mat3x3f& m) {
  mat3x3f t;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.c[i][j] = m.c[j][i];
  return t;
}
// WGSL leaves the evaluation order of determinant() to the implementation;
// this runtime takes the scalar triple product c0 . (c1 x c2), with cross()
// and dot() as defined below.
inline vec3f cross(const vec3f& a, const vec3f& b);
inline float dot(const vec3f& a, const vec3f& b);
inline float determinant(const mat3x3f& m) { return dot(m.c[0], cross(m.c[1], m.c[2])); }

// ---------------------------------------------------------------- arrays
template <class T, int N>
struct WArr {
  T a[N]{};
  T& operator[](int i) { return a[i]; }
  const T& operator[](int i) const { return a[i]; }
  T& operator[](unsigned i) { return a[i]; }
  const T& operator[](unsigned i) const { return a[i]; }
};

// ---------------------------------------------------------------- declarations
template <class T> inline T concretize(const T& x) { return x; }
inline float concretize(AF a) { return (float)a.v; }

// ---------------------------------------------------------------- builtins
// Two-argument builtins take one type: AF meets f32 as f32, and abstract
// integers (C++ int) take the other operand's type.
template <class A, class B> struct unify { using type = A; };
template <> struct unify<AF, float> { using type = float; };
template <> struct unify<float, AF> { using type = float; };
template <> struct unify<int, float> { using type = float; };
template <> struct unify<float, int> { using type = float; };
template <> struct unify<int, AF> { using type = AF; };
template <> struct unify<AF, int> { using type = AF; };
template <> struct unify<int, unsigned> { using type = unsigned; };
template <> struct unify<unsigned, int> { using type = unsigned; };
template <class A, class B> using unify_t = typename unify<std::decay_t<A>, std::decay_t<B>>::type;

inline float fmin_(float a, float b) { return std::fmin(a, b); }
inline float fmax_(float a, float b) { return std::fmax(a, b); }

template <class T> inline T min_impl(T a, T b) {
  if constexpr (is_vec<T>::value) {
    return vzip(a, b, [](auto p, auto q) { return min_impl(p, q); });
  } else if constexpr (std::is_same_v<T, float>) {
    return fmin_(a, b);
  } else if constexpr (std::is_same_v<T, AF>) {
    return AF(std::fmin(a.v, b.v));
  } else {
    return a < b ? a : b;
  }
}
template <class T> inline T max_impl(T a, T b) {
  if constexpr (is_vec<T>::value) {
    return vzip(a, b, [](auto p, auto q) { return max_impl(p, q); });
  } else if constexpr (std::is_same_v<T, float>) {
    return fmax_(a, b);
  } else if constexpr (std::is_same_v<T, AF>) {
    return AF(std::fmax(a.v, b.v));
  } else {
    return a > b ? a : b;
  }
}
template <class A, class B> inline auto min(A a, B b) {
  using T = unify_t<A, B>;
  return min_impl<T>(T(a), T(b));
}
template <class A, class B> inline auto max(A a, B b) {
  using T = unify_t<A, B>;
  return max_impl<T>(T(a), T(b));
}
// clamp(e, lo, hi) = min(max(e, lo), hi)
template <class A, class B, class C> inline auto clamp(A e, B lo, C hi) {
  using T = unify_t<unify_t<A, B>, C>;
  return min_impl<T>(max_impl<T>(T(e), T(lo)), T(hi));
}
template <class T, class C> inline T select(T f, T t, C cond) { return cond ? t : f; }
template <class A, class B, class C, std::enable_if_t<!std::is_same_v<std::decay_t<A>, std::decay_t<B>>, int> = 0>
inline auto select(A f, B t, C cond) {
  using T = unify_t<A, B>;
  return cond ? T(t) : T(f);
}

#define WGSL_UNARY(NAME, EXPR)                                                   \
  inline float NAME(float x) { return EXPR; }                                    \
  inline AF NAME(AF a) {                                                         \
    const double x = a.v;                                                        \
    return AF(EXPR);                                                             \
  }                                                                              \
  template <class Vt, std::enable_if_t<is_vec<Vt>::value, int> = 0>              \
  inline Vt NAME(const Vt& v) {                                                  \
    return vmap(v, [](auto p) { return NAME(p); });                              \
  }
WGSL_UNARY(sqrt, std::sqrt(x))
WGSL_UNARY(exp, std::exp(x))
WGSL_UNARY(log, std::log(x))
WGSL_UNARY(sinh, std::sinh(x))
WGSL_UNARY(cosh, std::cosh(x))
WGSL_UNARY(floor, std::floor(x))
WGSL_UNARY(ceil, std::ceil(x))
#undef WGSL_UNARY
inline float abs(float x) { return std::fabs(x); }
inline AF abs(AF a) { return AF(std::fabs(a.v)); }
inline int abs(int x) { return x < 0 ? -x : x; }
template <class Vt, std::enable_if_t<is_vec<Vt>::value, int> = 0>
inline Vt abs(const Vt& v) {
  return vmap(v, [](auto p) { return abs(p); });
}
inline float pow_impl(float a, float b) { return std::pow(a, b); }
inline AF pow_impl(AF a, AF b) { return AF(std::pow(a.v, b.v)); }
template <class A, class B> inline auto pow(A a, B b) {
  using T = unify_t<A, B>;
  if constexpr (is_vec<T>::value) {
    return vzip(T(a), T(b), [](auto p, auto q) { return pow_impl(p, q); });
  } else {
    return pow_impl(T(a), T(b));
  }
}
inline float dot(const vec2f& a, const vec2f& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3f& a, const vec3f& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4f& a, const vec4f& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3f cross(const vec3f& a, const vec3f& b) {
  return vec3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(float x) { return std::fabs(x); }
inline float length(const vec2f& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec3f& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec4f& v) { return std::sqrt(dot(v, v)); }
inline vec3f normalize(const vec3f& v) { return v / length(v); }

// ---------------------------------------------------------------- atomics
// Kernels that use them run their invocations one at a time, in index order.
inline u32 atomicAdd(u32* p, u32 v) {
  const u32 o = *p;
  *p = o + v;
  return o;
}
inline u32 atomicSub(u32* p, u32 v) {
  const u32 o = *p;
  *p = o - v;
  return o;
}
inline u32 atomicLoad(u32* p) { return *p; }
inline void atomicStore(u32* p, u32 v) { *p = v; }

// ---------------------------------------------------------------- workgroups
// Entry points with workgroupBarrier() are emitted as coroutines: a barrier
// is `co_await Barrier{}`. runWorkgroup resumes every invocation of the
// workgroup once per round, so no invocation passes a barrier before all
// have reached it (or returned).
using EntryFn = void (*)(vec3u, vec3u, vec3u);

struct WgTask {
  struct promise_type {
    WgTask get_return_object() { return WgTask{std::coroutine_handle<promise_type>::from_promise(*this)}; }
    std::suspend_always initial_suspend() noexcept { return {}; }
    std::suspend_always final_suspend() noexcept { return {}; }
    void return_void() {}
    void unhandled_exception() { std::terminate(); }
  };
  std::coroutine_handle<promise_type> h;
};
struct Barrier {
  bool await_ready() const noexcept { return false; }
  void await_suspend(std::coroutine_handle<>) const noexcept {}
  void await_resume() const noexcept {}
};
using BarrierFn = WgTask (*)(vec3u, vec3u, vec3u);

// Runs workgroup `wid` of a barrier kernel to completion.
inline void runWorkgroup(BarrierFn fn, u32 wg, u32 wid) {
  std::vector<std::coroutine_handle<WgTask::promise_type>> inv(wg);
  for (u32 k = 0; k < wg; ++k) inv[k] = fn(vec3u(wid * wg + k, 0u, 0u), vec3u(k, 0u, 0u), vec3u(wid, 0u, 0u)).h;
  bool any = true;
  while (any) {
    any = false;
    for (auto& h : inv) {
      if (h.done()) continue;
      h.resume();
      any = true;
    }
  }
  for (auto& h : inv) h.destroy();
}

// ---------------------------------------------------------------- uniform loads
inline void loadField(float& f, const uint32_t* w, uint32_t off) { std::memcpy(&f, w + off / 4, 4); }
inline void loadField(u32& f, const uint32_t* w, uint32_t off) { f = w[off / 4]; }
inline void loadField(i32& f, const uint32_t* w, uint32_t off) { std::memcpy(&f, w + off / 4, 4); }
template <class T> inline void loadField(V2<T>& f, const uint32_t* w, uint32_t off) {
  std::memcpy(&f.x, w + off / 4, 4);
  std::memcpy(&f.y, w + off / 4 + 1, 4);
}
template <class T> inline void loadField(V3<T>& f, const uint32_t* w, uint32_t off) {
  for (int k = 0; k < 3; ++k) std::memcpy(&f[k], w + off / 4 + k, 4);
}
template <class T> inline void loadField(V4<T>& f, const uint32_t* w, uint32_t off) {
  for (int k = 0; k < 4; ++k) std::memcpy(&f[k], w + off / 4 + k, 4);
}
inline void loadField(mat3x3f& f, const uint32_t* w, uint32_t off) {
  for (int c = 0; c < 3; ++c) loadField(f.c[c], w, off + 16u * c);
}

}  // namespace wgsl
