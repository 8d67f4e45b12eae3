// OpenCL C 1.2 shim for g++ (test infrastructure only).
//
// Lets the MambaTracer kernel translation unit (src/cl/kernel/*.cl, concatenated
// in the order of src/cl/kernel/CSource.java:18-38) compile as C++20 so that its
// kernels can run here, one work-item at a time, as the parity reference for the
// CPU restatement in oracle/ and, through it, for the CUDA kernels.
//
// Semantics chosen where OpenCL leaves them to the device (each one is the
// behaviour the CPU restatement and the CUDA kernels also follow):
//   * dot(a,b)   = ((a.x*b.x + a.y*b.y) + a.z*b.z) + a.w*b.w, left to right,
//                  no FMA (the build passes -ffp-contract=off).
//   * cross(a,b) = (ay*bz - az*by, az*bx - ax*bz, ax*by - ay*bx, 0).
//   * length(v)  = sqrt(dot(v,v)); normalize(v) = v / length(v) per lane.
//   * rsqrt(x)   = 1 / sqrt(x) (two correctly rounded steps).
//   * min/max    = OpenCL's "y < x ? y : x" / "x < y ? y : x".
//   * floating literals are single precision (-fsingle-precision-constant),
//     as an OpenCL device without fp64 or -cl-single-precision-constant does.
//   * lanes never written are zero (-ftrivial-auto-var-init=zero), where a GPU
//     driver would leave whatever the register held.
//   * transcendental functions are the host C library's float versions.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

typedef unsigned int uint;
typedef unsigned char uchar;

// ---------------------------------------------------------------- vectors
struct float2;
struct float3;
struct float4;

struct clswz_xy {  // .xy of a float3/float4 (aliases the first two lanes)
  float v[4];
  inline operator float2() const;
  inline clswz_xy& operator=(const float2& o);
};

struct clswz_xyz {  // .xyz of a float4 (aliases the first three lanes)
  float v[4];
  inline operator float3() const;
  inline clswz_xyz& operator=(const float3& o);
  inline clswz_xyz& operator+=(const float3& o);
  inline clswz_xyz& operator-=(const float3& o);
  inline clswz_xyz& operator*=(const float3& o);
  inline clswz_xyz& operator/=(float s);
  inline clswz_xyz& operator*=(float s);
};

struct alignas(8) float2 {
  union {
    struct { float x, y; };
    float s[2];
  };
  float2& operator=(float a) { x = y = a; return *this; }
};

struct alignas(16) float3 {
  union {
    struct { float x, y, z, pad_; };
    clswz_xy xy;
    float s[4];
  };
  float3& operator=(float a) { x = y = z = a; return *this; }
};

struct alignas(16) float4 {
  union {
    struct { float x, y, z, w; };
    clswz_xyz xyz;
    clswz_xy xy;
    float s[4];
  };
  float4& operator=(float a) { x = y = z = w = a; return *this; }
};

struct alignas(8) int2 {
  union {
    struct { int x, y; };
    int s[2];
  };
};

struct alignas(16) int4 {
  union {
    struct { int x, y, z, w; };
    int s[4];
  };
};

inline clswz_xy::operator float2() const { float2 r; r.x = v[0]; r.y = v[1]; return r; }
inline clswz_xy& clswz_xy::operator=(const float2& o) { v[0] = o.x; v[1] = o.y; return *this; }
inline clswz_xyz::operator float3() const { float3 r; r.x = v[0]; r.y = v[1]; r.z = v[2]; r.pad_ = 0; return r; }
inline clswz_xyz& clswz_xyz::operator=(const float3& o) { v[0] = o.x; v[1] = o.y; v[2] = o.z; return *this; }
inline clswz_xyz& clswz_xyz::operator+=(const float3& o) { v[0] += o.x; v[1] += o.y; v[2] += o.z; return *this; }
inline clswz_xyz& clswz_xyz::operator-=(const float3& o) { v[0] -= o.x; v[1] -= o.y; v[2] -= o.z; return *this; }
inline clswz_xyz& clswz_xyz::operator*=(const float3& o) { v[0] *= o.x; v[1] *= o.y; v[2] *= o.z; return *this; }
inline clswz_xyz& clswz_xyz::operator/=(float s) { v[0] /= s; v[1] /= s; v[2] /= s; return *this; }
inline clswz_xyz& clswz_xyz::operator*=(float s) { v[0] *= s; v[1] *= s; v[2] *= s; return *this; }

// ------------------------------------------------ vector literal factories
// "(float4)(a, b, c, d)" is rewritten to "clv_float4(a, b, c, d)"; scalars and
// vectors are flattened lane by lane, a single scalar is broadcast.
namespace clv {
template <typename T> struct lanes { static constexpr int n = 1; };
template <> struct lanes<float2> { static constexpr int n = 2; };
template <> struct lanes<float3> { static constexpr int n = 3; };
template <> struct lanes<float4> { static constexpr int n = 4; };
template <> struct lanes<int2> { static constexpr int n = 2; };
template <> struct lanes<int4> { static constexpr int n = 4; };
template <> struct lanes<clswz_xyz> { static constexpr int n = 3; };
template <> struct lanes<clswz_xy> { static constexpr int n = 2; };

template <typename E> struct sink { E* out; int k; };
template <typename E, typename T>
inline void put(sink<E>& s, const T& v) {
  if constexpr (lanes<T>::n == 1) {
    s.out[s.k++] = static_cast<E>(v);
  } else if constexpr (std::is_same_v<T, clswz_xyz> || std::is_same_v<T, clswz_xy>) {
    for (int i = 0; i < lanes<T>::n; ++i) s.out[s.k++] = static_cast<E>(v.v[i]);
  } else {
    for (int i = 0; i < lanes<T>::n; ++i) s.out[s.k++] = static_cast<E>(v.s[i]);
  }
}
template <typename V, typename E, int N, typename... A>
inline V make(const A&... a) {
  V r;
  std::memset(&r, 0, sizeof(r));
  E tmp[4] = {0, 0, 0, 0};
  sink<E> s{tmp, 0};
  (put<E>(s, a), ...);
  if (s.k == 1) for (int i = 1; i < N; ++i) tmp[i] = tmp[0];
  for (int i = 0; i < N; ++i) r.s[i] = tmp[i];
  return r;
}
}  // namespace clv

template <typename... A> inline float2 clv_float2(const A&... a) { return clv::make<float2, float, 2>(a...); }
template <typename... A> inline float3 clv_float3(const A&... a) { return clv::make<float3, float, 3>(a...); }
template <typename... A> inline float4 clv_float4(const A&... a) { return clv::make<float4, float, 4>(a...); }
template <typename... A> inline int2 clv_int2(const A&... a) { return clv::make<int2, int, 2>(a...); }
template <typename... A> inline int4 clv_int4(const A&... a) { return clv::make<int4, int, 4>(a...); }

// ------------------------------------------------------ vector arithmetic
#define CLSHIM_VEC_OPS(V, N)                                                                       \
  inline V operator+(V a, V b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] + b.s[i]; return a; } \
  inline V operator-(V a, V b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] - b.s[i]; return a; } \
  inline V operator*(V a, V b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] * b.s[i]; return a; } \
  inline V operator/(V a, V b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] / b.s[i]; return a; } \
  inline V operator+(V a, float b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] + b; return a; }  \
  inline V operator-(V a, float b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] - b; return a; }  \
  inline V operator*(V a, float b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] * b; return a; }  \
  inline V operator/(V a, float b) { for (int i = 0; i < N; ++i) a.s[i] = a.s[i] / b; return a; }  \
  inline V operator+(float b, V a) { for (int i = 0; i < N; ++i) a.s[i] = b + a.s[i]; return a; }  \
  inline V operator-(float b, V a) { for (int i = 0; i < N; ++i) a.s[i] = b - a.s[i]; return a; }  \
  inline V operator*(float b, V a) { for (int i = 0; i < N; ++i) a.s[i] = b * a.s[i]; return a; }  \
  inline V operator/(float b, V a) { for (int i = 0; i < N; ++i) a.s[i] = b / a.s[i]; return a; }  \
  inline V operator-(V a) { for (int i = 0; i < N; ++i) a.s[i] = -a.s[i]; return a; }              \
  inline V& operator+=(V& a, V b) { a = a + b; return a; }                                         \
  inline V& operator-=(V& a, V b) { a = a - b; return a; }                                         \
  inline V& operator*=(V& a, V b) { a = a * b; return a; }                                         \
  inline V& operator/=(V& a, V b) { a = a / b; return a; }                                         \
  inline V& operator*=(V& a, float b) { a = a * b; return a; }                                     \
  inline V& operator/=(V& a, float b) { a = a / b; return a; }

CLSHIM_VEC_OPS(float2, 2)
CLSHIM_VEC_OPS(float3, 3)
CLSHIM_VEC_OPS(float4, 4)
#undef CLSHIM_VEC_OPS

inline int2 operator+(int2 a, int2 b) { a.x += b.x; a.y += b.y; return a; }
inline int2 operator-(int2 a, int2 b) { a.x -= b.x; a.y -= b.y; return a; }

// ------------------------------------------------------------- built-ins
inline float sqrt(float x) { return sqrtf(x); }
inline float rsqrt(float x) { return 1.0f / sqrtf(x); }
inline float sin(float x) { return sinf(x); }
inline float cos(float x) { return cosf(x); }
inline float tan(float x) { return tanf(x); }
inline float acos(float x) { return acosf(x); }
inline float atan2(float y, float x) { return atan2f(y, x); }
inline float exp(float x) { return expf(x); }
inline float log(float x) { return logf(x); }
inline float pow(float x, float y) { return powf(x, y); }
inline float fabs(float x) { return fabsf(x); }
inline float fmax(float a, float b) { return fmaxf(a, b); }
inline float fmin(float a, float b) { return fminf(a, b); }
inline float radians(float d) { return d * 0.017453292519943295f; }
inline int isinf(float x) { return std::isinf(x) ? 1 : 0; }
inline int isnan(float x) { return std::isnan(x) ? 1 : 0; }

inline float3 pow(float3 a, float3 b) { for (int i = 0; i < 3; ++i) a.s[i] = powf(a.s[i], b.s[i]); return a; }

inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline float4 min(float4 a, float4 b) { for (int i = 0; i < 4; ++i) a.s[i] = min(a.s[i], b.s[i]); return a; }
inline float4 max(float4 a, float4 b) { for (int i = 0; i < 4; ++i) a.s[i] = max(a.s[i], b.s[i]); return a; }
inline float clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

template <typename T> inline T select(T a, T b, int c) { return c ? b : a; }
inline float4 select(float4 a, float4 b, int4 c) {
  for (int i = 0; i < 4; ++i) a.s[i] = (c.s[i] < 0) ? b.s[i] : a.s[i];
  return a;
}

inline float dot(float4 a, float4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float dot(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float4 cross(float4 a, float4 b) {
  return clv_float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
inline float3 cross(float3 a, float3 b) {
  return clv_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(float4 v) { return sqrtf(dot(v, v)); }
inline float length(float3 v) { return sqrtf(dot(v, v)); }
inline float4 normalize(float4 v) { float l = length(v); return v / l; }
inline float3 normalize(float3 v) { float l = length(v); return v / l; }

// --------------------------------------------------------- work-items
namespace clshim {
struct WorkItem {
  int global_id = 0, local_id = 0, group_id = 0, local_size = 1, global_size = 1;
  void (*barrier_fn)(void*) = nullptr;
  void* barrier_ctx = nullptr;
};
inline thread_local WorkItem wi;
}  // namespace clshim

inline int get_global_id(int) { return clshim::wi.global_id; }
inline int get_local_id(int) { return clshim::wi.local_id; }
inline int get_group_id(int) { return clshim::wi.group_id; }
inline int get_local_size(int) { return clshim::wi.local_size; }
inline int get_global_size(int) { return clshim::wi.global_size; }

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
inline void barrier(int) {
  if (clshim::wi.barrier_fn) clshim::wi.barrier_fn(clshim::wi.barrier_ctx);
}

inline int atomic_inc(volatile int* p) { return __atomic_fetch_add(const_cast<int*>(p), 1, __ATOMIC_SEQ_CST); }
inline unsigned int atomic_cmpxchg(volatile unsigned int* p, unsigned int cmp, unsigned int val) {
  unsigned int expected = cmp;
  __atomic_compare_exchange_n(const_cast<unsigned int*>(p), &expected, val, false, __ATOMIC_SEQ_CST,
                              __ATOMIC_SEQ_CST);
  return expected;
}

// ------------------------------------------------ address-space qualifiers
#define __kernel
#define __global
#define global
#define __local
#define local
#define __private
#define private
#define __constant const
#define constant const
#define initIsect InitIsect  // src/cl/kernel/Initialize.cl:59 calls an undefined name

// A fresh local SATRegion (see make_ref.py): nu = nv = INT_MAX, the rest 0.
#define clshim_unset_region() {2147483647, 2147483647, 0, 0, 0, 0}
