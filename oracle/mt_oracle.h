// CPU restatement of MambaTracer's wavefront GI path (test infrastructure).
//
// This is the oracle: tests and __graft_entry__.smoke() check results against
// it, and bench.py's CPU baseline times it. The product (mambatracer_gb300) never
// includes, links or calls anything here.
//
// Templated on the scalar type: R = float restates the reference kernels in
// FP32 with the evaluation order of oracle/ref/clshim.h (the order the parity
// tests pin against the reference's own kernels compiled as C++); R = double
// is the FP64 image oracle (same formulas; the RNG stays the reference's
// integer/FP32 stream). Citations are file:line in mambastudio/MambaTracer.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace mto {

template <class R>
struct V4 {
  R x, y, z, w;
};
template <class R> inline V4<R> v4(R x, R y, R z, R w) { return V4<R>{x, y, z, w}; }
template <class R> inline V4<R> operator+(V4<R> a, V4<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class R> inline V4<R> operator-(V4<R> a, V4<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class R> inline V4<R> operator*(V4<R> a, V4<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
template <class R> inline V4<R> operator*(V4<R> a, R s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class R> inline V4<R> operator*(R s, V4<R> a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
template <class R> inline V4<R> operator/(V4<R> a, R s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
template <class R> inline V4<R> operator-(V4<R> a) { return {-a.x, -a.y, -a.z, -a.w}; }

// dot/cross/length/normalize: the lane order fixed in oracle/ref/clshim.h.
template <class R> inline R dot4(V4<R> a, V4<R> b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
template <class R> inline R dot3(V4<R> a, V4<R> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class R> inline V4<R> cross4(V4<R> a, V4<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, R(0)};
}
template <class R> inline R sqrt_(R x) { return std::sqrt(x); }
template <class R> inline V4<R> normalize4(V4<R> v) { R l = sqrt_(dot4(v, v)); return v / l; }
// float3 normalize: w lane excluded, result w = 0
template <class R> inline V4<R> normalize3(V4<R> v) {
  R l = sqrt_(dot3(v, v));
  return {v.x / l, v.y / l, v.z / l, R(0)};
}
template <class R> inline V4<R> xyz0(V4<R> v) { return {v.x, v.y, v.z, R(0)}; }

template <class R> inline R min_(R a, R b) { return b < a ? b : a; }
template <class R> inline R max_(R a, R b) { return a < b ? b : a; }
template <class R> inline R fmax_(R a, R b) { return std::fmax(a, b); }
template <class R> inline R fmin_(R a, R b) { return std::fmin(a, b); }
template <class R> inline R clamp_(R x, R lo, R hi) { return fmin_(fmax_(x, lo), hi); }

// Reference layouts (byte-identical to the OpenCL structs).
struct Face { int vx, vy, vz, uvx, uvy, uvz, nx, ny, nz, mat; };        // Util.cl:95-102
struct BVHNode { int bound, sibling, left, right, parent, isLeaf, child; };  // NormalBVH.cl:1-11
struct BoundingBox { float mn[4], mx[4]; };                             // Util.cl:116-121
struct SurfaceParameter {                                               // Bsdf.cl:24-42
  int isDiffuseTexture, isGlossyTexture, isRoughnessTexture, isMirrorTexture;
  float diffuse_color[4], diffuse_param[4], glossy_color[4], glossy_param[4];
  float mirror_color[4], mirror_param[4], emission_color[4], emission_param[4];
};
struct alignas(16) RayF {                                               // Util.cl:129-138
  float o[4], d[4], inv_d[4];
  int sign[4];
  int extra[2];
  float tMin, tMax;
};
struct alignas(16) CameraF {                                            // Util.cl:78-85
  float position[4], lookat[4], up[4], dimension[2], fov, pad_;
};
static_assert(sizeof(RayF) == 80, "Ray layout");
static_assert(sizeof(CameraF) == 64, "CameraStruct layout");
static_assert(sizeof(SurfaceParameter) == 144, "Material layout");

struct Mesh {
  const float* points;   // float4 per vertex
  const float* uvs;      // float2 per uv
  const float* normals;  // float4 per normal
  const Face* faces;
  int nfaces;
};

}  // namespace mto
