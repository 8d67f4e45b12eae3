// CPU restatement of MambaTracer's wavefront GI path: the oracle (test
// infrastructure only; see mt_oracle.h). Every function cites the reference
// file:line it restates (paths relative to the MambaTracer project).
//
// Conventions shared with oracle/ref/clshim.h (pinned by tests against the
// reference kernels compiled as C++):
//   * vector lanes the reference never writes read as 0;
//   * floating literals are single precision in the FP32 instantiation;
//   * out-of-range environment indices (a direction exactly at u = 1 or
//     v = 1) are clamped to the last texel, where the reference reads past
//     the end of its buffer.
#include "mt_oracle.h"

#include <algorithm>
#include <type_traits>
#include <vector>

namespace mto {

// single-precision literal for R = float, the same decimal for R = double
#define KF(x) (std::is_same_v<R, float> ? R(x##f) : R(x))

template <class R> inline R sin_(R x) { if constexpr (std::is_same_v<R, float>) return sinf(x); else return std::sin(x); }
template <class R> inline R cos_(R x) { if constexpr (std::is_same_v<R, float>) return cosf(x); else return std::cos(x); }
template <class R> inline R tan_(R x) { if constexpr (std::is_same_v<R, float>) return tanf(x); else return std::tan(x); }
template <class R> inline R acos_(R x) { if constexpr (std::is_same_v<R, float>) return acosf(x); else return std::acos(x); }
template <class R> inline R atan2_(R y, R x) { if constexpr (std::is_same_v<R, float>) return atan2f(y, x); else return std::atan2(y, x); }
template <class R> inline R pow_(R x, R y) { if constexpr (std::is_same_v<R, float>) return powf(x, y); else return std::pow(x, y); }
template <class R> inline R fabs_(R x) { return std::fabs(x); }
template <class R> inline bool isinf_(R x) { return std::isinf(x); }
template <class R> inline bool isnan_(R x) { return std::isnan(x); }

template <class R> inline R PI_() { return KF(3.14159265359); }  // Util.cl:7
template <class R> inline R EPS_COSINE_() { return KF(1e-6); }   // Util.cl:5

template <class R> inline V4<R> ld4(const float* p) { return {R(p[0]), R(p[1]), R(p[2]), R(p[3])}; }

// ------------------------------------------------------------------ RNG
// Sampling.cl:15-23 (signed shifts are arithmetic, products wrap)
inline uint32_t wanghash(int32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed = (int32_t)((uint32_t)seed * 9u);
  seed = seed ^ (seed >> 4);
  seed = (int32_t)((uint32_t)seed * 0x27d4eb2du);
  seed = seed ^ (seed >> 15);
  return (uint32_t)seed;
}
struct Seed { int32_t x, y; };
// Sampling.cl:32-40
inline Seed generate_seed(int32_t sx, int32_t sy, float frameCount, int32_t gid) {
  uint32_t fc = (uint32_t)(int32_t)frameCount;
  return {(int32_t)((uint32_t)gid + fc * (uint32_t)sx), (int32_t)((uint32_t)gid + fc * (uint32_t)sy)};
}
// Sampling.cl:43-59
inline float get_random(Seed& s) {
  s.x = (int32_t)wanghash(s.x);
  s.y = (int32_t)wanghash(s.y);
  uint32_t ires = ((uint32_t)s.x << 16) + (uint32_t)s.y;
  uint32_t bits = (ires & 0x007fffffu) | 0x40000000u;
  float f;
  std::memcpy(&f, &bits, 4);
  return (f - 2.0f) / 2.0f;
}
// Sampling.cl:100-104
inline int random_int_range(Seed& s, int range) { float rf = get_random(s); return (int)(rf * (float)range); }

// ------------------------------------------------------------------- rays
template <class R>
struct Ray {
  V4<R> o, d, inv_d;
  int sign[3];
  R tMin, tMax;
};
// Util.cl:577-600
template <class R>
inline void init_ray(Ray<R>& r, V4<R> o, V4<R> d, R tMin, R tMax) {
  r.o = o;
  r.d = d;
  r.inv_d = {R(1) / d.x, R(1) / d.y, R(1) / d.z, R(0)};
  r.sign[0] = r.inv_d.x < R(0) ? 1 : 0;
  r.sign[1] = r.inv_d.y < R(0) ? 1 : 0;
  r.sign[2] = r.inv_d.z < R(0) ? 1 : 0;
  r.tMin = tMin;
  r.tMax = tMax;
}
template <class R> inline R INF_() { return std::numeric_limits<R>::infinity(); }

// Util.cl:707-732 (slab test with the 1.00000024 widening of the exit)
template <class R>
inline bool intersect_bound(const Ray<R>& r, const BoundingBox& b, R* t) {
  auto ext = [&](int s, int axis) -> R { return R(s == 0 ? b.mn[axis] : b.mx[axis]); };
  R tmin = (ext(r.sign[0], 0) - r.o.x) * r.inv_d.x;
  R tmax = (ext(1 - r.sign[0], 0) - r.o.x) * r.inv_d.x;
  R tymin = (ext(r.sign[1], 1) - r.o.y) * r.inv_d.y;
  R tymax = (ext(1 - r.sign[1], 1) - r.o.y) * r.inv_d.y;
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  R tzmin = (ext(r.sign[2], 2) - r.o.z) * r.inv_d.z;
  R tzmax = (ext(1 - r.sign[2], 2) - r.o.z) * r.inv_d.z;
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  tmax *= KF(1.00000024);
  t[0] = tmin;
  t[1] = tmax;
  return (tmin < r.tMax) && (tmax > r.tMin);
}

// Primitive.cl:3-29 (Moller-Trumbore; returns tMax on a miss)
template <class R>
inline R triangle_t(const Ray<R>& r, V4<R> p1, V4<R> p2, V4<R> p3) {
  V4<R> e1 = p2 - p1, e2 = p3 - p1;
  V4<R> h = cross4(r.d, e2);
  R a = dot4(e1, h);
  if (a > -KF(0.0000001) && a < KF(0.0000001)) return r.tMax;
  R f = R(1) / a;
  V4<R> s = r.o - p1;
  R b1 = f * dot4(s, h);
  V4<R> q = cross4(s, e1);
  R b2 = f * dot4(r.d, q);
  R t = f * dot4(e2, q);
  if (b1 < R(0) || b1 > R(1) || b2 < R(0) || b1 + b2 > R(1) || t < R(0) || t > r.tMax) return r.tMax;
  return f * dot4(e2, q);
}

template <class R> inline V4<R> P1(const Mesh& m, int id) { return ld4<R>(m.points + 4 * m.faces[id].vx); }
template <class R> inline V4<R> P2(const Mesh& m, int id) { return ld4<R>(m.points + 4 * m.faces[id].vy); }
template <class R> inline V4<R> P3(const Mesh& m, int id) { return ld4<R>(m.points + 4 * m.faces[id].vz); }

struct TraceCounts { long long interior = 0, tris = 0; };

// NormalBVH.cl:14-92 (closest hit; any hit when bailout) and :235-317
template <class R>
bool intersect_mesh(Ray<R>& ray, int* childIndex, const Mesh& mesh, const BVHNode* nodes,
                    const BoundingBox* bounds, bool bailout, TraceCounts* cnt) {
  bool hit = false;
  int nodeId = 0;
  int64_t bitstack = 0;
  int parentId = 0, siblingId = 0;
  for (;;) {
    while (!nodes[nodeId].isLeaf) {
      const BVHNode& node = nodes[nodeId];
      parentId = node.parent;
      siblingId = node.sibling;
      const BVHNode& left = nodes[node.left];
      const BVHNode& right = nodes[node.right];
      R leftT[2], rightT[2];
      bool leftHit = intersect_bound(ray, bounds[left.bound], leftT);
      bool rightHit = intersect_bound(ray, bounds[right.bound], rightT);
      if (cnt) cnt->interior++;
      if (!leftHit && !rightHit) break;
      bitstack = (int64_t)((uint64_t)bitstack << 1);
      if (leftHit && rightHit) {
        nodeId = (rightT[0] < leftT[0]) ? node.right : node.left;
        bitstack |= 1;
      } else {
        nodeId = leftHit ? node.left : node.right;
      }
    }
    if (nodes[nodeId].isLeaf) {
      const BVHNode& node = nodes[nodeId];
      R t = triangle_t(ray, P1<R>(mesh, node.child), P2<R>(mesh, node.child), P3<R>(mesh, node.child));
      if (cnt) cnt->tris++;
      if ((ray.tMin < t) && (t < ray.tMax)) {  // isInside, Util.cl:552-555
        if (bailout) return true;
        hit = true;
        ray.tMax = t;
        *childIndex = node.child;
      }
      parentId = node.parent;
      siblingId = node.sibling;
    }
    while ((bitstack & 1) == 0) {
      if (bitstack == 0) return hit;
      nodeId = parentId;
      const BVHNode& node = nodes[nodeId];
      parentId = node.parent;
      siblingId = node.sibling;
      bitstack >>= 1;
    }
    nodeId = siblingId;
    bitstack ^= 1;
  }
}

// ---------------------------------------------------------- hit record
template <class R>
struct Isect {
  V4<R> p, n, ng, d;
  R uv[2];
  int mat, id, hit;
};

// Util.cl:349-357
template <class R> inline V4<R> get_normal(V4<R> p1, V4<R> p2, V4<R> p3) {
  return normalize4(cross4(p2 - p1, p3 - p1));
}

// NormalBVH.cl:124-221 with Primitive.cl:31-71
template <class R>
void hit_record(const Ray<R>& ray, int id, const Mesh& mesh, Isect<R>& is) {
  V4<R> p1 = P1<R>(mesh, id), p2 = P2<R>(mesh, id), p3 = P3<R>(mesh, id);
  R t = ray.tMax;
  V4<R> p = {ray.o.x + t * ray.d.x, ray.o.y + t * ray.d.y, ray.o.z + t * ray.d.z, R(0)};
  const Face& f = mesh.faces[id];
  bool hasTexUV = f.uvx > -1;
  R texuv[2] = {R(0), R(0)};
  if (hasTexUV) {
    V4<R> f1 = xyz0(p1 - p), f2 = xyz0(p2 - p), f3 = xyz0(p3 - p);
    auto len3 = [](V4<R> v) { return sqrt_(dot3(v, v)); };
    R a = len3(cross4(xyz0(p1 - p2), xyz0(p1 - p3)));
    R a1 = len3(cross4(f2, f3)) / a;
    R a2 = len3(cross4(f3, f1)) / a;
    R a3 = len3(cross4(f1, f2)) / a;
    const float* u1 = mesh.uvs + 2 * f.uvx;
    const float* u2 = mesh.uvs + 2 * f.uvy;
    const float* u3 = mesh.uvs + 2 * f.uvz;
    texuv[0] = (R(u1[0]) * a1 + R(u2[0]) * a2) + R(u3[0]) * a3;
    texuv[1] = (R(u1[1]) * a1 + R(u2[1]) * a2) + R(u3[1]) * a3;
  }
  R u = R(0), v = R(0);
  {
    V4<R> e1 = xyz0(p2 - p1), e2 = xyz0(p3 - p1), e = xyz0(p - p1);
    R d00 = dot3(e1, e1), d01 = dot3(e1, e2), d11 = dot3(e2, e2), d20 = dot3(e, e1), d21 = dot3(e, e2);
    R denom = d00 * d11 - d01 * d01;
    if (!(denom == R(0))) {
      R inv = R(1) / denom;
      u = (d11 * d20 - d01 * d21) * inv;
      v = (d00 * d21 - d01 * d20) * inv;
    }
  }
  V4<R> n;
  if (f.nx > -1) {
    V4<R> n1 = ld4<R>(mesh.normals + 4 * f.nx), n2 = ld4<R>(mesh.normals + 4 * f.ny),
          n3 = ld4<R>(mesh.normals + 4 * f.nz);
    n = (n1 * ((R(1) - u) - v) + n2 * u) + n3 * v;
    if (dot4(n, ray.d) > KF(0.00001)) {
      n = -n;
      n1 = -n1;
      n2 = -n2;
      n3 = -n3;
    }
    n = normalize4(n);
    V4<R> tu = xyz0(p - p1), tv = xyz0(p - p2), tw = xyz0(p - p3);
    V4<R> m1 = normalize3(n1), m2 = normalize3(n2), m3 = normalize3(n3);
    R du = min_(R(0), dot3(tu, m1));
    R dv = min_(R(0), dot3(tv, m2));
    R dw = min_(R(0), dot3(tw, m3));
    tu = tu - xyz0(du * m1);
    tv = tv - xyz0(dv * m2);
    tw = tw - xyz0(dw * m3);
    p = ((p + ((R(1) - u) - v) * tu) + u * tv) + v * tw;
  } else {
    n = get_normal(p1, p2, p3);
    if (dot4(n, ray.d) > KF(0.00001)) n = -n;
  }
  V4<R> ng = get_normal(p1, p2, p3);
  if (dot4(ng, ray.d) > KF(0.00001)) ng = -ng;
  is.p = p;
  is.n = n;
  is.ng = ng;
  is.d = ray.d;
  is.uv[0] = hasTexUV ? texuv[0] : u;
  is.uv[1] = hasTexUV ? texuv[1] : v;
  is.id = id;
  is.mat = f.mat & 0xFFFF;
  is.hit = 1;
}

// Initialize.cl:13-23 (InitIsect; ng is left as it was)
template <class R> inline void init_isect(Isect<R>& is) {
  is.p = is.n = is.d = V4<R>{R(0), R(0), R(0), R(0)};
  is.uv[0] = is.uv[1] = R(0);
  is.id = -1;
  is.hit = 0;
  is.mat = -1;
}

// ------------------------------------------------------------- frames
template <class R> struct Frame { V4<R> mX, mY, mZ; };
// Util.cl:196-211
template <class R> inline Frame<R> get_frame(V4<R> n) {
  Frame<R> fr;
  fr.mZ = n;
  R a = R(1) / (R(1) + n.z);
  R b = -n.x * n.y * a;
  fr.mX = {R(1) - n.x * n.x * a, b, -n.x, R(0)};
  fr.mY = {b, R(1) - n.y * n.y * a, -n.y, R(0)};
  if (n.z < -KF(0.9999999)) {
    fr.mX = {R(0), R(-1), R(0), R(0)};
    fr.mY = {R(-1), R(0), R(0), R(0)};
  }
  return fr;
}
// Util.cl:213-221
template <class R> inline V4<R> world_coordinate(const Frame<R>& f, V4<R> a) { return (f.mX * a.x + f.mY * a.y) + f.mZ * a.z; }
template <class R> inline V4<R> local_coordinate(const Frame<R>& f, V4<R> a) {
  return {dot4(f.mX, a), dot4(f.mY, a), dot4(f.mZ, a), R(0)};
}

// RGBSpace.cl:28-32
template <class R> inline R luminance(R x, R y, R z) { return (KF(0.2989) * x + KF(0.5866) * y) + KF(0.1145) * z; }

// ---------------------------------------------------------------- BSDF
template <class R>
struct Bsdf {
  const SurfaceParameter* param = nullptr;
  Frame<R> frame;
  V4<R> localDirFix, localGeomN;
  int materialID = -1;
  R diffProb = R(0), glossyProb = R(0);
};
template <class R> inline V4<R> col(const float* c) { return ld4<R>(c); }

// Bsdf.cl:70-128
template <class R> inline void component_probabilities(Bsdf<R>& b) {
  V4<R> cd = col<R>(b.param->diffuse_color) * R(b.param->diffuse_param[0]);
  V4<R> cg = col<R>(b.param->glossy_color) * R(b.param->glossy_param[0]);
  R ad = luminance(cd.x, cd.y, cd.z);
  R ag = luminance(cg.x, cg.y, cg.z);
  R total = ad + ag;
  if (total < KF(1e-9)) {
    b.diffProb = R(0);
    b.glossyProb = R(0);
  } else {
    b.diffProb = ad / total;
    b.glossyProb = ag / total;
  }
}
// Bsdf.cl:130-160
template <class R>
inline Bsdf<R> setup_bsdf(V4<R> rayd, const Isect<R>& is, const SurfaceParameter* materials) {
  Bsdf<R> b;
  b.frame = get_frame(is.n);
  b.localDirFix = local_coordinate(b.frame, -rayd);
  if (fabs_(b.localDirFix.z) < EPS_COSINE_<R>()) {
    b.materialID = -1;
    return b;
  }
  b.localGeomN = local_coordinate(b.frame, is.ng);
  b.materialID = is.mat;
  b.param = materials + b.materialID;
  component_probabilities(b);
  return b;
}
// Bsdf.cl:162-166, Material.cl:27-31
inline bool is_emitter(const SurfaceParameter* p) {
  float s = p->emission_param[0];
  return luminance(p->emission_color[0] * s, p->emission_color[1] * s, p->emission_color[2] * s) != 0.0f;
}
template <class R> inline bool is_emitter_r(const SurfaceParameter* p) {
  V4<R> c = col<R>(p->emission_color) * R(p->emission_param[0]);
  return luminance(c.x, c.y, c.z) != R(0);
}

// Geometry.cl:1-56
template <class R> inline R Cos2Theta(V4<R> w) { return w.z * w.z; }
template <class R> inline R Sin2Theta(V4<R> w) { return fmax_(R(0), R(1) - Cos2Theta(w)); }
template <class R> inline R SinTheta(V4<R> w) { return sqrt_(Sin2Theta(w)); }
template <class R> inline R TanTheta(V4<R> w) { return SinTheta(w) / w.z; }
template <class R> inline R Tan2Theta(V4<R> w) { return Sin2Theta(w) / Cos2Theta(w); }
template <class R> inline R CosPhi(V4<R> w) { R st = SinTheta(w); return st == R(0) ? R(1) : clamp_(w.x / st, R(-1), R(1)); }
template <class R> inline R SinPhi(V4<R> w) { R st = SinTheta(w); return st == R(0) ? R(0) : clamp_(w.y / st, R(-1), R(1)); }
template <class R> inline R Cos2Phi(V4<R> w) { return CosPhi(w) * CosPhi(w); }
template <class R> inline R Sin2Phi(V4<R> w) { return SinPhi(w) * SinPhi(w); }

// Bsdf.cl:229-264
template <class R> inline R alpha_(V4<R> w, R ax, R ay) { return sqrt_(Cos2Phi(w) * ax * ax + Sin2Phi(w) * ay * ay); }
template <class R> inline R lambda_(V4<R> w, R ax, R ay) {
  R absTan = fabs_(TanTheta(w));
  R a = alpha_(w, ax, ay);
  R a2t = (a * absTan) * (a * absTan);
  R lam = (R(-1) + sqrt_(R(1) + a2t)) / R(2);
  return isinf_(absTan) ? R(0) : lam;
}
template <class R> inline R D_H(V4<R> wh, R ax, R ay) {
  R tan2 = Tan2Theta(wh);
  R cos4 = Cos2Theta(wh) * Cos2Theta(wh);
  R e = (Cos2Phi(wh) / (ax * ax) + Sin2Phi(wh) / (ay * ay)) * tan2;
  R d = R(1) / (PI_<R>() * ax * ay * cos4 * (R(1) + e) * (R(1) + e));
  return isinf_(tan2) ? R(0) : d;
}
template <class R> inline R G_Atten(V4<R> w1, V4<R> w2, R ax, R ay) { return R(1) / (R(1) + lambda_(w1, ax, ay) + lambda_(w2, ax, ay)); }
template <class R> inline R G1_(V4<R> w, R ax, R ay) { return R(1) / (R(1) + lambda_(w, ax, ay)); }

// Bsdf.cl:270-294 (Heitz VNDF sampling)
template <class R> inline V4<R> sample_ggx_vndf(V4<R> v, R ax, R ay, R r1, R r2) {
  V4<R> Vh = normalize4(V4<R>{ax * v.x, ay * v.y, v.z, R(0)});
  R lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  V4<R> T1 = V4<R>{R(1), R(0), R(0), R(0)};
  if (lensq > R(0)) {
    R rs = R(1) / sqrt_(lensq);
    T1 = V4<R>{-Vh.y, Vh.x, R(0), R(0)} * rs;
  }
  V4<R> T2 = cross4(Vh, T1);
  R r = sqrt_(r1);
  R phi = KF(2.0) * PI_<R>() * r2;
  R t1 = r * cos_(phi);
  R t2 = r * sin_(phi);
  R s = KF(0.5) * (KF(1.0) + Vh.z);
  t2 = (KF(1.0) - s) * sqrt_(KF(1.0) - t1 * t1) + s * t2;
  V4<R> Nh = (t1 * T1 + t2 * T2) + sqrt_(max_(R(0), R(1) - t1 * t1 - t2 * t2)) * Vh;
  return normalize4(V4<R>{ax * Nh.x, ay * Nh.y, max_(R(0), Nh.z), R(0)});
}
// Bsdf.cl:297-311
template <class R> inline R VNDF(V4<R> v, V4<R> n, R ax, R ay) {
  return G1_(v, ax, ay) * max_(KF(0.001), dot4(v, n)) * D_H(n, ax, ay) / max_(KF(0.001), v.z);
}
template <class R> inline R pdf_ggx_vndf(V4<R> v, V4<R> ni, R ax, R ay) {
  R DvNi = VNDF(v, ni, ax, ay);
  R VNi = dot4(v, ni);
  return DvNi / (R(4) * VNi);
}
// Bsdf.cl:325-341
template <class R> inline V4<R> reflect_n(V4<R> v, V4<R> n) { return -v + (R(2) * dot4(v, n)) * n; }
// Bsdf.cl:185-189
template <class R> inline V4<R> schlick3(R cosTheta, const float* f0c) {
  R ex = pow_(R(1) - cosTheta, KF(5.0));
  V4<R> f0 = {R(f0c[0]), R(f0c[1]), R(f0c[2]), R(0)};
  return {f0.x + (R(1) - f0.x) * ex, f0.y + (R(1) - f0.y) * ex, f0.z + (R(1) - f0.z) * ex, R(0)};
}
template <class R> inline bool zero4(V4<R> v) { return v.x == R(0) && v.y == R(0) && v.z == R(0) && v.w == R(0); }
template <class R> inline bool zero3(V4<R> v) { return v.x == R(0) && v.y == R(0) && v.z == R(0); }

// Sampling.cl:129-148
template <class R> inline V4<R> sample_cos_hemisphere(R sx, R sy, R* pdfW) {
  R term1 = KF(2.0) * PI_<R>() * sx;
  R term2 = sqrt_(R(1) - sy);
  V4<R> ret = {cos_(term1) * term2, sin_(term1) * term2, sqrt_(sy), R(0)};
  *pdfW = ret.z * R(1) / PI_<R>();  // "ret.z * M_1_PI" with M_1_PI = 1.f/M_PI
  return ret;
}
// Bsdf.cl:380-394
template <class R> inline V4<R> sample_diffuse(const Bsdf<R>& b, R sx, R sy, V4<R>* gen, R* pdfW) {
  if (b.localDirFix.z < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  R unweighted;
  *gen = sample_cos_hemisphere(sx, sy, &unweighted);
  *pdfW += unweighted * b.diffProb;
  // "diffuse_color.xyz * (float)M_1_PI" expands to "xyz * (float)1.f/M_PI" = (xyz * 1) / pi
  V4<R> c = col<R>(b.param->diffuse_color);
  return {c.x * R(1) / PI_<R>(), c.y * R(1) / PI_<R>(), c.z * R(1) / PI_<R>(), R(1)};
}
// Bsdf.cl:396-432
template <class R> inline V4<R> sample_glossy(const Bsdf<R>& b, R sx, R sy, V4<R>* gen, R* pdfW) {
  if (b.localDirFix.z < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  R ax = R(b.param->glossy_param[1]), ay = R(b.param->glossy_param[2]);
  V4<R> wh = sample_ggx_vndf(b.localDirFix, ax, ay, sx, sy);
  *gen = reflect_n(b.localDirFix, wh);
  V4<R> wi = b.localDirFix, wo = *gen;
  R cI = fabs_(b.localDirFix.z), cO = fabs_(gen->z);
  *pdfW += b.glossyProb * pdf_ggx_vndf(wo, wh, ax, ay);
  R fr = G_Atten(wi, wo, ax, ay) * D_H(wh, ax, ay) / (R(4) * cI * cO);
  R whdot = fabs_(dot4(wh, wo));
  V4<R> Fc = schlick3(whdot, b.param->glossy_color);
  if (cI == R(0) || cO == R(0)) Fc = {R(0), R(0), R(0), R(0)};
  if (wh.x == R(0) && wh.y == R(0) && wh.z == R(0)) Fc = {R(0), R(0), R(0), R(0)};
  return {Fc.x * fr, Fc.y * fr, Fc.z * fr, R(0)};
}
// Bsdf.cl:452-467
template <class R> inline V4<R> evaluate_diffuse(const Bsdf<R>& b, V4<R> gen, R* pdfW) {
  if (b.diffProb == R(0)) return {R(0), R(0), R(0), R(0)};
  if (b.localDirFix.z < EPS_COSINE_<R>() || gen.z < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  if (pdfW) *pdfW += b.diffProb * fmax_(R(0), gen.z * R(1) / PI_<R>());
  V4<R> c = col<R>(b.param->diffuse_color);
  return {c.x * R(1) / PI_<R>(), c.y * R(1) / PI_<R>(), c.z * R(1) / PI_<R>(), R(1)};
}
// Bsdf.cl:469-507
template <class R> inline V4<R> evaluate_glossy(const Bsdf<R>& b, V4<R> gen, R* pdfW) {
  if (b.glossyProb == R(0)) return {R(0), R(0), R(0), R(0)};
  if (b.localDirFix.z < EPS_COSINE_<R>() || gen.z < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  R ax = R(b.param->glossy_param[1]), ay = R(b.param->glossy_param[2]);
  V4<R> wi = b.localDirFix, wo = gen;
  V4<R> wh = normalize4(wi + wo);
  R cI = fabs_(wi.z), cO = fabs_(wo.z);
  *pdfW += b.glossyProb * pdf_ggx_vndf(wo, wh, ax, ay);
  R fr = G_Atten(wi, wo, ax, ay) * D_H(wh, ax, ay) / (R(4) * cI * cO);
  R whdot = fabs_(dot4(wh, wo));
  V4<R> Fc = schlick3(whdot, b.param->glossy_color);
  if (cI == R(0) || cO == R(0)) Fc = {R(0), R(0), R(0), R(0)};
  if (wh.x == R(0) && wh.y == R(0) && wh.z == R(0)) Fc = {R(0), R(0), R(0), R(0)};
  return {Fc.x * fr, Fc.y * fr, Fc.z * fr, R(0)};
}
// Bsdf.cl:525-545
template <class R> inline V4<R> evaluate_bsdf(const Bsdf<R>& b, V4<R> worldGen, R* pdfW, R* cosGen) {
  V4<R> result = {R(0), R(0), R(0), R(1)};
  V4<R> gen = local_coordinate(b.frame, worldGen);
  if (gen.z * b.localDirFix.z < R(0)) return result;
  *cosGen = gen.z;
  result = result + evaluate_diffuse(b, gen, pdfW);
  result = result + evaluate_glossy(b, gen, pdfW);
  return result;
}
// Bsdf.cl:555-606
template <class R> inline V4<R> sample_bsdf(const Bsdf<R>& b, R s0, R s1, R s2, V4<R>* worldGen, R* pdfW, R* cosGen) {
  V4<R> result = {R(0), R(0), R(0), R(1)};
  V4<R> gen = {R(0), R(0), R(0), R(0)};
  if (s2 < b.diffProb) {
    result = result + sample_diffuse(b, s0, s1, &gen, pdfW);
    if (zero4(result)) return {R(0), R(0), R(0), R(0)};
    result = result + evaluate_glossy(b, gen, pdfW);
  } else {
    result = result + sample_glossy(b, s0, s1, &gen, pdfW);
    if (zero4(result)) return {R(0), R(0), R(0), R(0)};
    result = result + evaluate_diffuse(b, gen, pdfW);
  }
  *cosGen = fabs_(gen.z);
  if (*cosGen < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  *worldGen = world_coordinate(b.frame, gen);
  return result;
}

// Sampling.cl:212-235
template <class R> inline R mis2(R a, R b) { return a / (a + b); }
template <class R> inline R pdf_a_to_w(R pdfA, R dist, R cosThere) { return pdfA * (dist * dist) / fabs_(cosThere); }

// ------------------------------------------------------------- lights
template <class R>
struct AreaLight {
  V4<R> p1, e1, e2;
  Frame<R> frame;
  V4<R> intensity;
  R invArea;
};
// Light.cl:43-77
template <class R> inline AreaLight<R> get_area_light(const SurfaceParameter* param, const Mesh& m, int tri) {
  AreaLight<R> L;
  V4<R> p1 = P1<R>(m, tri), p2 = P2<R>(m, tri), p3 = P3<R>(m, tri);
  const Face& f = m.faces[tri];
  V4<R> n;
  if (f.nx > -1) {
    V4<R> n1 = ld4<R>(m.normals + 4 * f.nx), n2 = ld4<R>(m.normals + 4 * f.ny), n3 = ld4<R>(m.normals + 4 * f.nz);
    n = normalize4(((n1 + n2) + n3) / KF(3.0));
  } else {
    n = get_normal(p1, p2, p3);
  }
  V4<R> e1 = xyz0(p2 - p1), e2 = xyz0(p3 - p1);
  V4<R> nn = cross4(e1, e2);
  R len = sqrt_(dot3(nn, nn));
  L.invArea = R(2) / len;
  L.frame = get_frame(n);
  L.p1 = p1;
  L.e1 = e1;
  L.e2 = e2;
  L.intensity = col<R>(param->emission_color) * R(param->emission_param[1]);
  return L;
}
// Light.cl:85-109 with Sampling.cl:182-186
template <class R> inline V4<R> illuminate_area_light(const AreaLight<R>& L, V4<R> recv, R sx, R sy, V4<R>* dir, R* dist, R* pdfW) {
  R term = sqrt_(sx);
  R bu = R(1) - term, bv = sy * term;
  V4<R> lp = (L.p1 + L.e1 * bu) + L.e2 * bv;
  *dir = lp - recv;
  R distSqr = dot4(*dir, *dir);
  *dist = sqrt_(distSqr);
  *dir = *dir / *dist;
  R cosN = dot4(L.frame.mZ, -*dir);
  if (cosN < EPS_COSINE_<R>()) return {R(0), R(0), R(0), R(0)};
  *pdfW = L.invArea * distSqr / cosN;
  return L.intensity;
}
// Light.cl:111-127
template <class R> inline V4<R> radiance_area_light(const AreaLight<R>& L, V4<R> rayd, R* pdfA) {
  R cosOut = max_(R(0), dot4(L.frame.mZ, -rayd));
  if (cosOut == R(0)) return {R(0), R(0), R(0), R(0)};
  if (pdfA) *pdfA = L.invArea;
  return L.intensity;
}

// SAT.cl (region sampling straight off an inclusive SAT)
struct SATRegion { int nu, nv, minX, minY, strideX, strideY; };
template <class R> struct SATView { const R* sat; const R* func; };
inline int sat_index(const SATRegion& r, int x, int y) {
  if (x < 0 || y < 0) return -1;
  if (x > r.nu - 1 || y > r.nv - 1) return -1;
  return y * r.nu + x;
}
inline int last_x(const SATRegion& r) { return r.minX + r.strideX - 1; }
inline int last_y(const SATRegion& r) { return r.minY + r.strideY - 1; }
template <class R> inline R sat_value(const SATRegion& r, int x, int y, const R* sat) {  // SAT.cl:135-147
  if (x < 0) return R(0);
  if (y < 0) return R(0);
  if (x > last_x(r)) return R(0);
  if (y > last_y(r)) return R(0);
  return sat[sat_index(r, x, y)];
}
template <class R> inline R sat_range(const SATRegion& r, int minX, int minY, int maxX, int maxY, const R* sat) {  // :149-156
  R D1 = sat_value(r, maxX, maxY, sat);
  R C1 = sat_value(r, minX - 1, maxY, sat);
  R B1 = sat_value(r, maxX, minY - 1, sat);
  R A1 = sat_value(r, minX - 1, minY - 1, sat);
  return A1 + D1 - B1 - C1;
}
template <class R> inline R func_int_cond(const SATRegion& r, int y, const R* sat) { return sat_range(r, r.minX, y, last_x(r), y, sat); }
template <class R> inline R conditional(const SATRegion& r, int x, int y, const R* sat) {
  R fi = func_int_cond(r, y, sat);
  return sat_range(r, r.minX, y, x - 1, y, sat) / fi;
}
template <class R> inline R marginal(const SATRegion& r, int y, const R* sat) {
  R last = sat_range(r, r.minX, r.minY, last_x(r), last_y(r), sat);
  return sat_range(r, r.minX, r.minY, last_x(r), y - 1, sat) / last;
}
template <class R> inline R func_at(const SATRegion& r, int x, int y, const R* func) {
  int i = sat_index(r, x, y);
  return func[i < 0 ? 0 : i];
}
template <class R> inline R pdf_cond(const SATRegion& r, int x, int y, const R* sat, const R* func) {
  return func_at(r, x, y, func) / func_int_cond(r, y, sat);
}
template <class R> inline R pdf_marg(const SATRegion& r, int y, const R* sat) {
  R fi = func_int_cond(r, y, sat);
  R last = sat_range(r, r.minX, r.minY, last_x(r), last_y(r), sat);
  return (fi * R(r.strideX * r.strideY)) / last;
}
template <class R> inline int upper_bound_cond(const SATRegion& r, int y, int first, int last, R value, const R* sat) {
  int begin = first, end = last;
  while (begin != end) {
    int mid = begin + (end - begin) / 2;
    R mv = conditional(r, mid, y, sat);
    bool right = !(value < mv);
    begin = right ? mid + 1 : begin;
    end = right ? end : mid;
  }
  return begin;
}
template <class R> inline int upper_bound_marg(const SATRegion& r, int first, int last, R value, const R* sat) {
  int begin = first, end = last;
  while (begin != end) {
    int mid = begin + (end - begin) / 2;
    R mv = marginal(r, mid, sat);
    bool right = !(value < mv);
    begin = right ? mid + 1 : begin;
    end = right ? end : mid;
  }
  return begin;
}
// SAT.cl:244-259, :275-290, :313-323
template <class R> inline void sample_continuous(const SATRegion& r, R u0, R u1, R* uv, int* off, R* pdf, const R* sat, const R* func) {
  R pdfs[2];
  {
    int ptr = upper_bound_marg(r, r.minY, r.minY + r.strideY, u1, sat);
    int o = max_(0, ptr - 1);
    off[1] = o;
    R du = (u1 - marginal(r, o, sat)) / (marginal(r, o + 1, sat) - marginal(r, o, sat));
    pdfs[1] = pdf_marg(r, o, sat);
    uv[1] = (R(o) + du) / R(r.nv);
  }
  {
    int y = off[1];
    int ptr = upper_bound_cond(r, y, r.minX, r.minX + r.strideX, u0, sat);
    int o = max_(0, ptr - 1);
    off[0] = o;
    R du = (u0 - conditional(r, o, y, sat)) / (conditional(r, o + 1, y, sat) - conditional(r, o, y, sat));
    pdfs[0] = pdf_cond(r, o, y, sat, func);
    uv[0] = (R(o) + du) / R(r.nu);
  }
  pdf[0] = pdfs[0] * pdfs[1];
}
// SAT.cl:261-273, :292-300, :325-334
template <class R> inline void sample_discrete(const SATRegion& r, R u0, R u1, int* off, R* pdf, const R* sat, const R* func) {
  R pdfs[2];
  int ptr = upper_bound_marg(r, r.minY, r.minY + r.strideY, u1, sat);
  off[1] = max_(0, ptr - 1);
  pdfs[1] = pdf_marg(r, off[1], sat);
  ptr = upper_bound_cond(r, off[1], r.minX, r.minX + r.strideX, u0, sat);
  off[0] = max_(0, ptr - 1);
  pdfs[0] = pdf_cond(r, off[0], off[1], sat, func);
  pdf[0] = pdfs[0] * pdfs[1] / R(r.strideX * r.strideY);
}
// SAT.cl:336-342
template <class R> inline R pdf_sat(const SATRegion& r, int x, int y, const R* sat, const R* func) {
  return pdf_cond(r, x, y, sat, func) * pdf_marg(r, y, sat);
}

// Util.cl:397-417, :423-439
template <class R> inline void spherical_xy(int w, int h, V4<R> d, int* x, int* y) {
  R phi = acos_(d.y);
  R theta = atan2_(d.z, d.x);
  *x = (int)((KF(0.5) - KF(0.5) * theta / PI_<R>()) * R(w));
  *y = (int)((phi / PI_<R>()) * R(h));
}
template <class R> inline int spherical_index(int w, int h, V4<R> d) {
  int x, y;
  spherical_xy(w, h, d, &x, &y);
  int idx = (int)((float)x + (float)y * (float)w);
  if (idx < 0) idx = 0;
  if (idx > w * h - 1) idx = w * h - 1;
  return idx;
}
template <class R> inline V4<R> spherical_direction(R u, R v) {
  R phi = PI_<R>() * v;
  R theta = u * R(2) * PI_<R>();
  return {-sin_(phi) * cos_(theta), cos_(phi), sin_(phi) * sin_(theta), R(0)};
}

template <class R>
struct Env {
  const float* rgb = nullptr;  // float4 per texel
  const R* lum = nullptr;
  const R* sat = nullptr;
  int w = 0, h = 0;
  bool present = false;
  // adaptive light grid (mode 1): FP32 func and per-cell SAT of nu x nv values,
  // (nu/rx) x (nv/ry) cells of rx x ry tiles; accum may be NULL
  bool grid_on = false;
  const float* gfunc = nullptr;
  const float* gsat = nullptr;
  float* gaccum = nullptr;
  int nu = 0, nv = 0, rx = 0, ry = 0;
  float cam[4] = {0, 0, 0, 0};
  SATRegion region() const { return SATRegion{w, h, 0, 0, w, h}; }
};
// Light.cl:195-227
template <class R> inline V4<R> illuminate_env(const Env<R>& E, V4<R> s, V4<R>* dir, R* dist, R* pdfW) {
  R uv[2];
  int off[2];
  R pdf[1];
  SATRegion reg = E.region();
  sample_continuous(reg, s.x, s.y, uv, off, pdf, E.sat, E.lum);
  *dir = spherical_direction(uv[0], uv[1]);
  int idx = spherical_index(E.w, E.h, *dir);
  V4<R> c = ld4<R>(E.rgb + 4 * (size_t)idx);
  R sinT = sin_(uv[1] * PI_<R>());
  *pdfW = pdf[0] / (R(2) * PI_<R>() * PI_<R>() * sin_(uv[1] * PI_<R>()));
  *dist = KF(3.402823e+38);
  if (sinT == R(0)) *pdfW = R(0);
  return c;
}
// Light.cl:270-286
template <class R> inline V4<R> radiance_env(const Env<R>& E, V4<R> d, R* pdfA) {
  int x, y;
  spherical_xy(E.w, E.h, d, &x, &y);
  int idx = spherical_index(E.w, E.h, d);
  V4<R> c = ld4<R>(E.rgb + 4 * (size_t)idx);
  SATRegion reg = E.region();
  int xc = x > E.w - 1 ? E.w - 1 : x, yc = y > E.h - 1 ? E.h - 1 : y;
  R pdfXY = pdf_sat(reg, xc, yc, E.sat, E.lum);
  R v = R(y) / R(reg.strideY);
  *pdfA = pdfXY / (R(2) * PI_<R>() * PI_<R>() * sin_(v * PI_<R>()));
  return c;
}

// ------------------------------------------------ adaptive light grid
// LightGrid.cl:39-343 and the grid versions of the environment light
// (illuminateEnvironmentLight1 / getRadianceEnvironmentLight1, Light.cl:140-268),
// which the reference never calls. The restatement wires them in: the shading
// point's cell is the direction camera -> point (subgridIndexFromCamera, xyz
// lanes), the tile is drawn from the cell's SAT (sampleSubgridContinuous,
// cell (cx, cy) starting at (cx * rx, cy * ry) as subgridGlobalIndex2), the texel
// from the tile's region of the full-map SAT (getSubgridUnitBound +
// getSubRegionFromUnitBound, SAT.cl:28-44), and the direction pdf is
// pdfLL * pdfSS / (2 pi^2 sin) (the reference leaves out pdfLL). An empty cell
// or tile gives no light sample and pdf 0.
template <class R> inline int grid_cell(const Env<R>& E, V4<R> p) {
  const int cw = E.nu / E.rx, ch = E.nv / E.ry;
  V4<R> d = normalize3(V4<R>{p.x - R(E.cam[0]), p.y - R(E.cam[1]), p.z - R(E.cam[2]), R(0)});
  return spherical_index(cw, ch, d);
}
// A cell holds its own SAT: it is sampled as region (0, 0, rx, ry) of the grid
// arrays offset to its first tile (row pitch nu), so reads left of or above the
// cell give 0 as getSubgridValueSAT's range check does (LightGrid.cl:142-147).
template <class R> inline size_t grid_cell_base(const Env<R>& E, int cell) {
  const int cw = E.nu / E.rx;
  return (size_t)((cell / cw) * E.ry) * E.nu + (size_t)((cell % cw) * E.rx);
}
template <class R> inline SATRegion grid_cell_region(const Env<R>& E) { return SATRegion{E.nu, E.nv, 0, 0, E.rx, E.ry}; }
template <class R> inline SATRegion env_tile_region(const Env<R>& E, int tx, int ty) {
  const float ux0 = (float)tx / (float)E.rx, uy0 = (float)ty / (float)E.ry;
  const float ux1 = (float)(tx + 1) / (float)E.rx, uy1 = (float)(ty + 1) / (float)E.ry;
  const int x0 = (int)((float)E.w * ux0), y0 = (int)((float)E.h * uy0);
  const int x1 = (int)((float)E.w * ux1), y1 = (int)((float)E.h * uy1);
  return SATRegion{E.w, E.h, x0, y0, x1 - x0, y1 - y0};
}
template <class R> inline V4<R> illuminate_env_grid(const Env<R>& E, V4<R> p, V4<R> s, V4<R>* dir, R* dist, R* pdfW) {
  const size_t base = grid_cell_base(E, grid_cell(E, p));
  const SATRegion rc = grid_cell_region(E);
  float uvLL[2], pdfLL[1];
  int offLL[2];
  sample_continuous<float>(rc, float(s.x), float(s.y), uvLL, offLL, pdfLL, E.gsat + base, E.gfunc + base);
  *dist = KF(3.402823e+38);
  *pdfW = R(0);
  if (!(pdfLL[0] > 0.f)) return {R(0), R(0), R(0), R(0)};
  const SATRegion rt = env_tile_region(E, offLL[0], offLL[1]);
  R uv[2], pdfSS[1];
  int off[2];
  sample_continuous(rt, s.z, s.w, uv, off, pdfSS, E.sat, E.lum);
  if (!(pdfSS[0] > R(0))) return {R(0), R(0), R(0), R(0)};
  *dir = spherical_direction(uv[0], uv[1]);
  int idx = spherical_index(E.w, E.h, *dir);
  V4<R> c = ld4<R>(E.rgb + 4 * (size_t)idx);
  R sinT = sin_(uv[1] * PI_<R>());
  *pdfW = (R(pdfLL[0]) * pdfSS[0]) / (R(2) * PI_<R>() * PI_<R>() * sin_(uv[1] * PI_<R>()));
  if (sinT == R(0)) *pdfW = R(0);
  return c;
}
// The pdf of direction d under illuminate_env_grid from point p (tile = the one
// holding d's texel; the sine term with v = y / h over the whole map), the
// radiance, and the accumulation of the texel's luminance at (cell, tile).
template <class R> inline V4<R> radiance_env_grid(const Env<R>& E, V4<R> p, V4<R> d, R* pdfA, bool accumulate) {
  int x, y;
  spherical_xy(E.w, E.h, d, &x, &y);
  int idx = spherical_index(E.w, E.h, d);
  V4<R> c = ld4<R>(E.rgb + 4 * (size_t)idx);
  const int xc = x > E.w - 1 ? E.w - 1 : (x < 0 ? 0 : x), yc = y > E.h - 1 ? E.h - 1 : (y < 0 ? 0 : y);
  const int tx = xc / (E.w / E.rx), ty = yc / (E.h / E.ry);
  const size_t base = grid_cell_base(E, grid_cell(E, p));
  const SATRegion rc = grid_cell_region(E);
  const float pdfLL = pdf_cond(rc, tx, ty, E.gsat + base, E.gfunc + base) * pdf_marg(rc, ty, E.gsat + base);
  const SATRegion rt = env_tile_region(E, tx, ty);
  const R pdfSS = pdf_cond(rt, xc, yc, E.sat, E.lum) * pdf_marg(rt, yc, E.sat);
  const R v = R(y) / R(E.h);
  R pdf = (R(pdfLL) * pdfSS) / (R(2) * PI_<R>() * PI_<R>() * sin_(v * PI_<R>()));
  *pdfA = pdf > R(0) ? pdf : R(0);
  if (accumulate && E.gaccum) {
    float* a = E.gaccum + base + (size_t)ty * E.nu + tx;
    *a = *a + luminance(float(c.x), float(c.y), float(c.z));
  }
  return c;
}

// Util.cl:537-549 (every lane finite and non-negative)
template <class R> inline bool abs_valid4(V4<R> v) {
  R a[4] = {v.x, v.y, v.z, v.w};
  for (int i = 0; i < 4; ++i)
    if (isnan_(a[i]) || isinf_(a[i]) || a[i] < R(0)) return false;
  return true;
}

// ------------------------------------------------------------ camera
template <class R> struct M4 { V4<R> m0, m1, m2, m3; };
template <class R> inline V4<R> column(const M4<R>& m, int i) {
  auto g = [&](V4<R> r) { return i == 0 ? r.x : i == 1 ? r.y : i == 2 ? r.z : r.w; };
  return {g(m.m0), g(m.m1), g(m.m2), g(m.m3)};
}
template <class R> inline M4<R> mul(const M4<R>& a, const M4<R>& b) {  // Matrix.cl:130-160
  M4<R> r;
  const V4<R>* rows[4] = {&a.m0, &a.m1, &a.m2, &a.m3};
  V4<R>* out[4] = {&r.m0, &r.m1, &r.m2, &r.m3};
  for (int i = 0; i < 4; ++i)
    *out[i] = {dot4(*rows[i], column(b, 0)), dot4(*rows[i], column(b, 1)), dot4(*rows[i], column(b, 2)),
               dot4(*rows[i], column(b, 3))};
  return r;
}
template <class R> inline void set_col(M4<R>& m, int i, V4<R> c) {  // Matrix.cl:100-118
  R* r0 = &m.m0.x + i;
  R* r1 = &m.m1.x + i;
  R* r2 = &m.m2.x + i;
  R* r3 = &m.m3.x + i;
  *r0 = c.x;
  *r1 = c.y;
  *r2 = c.z;
  *r3 = c.w;
}
template <class R> inline M4<R> identity() {
  return {{R(1), R(0), R(0), R(0)}, {R(0), R(1), R(0), R(0)}, {R(0), R(0), R(1), R(0)}, {R(0), R(0), R(0), R(1)}};
}
// Matrix.cl:216-241 (view_to_world = camera.mInv)
template <class R> inline M4<R> camera_to_world(V4<R> pos, V4<R> lookat, V4<R> up) {
  V4<R> d = normalize4(lookat - pos);
  V4<R> r = normalize4(cross4(d, up));
  V4<R> u = cross4(r, d);
  M4<R> eInv = identity<R>();
  set_col(eInv, 3, V4<R>{pos.x, pos.y, pos.z, R(1)});
  M4<R> v2w = identity<R>();
  set_col(v2w, 0, r);
  set_col(v2w, 1, u);
  set_col(v2w, 2, d * R(-1));
  return mul(eInv, v2w);
}
// Matrix.cl:188-214
template <class R> inline V4<R> transform_vector(const M4<R>& m, V4<R> v) { return {dot4(m.m0, v), dot4(m.m1, v), dot4(m.m2, v), R(0)}; }
template <class R> inline V4<R> transform_point(const M4<R>& m, V4<R> v) {
  V4<R> res = {dot3(m.m0, v) + m.m0.w, dot3(m.m1, v) + m.m1.w, dot3(m.m2, v) + m.m2.w, dot3(m.m3, v) + m.m3.w};
  if (res.w == R(1)) return {res.x, res.y, res.z, R(0)};
  return {res.x / res.w, res.y / res.w, res.z / res.w, R(0)};
}

// Initialize.cl:129-172 (ray for pixel `id`, random pair already drawn)
template <class R> inline void camera_ray(const CameraF& cam, int id, R sx, R sy, Ray<R>& r) {
  int wdt = (int)cam.dimension[0];
  R px = R(id % wdt), py = R(id / wdt);
  V4<R> pos = ld4<R>(cam.position), look = ld4<R>(cam.lookat), up = ld4<R>(cam.up);
  M4<R> mInv = camera_to_world(pos, look, up);
  R dimx = R(cam.dimension[0]), dimy = R(cam.dimension[1]);
  R fov_rad = R(cam.fov) * KF(0.017453292519943295);
  R dd = R(1) / tan_(fov_rad / R(2));
  R a = dimx / dimy;
  R j1 = R(1) / dimx * (R(2) * sx - R(1));
  R j2 = R(1) / dimy * (R(2) * sy - R(1));
  V4<R> d = normalize4(V4<R>{a * (R(2) * px / dimx - R(1) + j1), R(-2) * py / dimy + R(1) + j2, -dd, R(0)});
  V4<R> o = transform_point(mInv, V4<R>{R(0), R(0), R(0), R(0)});
  d = transform_vector(mInv, d);
  init_ray(r, o, d, KF(0.001), INF_<R>());
}

// --------------------------------------------------------- render loop
struct RenderParams {
  int width, height, max_depth;
  int mode;          // 0: reference semantics; 1: benchmark-config semantics
  float frame_count; // State.frameCount (1 for the first frame)
  int rr_depth;      // mode 1: Russian roulette from this bounce on (0 = off)
  bool grid_accum = false;  // mode 1 with the grid on: environment hits accumulate into it
  // mode 1 only: render just these pixels of the frame (npix of them); queue slot
  // q starts pixel pix_of[q], keyed on it as the full frame keys it, and
  // accumulates into accum[q]. NULL: every pixel, accum indexed by pixel.
  const int* pix_of = nullptr;
  int npix = 0;
};

// Config-mode seed pair of a (bounce, stage): stage 0 raygen, 1 light pick+sample,
// 2 BSDF sample, 3 Russian roulette.
inline void stage_seed(int bounce, int stage, int32_t* sx, int32_t* sy) {
  *sx = (int32_t)(wanghash((int32_t)(0x5EED0000u + 16u * (uint32_t)bounce + 2u * (uint32_t)stage)) | 1u);
  *sy = (int32_t)(wanghash((int32_t)(0x5EED8000u + 16u * (uint32_t)bounce + 2u * (uint32_t)stage)) | 1u);
}
inline int32_t pixel_gid(int pixel) { return (int32_t)((uint32_t)pixel ^ 0x9E3779B9u); }

// ------------------------------------------------------------ textures
// Textures bound for the next frames (test infrastructure state): an ARGB texel
// pool and, per material, 4 entries (first texel, width, height, 0) for
// diffuse, glossy, roughness, mirror; width 0 = no image.
struct Textures {
  const int* texels = nullptr;
  const int* ref = nullptr;
  int nref = 0;  // entries (4 ints each)
};
Textures g_tex;

// Java's (int) cast of a float (JLS 5.1.3): NaN -> 0, saturating.
inline int java_f2i(float x) {
  if (x != x) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return -2147483647 - 1;
  return (int)x;
}
// TextureInfoCache.getDomainValue (TextureInfoCache.java:131-136)
inline float domain_value(float x) { return x < 0 ? (x - (float)java_f2i(x)) + 1.0f : x - (float)java_f2i(x); }
// CTextureApplyPass.process (CTextureApplyPass.java:47-87): the ARGB texel at
// ((int)(u' (W - 1)), (int)(v' (H - 1))), the index clamped to the image.
inline int texel_at(const Textures& T, int entry, float u, float v) {
  const int* r = T.ref + 4 * (size_t)entry;
  float dx = domain_value(u) * ((float)r[1] - 1.0f);
  float dy = domain_value(v) * ((float)r[2] - 1.0f);
  int x = std::min(std::max(java_f2i(dx), 0), r[1] - 1);
  int y = std::min(std::max(java_f2i(dy), 0), r[2] - 1);
  return T.texels[r[0] + (size_t)y * r[1] + x];
}
// getFloat4ARGB (Util.cl:482-493)
inline void argb_to_float4(int c, float* out) {
  out[3] = ((c >> 24) & 0xFF) / 255.0f;
  out[0] = ((c >> 16) & 0xFF) / 255.0f;
  out[1] = ((c >> 8) & 0xFF) / 255.0f;
  out[2] = (c & 0xFF) / 255.0f;
}
// texturePassGI, CTextureApplyPass.process and updateToTextureColorGI
// (Render.cl:127-231): the flagged textures of material `mat` at uv replace the
// diffuse colour, the glossy colour, and the roughness (glossy_param.y/z from red
// and green, at least 0.001). A flagged texture without an image reads ARGB 0.
inline void apply_textures(const Textures& T, int mat, float u, float v, SurfaceParameter& p) {
  auto argb = [&](int kind) {
    int e = 4 * mat + kind;
    return (e < T.nref && T.ref[4 * (size_t)e + 1] > 0) ? texel_at(T, e, u, v) : 0;
  };
  if (p.isDiffuseTexture) argb_to_float4(argb(0), p.diffuse_color);
  if (p.isGlossyTexture) argb_to_float4(argb(1), p.glossy_color);
  if (p.isRoughnessTexture) {
    float c[4];
    argb_to_float4(argb(2), c);
    p.glossy_param[1] = std::fmax(0.001f, c[0]);
    p.glossy_param[2] = std::fmax(0.001f, c[1]);
  }
}
inline bool has_textures(const SurfaceParameter& p) {
  return p.isDiffuseTexture || p.isGlossyTexture || p.isRoughnessTexture;
}

template <class R>
struct Path {
  V4<R> throughput, hitpoint;
  int lastSpecular;
  R lastPdfW;
  Bsdf<R> bsdf;
  SurfaceParameter textured;  // the path's textured copy of its material
};

struct Scene {
  Mesh mesh;
  const SurfaceParameter* materials;
  const BVHNode* nodes;
  const BoundingBox* bounds;
  const int* light_faces;  // LightInfo.faceId list (prefix-scan order)
  int nlights;
};

struct RayCounts { long long primary = 0, extension = 0, shadow = 0; };

template <class R>
void render_frame(const Scene& S, const Env<R>& E, const CameraF& cam_in, const RenderParams& P,
                  const int* seeds /* mode 0: 1 + 2*max_depth pairs */, R* accum /* float4 per pixel */,
                  int* counts_out, RayCounts* rc) {
  const int N = P.pix_of ? P.npix : P.width * P.height;
  auto pix = [&](int q) { return P.pix_of ? P.pix_of[q] : q; };  // the frame pixel of queue origin q
  CameraF cam = cam_in;
  cam.dimension[0] = (float)P.width;
  cam.dimension[1] = (float)P.height;
  std::vector<Ray<R>> rays(N);
  std::vector<Isect<R>> isects(N);
  std::vector<Path<R>> paths(N);
  std::vector<int> pixels(N);
  int count = N;
  int k = 0;
  auto next_state = [&](int32_t* sx, int32_t* sy) { *sx = seeds[2 * k]; *sy = seeds[2 * k + 1]; ++k; };
  auto add = [&](int pixel, V4<R> v) {
    if (!abs_valid4(v)) return;
    R* a = accum + 4 * (size_t)pixel;
    a[0] = a[0] + v.x;
    a[1] = a[1] + v.y;
    a[2] = a[2] + v.z;
    a[3] = a[3] + v.w;
  };

  // frame start: InitCameraRayDataJitter, InitPathData, InitIntersection, InitIntDataToIndex
  int32_t sx = 0, sy = 0;
  if (P.mode == 0) next_state(&sx, &sy); else stage_seed(0, 0, &sx, &sy);
  for (int id = 0; id < N; ++id) {
    Seed s = generate_seed(sx, sy, P.frame_count, P.mode == 0 ? id : pixel_gid(pix(id)));
    R r0 = R(get_random(s));
    R r1 = R(get_random(s));
    camera_ray(cam, pix(id), r0, r1, rays[id]);
    Path<R>& pa = paths[id];
    pa.throughput = {R(1), R(1), R(1), R(1)};
    pa.lastSpecular = 1;
    pa.lastPdfW = R(1);
    pa.bsdf = Bsdf<R>();
    pa.hitpoint = {R(0), R(0), R(0), R(0)};
    init_isect(isects[id]);
    isects[id].ng = {R(0), R(0), R(0), R(0)};
    pixels[id] = id;
  }
  if (rc) rc->primary += N;

  for (int b = 1; b <= P.max_depth; ++b) {
    // IntersectPrimitives over the live queue
    for (int j = 0; j < count; ++j) {
      int child = -1;
      bool hit = intersect_mesh(rays[j], &child, S.mesh, S.nodes, S.bounds, false, nullptr);
      if (hit) hit_record(rays[j], child, S.mesh, isects[j]);
      else { isects[j].hit = 0; isects[j].mat = -1; }
    }
    for (int j = count; j < N; ++j) { isects[j].hit = 0; isects[j].mat = -1; }
    if (rc && b > 1) rc->extension += count;
    if (P.mode == 0) next_state(&sx, &sy);  // allocateState after the intersection (unused)

    // SetupBSDFPath (Render.cl:10-40)
    for (int j = 0; j < count; ++j) {
      Isect<R>& is = isects[j];
      if (!is.hit) continue;
      Bsdf<R> bs = setup_bsdf(rays[j].d, is, S.materials);
      if (bs.materialID < 0) { is.hit = 0; continue; }
      paths[pixels[j]].bsdf = bs;
    }
    // LightHitPass (Render.cl:42-125)
    for (int j = 0; j < count; ++j) {
      Isect<R>& is = isects[j];
      Path<R>& pa = paths[pixels[j]];
      if (is.hit) {
        const Bsdf<R>& bs = pa.bsdf;
        if (!is_emitter_r<R>(bs.param)) continue;
        R pick = R(1) / R(S.nlights);
        if (P.mode == 1 && E.present && S.nlights > 0) pick = pick * KF(0.5);
        AreaLight<R> L = get_area_light<R>(bs.param, S.mesh, is.id);
        R pdfA = R(0);
        V4<R> c = radiance_area_light(L, rays[j].d, &pdfA);
        if (zero3(c)) continue;
        R w = R(1);
        if (!pa.lastSpecular) {
          R pdfW = pdf_a_to_w(pdfA, rays[j].tMax, bs.localDirFix.z);
          w = mis2(pa.lastPdfW, pdfW * pick);
        }
        add(pixels[j], pa.throughput * c * w);
        is.hit = 0;
      } else if (E.present) {
        R pdfW;
        V4<R> c = (P.mode == 1 && E.grid_on)
                      ? radiance_env_grid(E, pa.hitpoint, rays[j].d, &pdfW, P.grid_accum && !pa.lastSpecular)
                      : radiance_env(E, rays[j].d, &pdfW);
        if (zero3(c)) continue;
        if (P.mode == 1 && S.nlights > 0) pdfW = pdfW * KF(0.5);
        R w = R(1);
        if (!pa.lastSpecular) w = mis2(pa.lastPdfW, pdfW);
        add(pixels[j], pa.throughput * c * w);
      }
    }
    // CCompact.execute: stable compaction of live hits with their pixel ids
    int kept = 0;
    for (int j = 0; j < count; ++j) {
      if (!isects[j].hit) continue;
      isects[kept] = isects[j];
      pixels[kept] = pixels[j];
      ++kept;
    }
    for (int j = kept; j < N; ++j) { init_isect(isects[j]); pixels[j] = 0; }
    count = kept;
    if (counts_out) counts_out[b - 1] = count;

    // texture pass (CDeviceGI.java:241-244) over the live queue
    if (g_tex.nref > 0) {
      for (int j = 0; j < count; ++j) {
        Path<R>& pa = paths[pixels[j]];
        if (!pa.bsdf.param || !has_textures(*pa.bsdf.param)) continue;
        pa.textured = *pa.bsdf.param;
        apply_textures(g_tex, pa.bsdf.materialID, (float)isects[j].uv[0], (float)isects[j].uv[1], pa.textured);
        pa.bsdf.param = &pa.textured;
      }
    }

    // DirectLight (Render.cl:377-466)
    int32_t lx = 0, ly = 0, bx = 0, by = 0;
    if (P.mode == 0) { next_state(&lx, &ly); bx = lx; by = ly; }
    else { stage_seed(b, 1, &lx, &ly); stage_seed(b, 2, &bx, &by); }
    for (int j = 0; j < count; ++j) {
      Isect<R>& is = isects[j];
      Path<R>& pa = paths[pixels[j]];
      Seed s = generate_seed(lx, ly, P.frame_count, P.mode == 0 ? j : pixel_gid(pix(pixels[j])));
      V4<R> dir = {R(0), R(0), R(0), R(0)};
      R dist = R(0), pdfW = R(0), pick = R(1);
      V4<R> smp = {R(get_random(s)), R(get_random(s)), R(get_random(s)), R(get_random(s))};
      V4<R> rad = {R(0), R(0), R(0), R(0)};
      bool sample_mesh = false, sample_env = false;
      if (E.present && S.nlights > 0) {
        R rnd = R(get_random(s));
        pick = pick * KF(0.5);
        if (rnd < KF(0.5)) sample_mesh = true; else sample_env = true;
      } else if (E.present) {
        sample_env = true;
      } else if (S.nlights > 0) {
        sample_mesh = true;
      }
      if (sample_mesh) {
        int li = random_int_range(s, S.nlights);
        int tri = S.light_faces[P.mode == 0 ? 0 : li];  // Render.cl:305 reads light 0
        pick = pick * (R(1) / R(S.nlights));
        const SurfaceParameter* lp = S.materials + (S.mesh.faces[tri].mat & 0xFFFF);
        AreaLight<R> L = get_area_light<R>(lp, S.mesh, tri);
        rad = illuminate_area_light(L, is.p, smp.x, smp.y, &dir, &dist, &pdfW);
      } else if (sample_env) {
        rad = (P.mode == 1 && E.grid_on) ? illuminate_env_grid(E, is.p, smp, &dir, &dist, &pdfW)
                                         : illuminate_env(E, smp, &dir, &dist, &pdfW);
      }
      if (!zero3(rad)) {
        R bsdfPdf = R(0), cosOut = R(0);
        V4<R> f = evaluate_bsdf(pa.bsdf, dir, &bsdfPdf, &cosOut);
        if (!zero3(f)) {
          R w = mis2(pdfW, bsdfPdf);
          R sc = (w * cosOut / (pick * pdfW));
          V4<R> contrib = {sc * (rad.x * f.x) * pa.throughput.x, sc * (rad.y * f.y) * pa.throughput.y,
                           sc * (rad.z * f.z) * pa.throughput.z, R(1)};
          Ray<R> sh;
          init_ray(sh, is.p, dir, KF(0.0001), dist - R(2) * KF(1e-3));
          if (rc) rc->shadow++;
          int dummy;
          if (!intersect_mesh(sh, &dummy, S.mesh, S.nodes, S.bounds, true, nullptr)) add(pixels[j], contrib);
        }
      }
    }
    // SampleBSDFRayDirection (Render.cl:233-285), then Russian roulette in mode 1
    int32_t rx = 0, ry = 0;
    if (P.mode == 1) stage_seed(b, 3, &rx, &ry);
    int live = 0;
    for (int j = 0; j < count; ++j) {
      Isect<R>& is = isects[j];
      Path<R>& pa = paths[pixels[j]];
      Seed s = generate_seed(bx, by, P.frame_count, P.mode == 0 ? j : pixel_gid(pix(pixels[j])));
      R s0 = R(get_random(s)), s1 = R(get_random(s)), s2 = R(get_random(s));
      V4<R> dir = {R(0), R(0), R(0), R(0)};
      R pdf = R(0), cosOut = R(0);
      V4<R> f = sample_bsdf(pa.bsdf, s0, s1, s2, &dir, &pdf, &cosOut);
      R q = cosOut / pdf;
      pa.throughput = pa.throughput * (f * q);
      pa.lastSpecular = 0;
      pa.lastPdfW = pdf;
      pa.hitpoint = is.p;
      bool alive = true;
      if (P.mode == 1 && P.rr_depth > 0 && b >= P.rr_depth) {
        Seed rs = generate_seed(rx, ry, P.frame_count, pixel_gid(pix(pixels[j])));
        R u = R(get_random(rs));
        R m = max_(pa.throughput.x, max_(pa.throughput.y, pa.throughput.z));
        R cont = min_(KF(0.95), m);
        if (!(u < cont)) alive = false;
        else pa.throughput = pa.throughput / cont;
      }
      init_ray(rays[j], is.p, dir, KF(0.001), INF_<R>());
      init_isect(is);
      if (P.mode == 1) {  // mode 1 compacts the terminated paths out right away
        if (alive) { rays[live] = rays[j]; pixels[live] = pixels[j]; ++live; }
      }
    }
    if (P.mode == 1) {
      count = live;
      if (counts_out) counts_out[b - 1] = count;  // queue entering the next bounce
    }
  }
}

// ------------------------------------------------------------ BVH build
// CNormalBVH.java:45-148. The partition of CNormalBVH.java:132 lives in an
// un-vendored library; this builder (and the product's) uses a stable split
// "centroid[dim] < split" on the triangle bounds' centres.
struct BvhBuilder {
  const float* pts;
  const Face* faces;
  int n;
  std::vector<int> objects;
  std::vector<BVHNode>* nodes;
  std::vector<BoundingBox>* bounds;
  std::vector<float> cen;  // 3 per triangle
  std::vector<float> tb;   // 6 per triangle: min xyz, max xyz
  std::vector<int> tmp;
  int ptr = 1;
  int max_depth = 0;

  void tri_bound(int t) {
    const Face& f = faces[t];
    const float* p[3] = {pts + 4 * f.vx, pts + 4 * f.vy, pts + 4 * f.vz};
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 3; ++k)
      for (int a = 0; a < 3; ++a) {
        if (p[k][a] < mn[a]) mn[a] = p[k][a];
        if (p[k][a] > mx[a]) mx[a] = p[k][a];
      }
    for (int a = 0; a < 3; ++a) {
      tb[6 * t + a] = mn[a];
      tb[6 * t + 3 + a] = mx[a];
      cen[3 * t + a] = 0.5f * (mn[a] + mx[a]);
    }
  }

  void subdivide(int parent, int start, int end, int depth) {
    if (depth > max_depth) max_depth = depth;
    float bmn[3] = {INFINITY, INFINITY, INFINITY}, bmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    float cmn[3] = {INFINITY, INFINITY, INFINITY}, cmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int p = start; p < end; ++p) {
      int t = objects[p];
      for (int a = 0; a < 3; ++a) {
        float lo = tb[6 * t + a], hi = tb[6 * t + 3 + a], c = cen[3 * t + a];
        if (lo < bmn[a]) bmn[a] = lo;
        if (lo > bmx[a]) bmx[a] = lo;
        if (hi < bmn[a]) bmn[a] = hi;
        if (hi > bmx[a]) bmx[a] = hi;
        if (c < cmn[a]) cmn[a] = c;
        if (c > cmx[a]) cmx[a] = c;
      }
    }
    (*nodes)[parent].bound = parent;
    BoundingBox& bb = (*bounds)[parent];
    for (int a = 0; a < 3; ++a) { bb.mn[a] = bmn[a]; bb.mx[a] = bmx[a]; }
    bb.mn[3] = 0.f;
    bb.mx[3] = 0.f;
    if (end - start < 2) {
      (*nodes)[parent].child = objects[start];
      (*nodes)[parent].isLeaf = 1;
      return;
    }
    int li = ptr++, ri = ptr++;
    BVHNode ln{}, rn{};
    ln.parent = parent;
    rn.parent = parent;
    ln.sibling = ri;
    rn.sibling = li;
    (*nodes)[li] = ln;
    (*nodes)[ri] = rn;
    (*nodes)[parent].left = li;
    (*nodes)[parent].right = ri;
    // maximum extent axis of the centroid bound
    float ex = cmx[0] - cmn[0], ey = cmx[1] - cmn[1], ez = cmx[2] - cmn[2];
    int dim = (ex > ey && ex > ez) ? 0 : (ey > ez ? 1 : 2);
    float split = 0.5f * (cmn[dim] + cmx[dim]);
    // stable partition
    int nl = 0;
    for (int p = start; p < end; ++p)
      if (cen[3 * objects[p] + dim] < split) ++nl;
    int mid = start + nl;
    if (mid != start && mid != end) {
      int a = start, b = 0;
      tmp.resize(end - start);
      for (int p = start; p < end; ++p) {
        int t = objects[p];
        if (cen[3 * t + dim] < split) objects[a++] = t; else tmp[b++] = t;
      }
      for (int q = 0; q < b; ++q) objects[mid + q] = tmp[q];
    } else {
      mid = start + (end - start) / 2;
    }
    subdivide(li, start, mid, depth + 1);
    subdivide(ri, mid, end, depth + 1);
  }
};

}  // namespace mto

// ======================================================================
// C entry points (ctypes). Prefix "or_".
// ======================================================================
using namespace mto;

namespace {
template <class R>
Ray<R> ray_from(const RayF& r) {
  Ray<R> o;
  o.o = ld4<R>(r.o);
  o.d = ld4<R>(r.d);
  o.inv_d = ld4<R>(r.inv_d);
  for (int a = 0; a < 3; ++a) o.sign[a] = r.sign[a];
  o.tMin = R(r.tMin);
  o.tMax = R(r.tMax);
  return o;
}
void store_ray(const Ray<float>& r, RayF& o) {
  std::memset(&o, 0, sizeof(o));
  auto st = [](float* d, V4<float> v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w; };
  st(o.o, r.o);
  st(o.d, r.d);
  st(o.inv_d, r.inv_d);
  for (int a = 0; a < 3; ++a) o.sign[a] = r.sign[a];
  o.tMin = r.tMin;
  o.tMax = r.tMax;
}
Mesh mesh_of(const float* points, const float* uvs, const float* normals, const int* faces, int nfaces) {
  return Mesh{points, uvs, normals, reinterpret_cast<const Face*>(faces), nfaces};
}
}  // namespace

extern "C" {

unsigned int or_wanghash(int seed) { return wanghash(seed); }

void or_random(const int* seed, float frame_count, int gid, int n, float* out) {
  Seed s = generate_seed(seed[0], seed[1], frame_count, gid);
  for (int i = 0; i < n; ++i) out[i] = get_random(s);
}

// BVH in the reference layout: nodes int[7]*(2N-1), bounds float[8]*(2N-1). Returns the depth.
int or_bvh_build(const float* points, const int* faces, int nfaces, int* nodes_out, float* bounds_out, int* order_out) {
  std::vector<BVHNode> nodes(2 * (size_t)nfaces - 1);
  std::vector<BoundingBox> bounds(2 * (size_t)nfaces - 1);
  BvhBuilder b;
  b.pts = points;
  b.faces = reinterpret_cast<const Face*>(faces);
  b.n = nfaces;
  b.objects.resize(nfaces);
  for (int i = 0; i < nfaces; ++i) b.objects[i] = i;
  b.cen.resize(3 * (size_t)nfaces);
  b.tb.resize(6 * (size_t)nfaces);
  for (int i = 0; i < nfaces; ++i) b.tri_bound(i);
  b.nodes = &nodes;
  b.bounds = &bounds;
  nodes[0] = BVHNode{};
  b.subdivide(0, 0, nfaces, 0);
  std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(BVHNode));
  std::memcpy(bounds_out, bounds.data(), bounds.size() * sizeof(BoundingBox));
  if (order_out) std::memcpy(order_out, b.objects.data(), sizeof(int) * (size_t)nfaces);
  return b.max_depth;
}

// IntersectPrimitives over `count` rays (AoS reference Ray/Intersection layouts).
// counts: optional [interior visits, triangle tests] per ray (2 longs per ray).
void or_intersect(void* rays, void* isects, int count, int launch, const float* points, const float* uvs,
                  const float* normals, const int* faces, int nfaces, const int* nodes, const float* bounds,
                  long long* counts) {
  Mesh m = mesh_of(points, uvs, normals, faces, nfaces);
  RayF* R_ = static_cast<RayF*>(rays);
  struct alignas(16) IsF { float p[4], n[4], ng[4], d[4], uv[2]; int mat, id, hit, pad; };
  static_assert(sizeof(IsF) == 96, "Intersection layout");
  IsF* I = static_cast<IsF*>(isects);
  for (int i = 0; i < launch; ++i) {
    if (i >= count) { I[i].hit = 0; I[i].mat = -1; continue; }
    Ray<float> r = ray_from<float>(R_[i]);
    int child = -1;
    TraceCounts tc;
    bool hit = intersect_mesh(r, &child, m, reinterpret_cast<const BVHNode*>(nodes),
                              reinterpret_cast<const BoundingBox*>(bounds), false, counts ? &tc : nullptr);
    if (counts) { counts[2 * i] = tc.interior; counts[2 * i + 1] = tc.tris; }
    R_[i].tMax = r.tMax;
    if (hit) {
      Isect<float> is;
      hit_record(r, child, m, is);
      auto st = [](float* d, V4<float> v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w; };
      st(I[i].p, is.p);
      st(I[i].n, is.n);
      st(I[i].ng, is.ng);
      st(I[i].d, is.d);
      I[i].uv[0] = is.uv[0];
      I[i].uv[1] = is.uv[1];
      I[i].mat = is.mat;
      I[i].id = is.id;
      I[i].hit = 1;
    } else {
      I[i].hit = 0;
      I[i].mat = -1;
    }
  }
}

// Closest hit only: t and primitive per ray (-1 on a miss), plus visit counts.
void or_trace_closest(const void* rays, int count, const float* points, const int* faces, int nfaces,
                      const int* nodes, const float* bounds, float* t_out, int* prim_out, long long* counts) {
  Mesh m = mesh_of(points, nullptr, nullptr, faces, nfaces);
  const RayF* R_ = static_cast<const RayF*>(rays);
  for (int i = 0; i < count; ++i) {
    Ray<float> r = ray_from<float>(R_[i]);
    int child = -1;
    TraceCounts tc;
    bool hit = intersect_mesh(r, &child, m, reinterpret_cast<const BVHNode*>(nodes),
                              reinterpret_cast<const BoundingBox*>(bounds), false, &tc);
    t_out[i] = r.tMax;
    prim_out[i] = hit ? child : -1;
    if (counts) { counts[2 * i] = tc.interior; counts[2 * i + 1] = tc.tris; }
  }
}

// testOcclusion per ray (1 = occluded).
void or_occlusion(const void* rays, int* occluded, int count, const float* points, const int* faces, int nfaces,
                  const int* nodes, const float* bounds, long long* counts) {
  Mesh m = mesh_of(points, nullptr, nullptr, faces, nfaces);
  const RayF* R_ = static_cast<const RayF*>(rays);
  for (int i = 0; i < count; ++i) {
    Ray<float> r = ray_from<float>(R_[i]);
    int dummy;
    TraceCounts tc;
    occluded[i] = intersect_mesh(r, &dummy, m, reinterpret_cast<const BVHNode*>(nodes),
                                 reinterpret_cast<const BoundingBox*>(bounds), true, &tc) ? 1 : 0;
    if (counts) { counts[2 * i] = tc.interior; counts[2 * i + 1] = tc.tris; }
  }
}

// InitCameraRayDataJitter; mode 1 keys the seed on pixel ^ 0x9E3779B9 with the raygen stage seeds.
void or_raygen(const void* camera, void* rays, const int* seed, float frame_count, int length, int mode) {
  const CameraF& cam = *static_cast<const CameraF*>(camera);
  RayF* out = static_cast<RayF*>(rays);
  int32_t sx = seed ? seed[0] : 0, sy = seed ? seed[1] : 0;
  if (mode == 1) stage_seed(0, 0, &sx, &sy);
  for (int id = 0; id < length; ++id) {
    Seed s = generate_seed(sx, sy, frame_count, mode == 0 ? id : pixel_gid(id));
    float r0 = get_random(s), r1 = get_random(s);
    Ray<float> r;
    camera_ray<float>(cam, id, r0, r1, r);
    store_ray(r, out[id]);
  }
}

void or_stage_seed(int bounce, int stage, int* out) { stage_seed(bounce, stage, &out[0], &out[1]); }

// Mesh-light list (identifyMeshLights + exclusive scan + prepareLightInfo).
int or_light_list(const int* faces, int nfaces, const float* materials, int* light_faces) {
  const Face* F = reinterpret_cast<const Face*>(faces);
  const SurfaceParameter* M = reinterpret_cast<const SurfaceParameter*>(materials);
  int n = 0;
  for (int i = 0; i < nfaces; ++i)
    if (is_emitter(M + (F[i].mat & 0xFFFF))) light_faces[n++] = i;
  return n;
}

// Serial FP32 inclusive SAT (SAT.cl:113-133, :304-311) and luminance (RGBSpace.cl:28-32).
void or_env_lum_sat(const float* envmap, int w, int h, float* lum, float* sat) {
  for (int i = 0; i < w * h; ++i) {
    const float* c = envmap + 4 * (size_t)i;
    lum[i] = luminance(c[0], c[1], c[2]);
    sat[i] = lum[i];
  }
  for (int y = 0; y < h; ++y) {
    float v = 0;
    for (int x = 0; x < w; ++x) { v = v + sat[(size_t)y * w + x]; sat[(size_t)y * w + x] = v; }
  }
  for (int x = 0; x < w; ++x) {
    float v = 0;
    for (int y = 0; y < h; ++y) { v = v + sat[(size_t)y * w + x]; sat[(size_t)y * w + x] = v; }
  }
}

// FP64 inclusive SAT of the same luminance (the precision the GPU's environment SAT build uses).
void or_env_sat_fp64(const float* lum, int w, int h, double* sat) {
  for (int y = 0; y < h; ++y) {
    double row = 0;
    for (int x = 0; x < w; ++x) {
      row += (double)lum[(size_t)y * w + x];
      sat[(size_t)y * w + x] = row + (y > 0 ? sat[(size_t)(y - 1) * w + x] : 0.0);
    }
  }
}

void or_sat_sample(const float* sat, const float* func, const int* r6, float u0, float u1, float* uv, int* off, float* pdf) {
  SATRegion r{r6[0], r6[1], r6[2], r6[3], r6[4], r6[5]};
  sample_continuous<float>(r, u0, u1, uv, off, pdf, sat, func);
}
void or_sat_sample_discrete(const float* sat, const float* func, const int* r6, float u0, float u1, int* off, float* pdf) {
  SATRegion r{r6[0], r6[1], r6[2], r6[3], r6[4], r6[5]};
  sample_discrete<float>(r, u0, u1, off, pdf, sat, func);
}
float or_sat_pdf(const float* sat, const float* func, const int* r6, int x, int y) {
  SATRegion r{r6[0], r6[1], r6[2], r6[3], r6[4], r6[5]};
  return pdf_sat<float>(r, x, y, sat, func);
}
void or_env_illuminate(const float* envmap, const float* lum, const float* sat, int w, int h, const float* s4,
                       float* dir_out, float* pdf_out, float* contrib_out) {
  Env<float> E;
  E.rgb = envmap;
  E.lum = lum;
  E.sat = sat;
  E.w = w;
  E.h = h;
  E.present = true;
  V4<float> dir{0, 0, 0, 0};
  float dist = 0, pdf = 0;
  V4<float> c = illuminate_env(E, V4<float>{s4[0], s4[1], s4[2], s4[3]}, &dir, &dist, &pdf);
  dir_out[0] = dir.x; dir_out[1] = dir.y; dir_out[2] = dir.z; dir_out[3] = dir.w;
  *pdf_out = pdf;
  contrib_out[0] = c.x; contrib_out[1] = c.y; contrib_out[2] = c.z; contrib_out[3] = c.w;
}
void or_env_radiance(const float* envmap, const float* lum, const float* sat, int w, int h, const float* d4,
                     float* pdf_out, float* contrib_out) {
  Env<float> E;
  E.rgb = envmap;
  E.lum = lum;
  E.sat = sat;
  E.w = w;
  E.h = h;
  E.present = true;
  float pdf = 0;
  V4<float> c = radiance_env(E, V4<float>{d4[0], d4[1], d4[2], d4[3]}, &pdf);
  *pdf_out = pdf;
  contrib_out[0] = c.x; contrib_out[1] = c.y; contrib_out[2] = c.z; contrib_out[3] = c.w;
}

// Light grid per-cell SAT: row then column Kogge-Stone passes (LightGrid.cl:347-400)
// restated as lane loops in the same addition order.
void or_lightgrid_sat(const float* func, float* sat, int nu, int nv, int rx, int ry) {
  size_t n = (size_t)nu * nv;
  std::vector<float> aux(64), old(64);
  for (size_t g = 0; g < n / rx; ++g) {  // prefixSumRowSubgrid: groups of rx consecutive
    for (int l = 0; l < rx; ++l) aux[l] = func[g * rx + l];
    for (int off = 1; off < rx; off *= 2) {
      old.assign(aux.begin(), aux.begin() + rx);
      for (int l = off; l < rx; ++l) aux[l] = old[l - off] + old[l];
    }
    for (int l = 0; l < rx; ++l) sat[g * rx + l] = aux[l];
  }
  for (size_t g = 0; g < n / ry; ++g) {  // prefixSumColSubgrid
    int i = (int)(ry * g);
    int xi = i / nv, y0 = i % nv;
    for (int l = 0; l < ry; ++l) aux[l] = sat[(size_t)xi + (size_t)(y0 + l) * nu];
    for (int off = 1; off < ry; off *= 2) {
      old.assign(aux.begin(), aux.begin() + ry);
      for (int l = off; l < ry; ++l) aux[l] = old[l - off] + old[l];
    }
    for (int l = 0; l < ry; ++l) sat[(size_t)xi + (size_t)(y0 + l) * nu] = aux[l];
  }
}

int or_bsdf_sample(const float* material, const float* n, const float* ng, const float* d, const float* s3,
                   float* dir_out, float* pdf_out, float* cos_out, float* factor_out, float* probs_out) {
  Isect<float> is{};
  is.n = ld4<float>(n);
  is.ng = ld4<float>(ng);
  is.mat = 0;
  Bsdf<float> b = setup_bsdf(ld4<float>(d), is, reinterpret_cast<const SurfaceParameter*>(material));
  if (b.materialID < 0) return 0;
  V4<float> dir{0, 0, 0, 0};
  float pdf = 0, c = 0;
  V4<float> f = sample_bsdf(b, s3[0], s3[1], s3[2], &dir, &pdf, &c);
  dir_out[0] = dir.x; dir_out[1] = dir.y; dir_out[2] = dir.z; dir_out[3] = dir.w;
  *pdf_out = pdf;
  *cos_out = c;
  factor_out[0] = f.x; factor_out[1] = f.y; factor_out[2] = f.z; factor_out[3] = f.w;
  probs_out[0] = b.diffProb;
  probs_out[1] = b.glossyProb;
  return 1;
}
int or_bsdf_eval(const float* material, const float* n, const float* ng, const float* d, const float* wgen,
                 float* pdf_out, float* cos_out, float* factor_out) {
  Isect<float> is{};
  is.n = ld4<float>(n);
  is.ng = ld4<float>(ng);
  is.mat = 0;
  Bsdf<float> b = setup_bsdf(ld4<float>(d), is, reinterpret_cast<const SurfaceParameter*>(material));
  if (b.materialID < 0) return 0;
  float pdf = 0, c = 0;
  V4<float> f = evaluate_bsdf(b, ld4<float>(wgen), &pdf, &c);
  *pdf_out = pdf;
  *cos_out = c;
  factor_out[0] = f.x; factor_out[1] = f.y; factor_out[2] = f.z; factor_out[3] = f.w;
  return 1;
}

int or_render_frame_subset(const void* camera, int width, int height, int max_depth, int mode, int rr_depth,
                           const int* seeds, float frame_count, const float* points, const float* uvs,
                           const float* normals, const int* faces, int nfaces, const float* materials,
                           const int* nodes, const float* bounds, const float* envmap, const void* env_lum,
                           const void* env_sat, int env_w, int env_h, int env_present, int fp64, void* accum,
                           int* counts_out, long long* ray_counts, const float* grid_func, const float* grid_sat,
                           float* grid_accum, int nu, int nv, int rx, int ry, const float* cam_pos, int grid_on,
                           int grid_accumulate, const int* pixels, int npixels);

// One frame. fp64 != 0 runs the FP64 instantiation (accum is then double*).
// env_sat/env_lum: FP32 arrays for fp64 == 0, FP64 arrays otherwise.
// ray_counts: [primary, extension, shadow].
int or_render_frame_grid(const void* camera, int width, int height, int max_depth, int mode, int rr_depth,
                         const int* seeds, float frame_count, const float* points, const float* uvs,
                         const float* normals, const int* faces, int nfaces, const float* materials,
                         const int* nodes, const float* bounds, const float* envmap, const void* env_lum,
                         const void* env_sat, int env_w, int env_h, int env_present, int fp64, void* accum,
                         int* counts_out, long long* ray_counts, const float* grid_func, const float* grid_sat,
                         float* grid_accum, int nu, int nv, int rx, int ry, const float* cam_pos, int grid_on,
                         int grid_accumulate) {
  return or_render_frame_subset(camera, width, height, max_depth, mode, rr_depth, seeds, frame_count, points, uvs,
                                normals, faces, nfaces, materials, nodes, bounds, envmap, env_lum, env_sat, env_w,
                                env_h, env_present, fp64, accum, counts_out, ray_counts, grid_func, grid_sat,
                                grid_accum, nu, nv, rx, ry, cam_pos, grid_on, grid_accumulate, nullptr, 0);
}

// or_render_frame_grid over a subset of the frame's pixels (mode 1 only; see
// RenderParams::pix_of): accum holds one float4 (fp64: double4) per listed pixel.
int or_render_frame_subset(const void* camera, int width, int height, int max_depth, int mode, int rr_depth,
                           const int* seeds, float frame_count, const float* points, const float* uvs,
                           const float* normals, const int* faces, int nfaces, const float* materials,
                           const int* nodes, const float* bounds, const float* envmap, const void* env_lum,
                           const void* env_sat, int env_w, int env_h, int env_present, int fp64, void* accum,
                           int* counts_out, long long* ray_counts, const float* grid_func, const float* grid_sat,
                           float* grid_accum, int nu, int nv, int rx, int ry, const float* cam_pos, int grid_on,
                           int grid_accumulate, const int* pixels, int npixels) {
  if (pixels && mode != 1) return -1;
  Scene S;
  S.mesh = mesh_of(points, uvs, normals, faces, nfaces);
  S.materials = reinterpret_cast<const SurfaceParameter*>(materials);
  S.nodes = reinterpret_cast<const BVHNode*>(nodes);
  S.bounds = reinterpret_cast<const BoundingBox*>(bounds);
  std::vector<int> lf(nfaces > 0 ? nfaces : 1);
  S.nlights = or_light_list(faces, nfaces, materials, lf.data());
  S.light_faces = lf.data();
  RenderParams P{width, height, max_depth, mode, frame_count, rr_depth};
  P.grid_accum = grid_accumulate != 0;
  P.pix_of = pixels;
  P.npix = npixels;
  RayCounts rc;
  const CameraF& cam = *static_cast<const CameraF*>(camera);
  auto set_grid = [&](auto& E) {
    E.grid_on = grid_on != 0 && env_present != 0;
    E.gfunc = grid_func;
    E.gsat = grid_sat;
    E.gaccum = grid_accum;
    E.nu = nu;
    E.nv = nv;
    E.rx = rx;
    E.ry = ry;
    if (cam_pos) for (int i = 0; i < 4; ++i) E.cam[i] = cam_pos[i];
  };
  if (fp64) {
    Env<double> E;
    E.rgb = envmap;
    E.lum = static_cast<const double*>(env_lum);
    E.sat = static_cast<const double*>(env_sat);
    E.w = env_w;
    E.h = env_h;
    E.present = env_present != 0;
    set_grid(E);
    render_frame<double>(S, E, cam, P, seeds, static_cast<double*>(accum), counts_out, &rc);
  } else {
    Env<float> E;
    E.rgb = envmap;
    E.lum = static_cast<const float*>(env_lum);
    E.sat = static_cast<const float*>(env_sat);
    E.w = env_w;
    E.h = env_h;
    E.present = env_present != 0;
    set_grid(E);
    render_frame<float>(S, E, cam, P, seeds, static_cast<float*>(accum), counts_out, &rc);
  }
  if (ray_counts) { ray_counts[0] = rc.primary; ray_counts[1] = rc.extension; ray_counts[2] = rc.shadow; }
  return S.nlights;
}

// Textures for the frames that follow (NULL / 0 entries: none).
void or_set_textures(const int* texels, const int* tex_ref, int nentries) {
  g_tex.texels = texels;
  g_tex.ref = tex_ref;
  g_tex.nref = texels && tex_ref ? nentries : 0;
}

// The texture pass on one material at one uv (material: 144 B in, out).
void or_texture_apply(const float* material, int mat, float u, float v, const int* texels, const int* tex_ref,
                      int nentries, float* material_out) {
  SurfaceParameter p;
  std::memcpy(&p, material, sizeof(p));
  Textures T{texels, tex_ref, nentries};
  apply_textures(T, mat, u, v, p);
  std::memcpy(material_out, &p, sizeof(p));
}

int or_render_frame(const void* camera, int width, int height, int max_depth, int mode, int rr_depth,
                    const int* seeds, float frame_count, const float* points, const float* uvs,
                    const float* normals, const int* faces, int nfaces, const float* materials,
                    const int* nodes, const float* bounds, const float* envmap, const void* env_lum,
                    const void* env_sat, int env_w, int env_h, int env_present, int fp64, void* accum,
                    int* counts_out, long long* ray_counts) {
  return or_render_frame_grid(camera, width, height, max_depth, mode, rr_depth, seeds, frame_count, points, uvs,
                              normals, faces, nfaces, materials, nodes, bounds, envmap, env_lum, env_sat, env_w,
                              env_h, env_present, fp64, accum, counts_out, ray_counts, nullptr, nullptr, nullptr, 0,
                              0, 0, 0, nullptr, 0, 0);
}

// The preview device's frame (CDeviceRT.loop, src/cl/device/CDeviceRT.java:176-197,
// kernels of Raytrace.cl): unjittered camera rays, closest hit, quick surface
// colour (getQuickSurfaceColor, Material.cl:33-43: emission, or diffuse colour x
// the cosine localDirFix.z) or the environment texel with gamma 2.2
// (backgroundShade), packed as ARGB; group = the hit's material index, -1 on a
// miss (updateGroupbufferShadeImage). A hit whose BSDF is invalid is shaded with
// its material's parameters (the reference reads an unset parameter block; the
// cosine below 1e-6 makes the colour black either way).
void or_preview(const void* camera, int width, int height, const float* points, const float* uvs,
                const float* normals, const int* faces, int nfaces, const float* materials, const int* nodes,
                const float* bounds, const float* envmap, int ew, int eh, int env_present, int* argb, int* group) {
  CameraF cam = *static_cast<const CameraF*>(camera);
  cam.dimension[0] = (float)width;
  cam.dimension[1] = (float)height;
  Mesh m = mesh_of(points, uvs, normals, faces, nfaces);
  const SurfaceParameter* mats = reinterpret_cast<const SurfaceParameter*>(materials);
  auto pack = [](float r, float g, float b, float a) {
    auto q = [](float v) { return (int)(std::fmin(std::fmax(v, 0.f), 1.f) * 255.0f); };
    return (q(a) << 24) | (q(r) << 16) | (q(g) << 8) | q(b);
  };
  for (int id = 0; id < width * height; ++id) {
    Ray<float> r;
    camera_ray(cam, id, 0.5f, 0.5f, r);
    int child = -1;
    bool hit = intersect_mesh(r, &child, m, reinterpret_cast<const BVHNode*>(nodes),
                              reinterpret_cast<const BoundingBox*>(bounds), false, nullptr);
    if (hit) {
      Isect<float> is;
      hit_record(r, child, m, is);
      Bsdf<float> b = setup_bsdf(r.d, is, mats);
      const float coeff = b.localDirFix.z;
      SurfaceParameter tp = mats[is.mat];
      // textureInitPassRT, CTextureApplyPass.process, updateToTextureColorRT
      // (Raytrace.cl:52-145, CDeviceRT.java:179-182): the texture pass of the
      // frames that follow or_set_textures
      if (g_tex.nref > 0 && !is_emitter(&tp)) apply_textures(g_tex, is.mat, is.uv[0], is.uv[1], tp);
      const SurfaceParameter* p = &tp;
      V4<float> c;
      if (is_emitter(p)) c = col<float>(p->emission_color);
      else c = col<float>(p->diffuse_color) * coeff;
      argb[id] = pack(c.x, c.y, c.z, 1.f);
      group[id] = is.mat;
    } else {
      if (env_present) {
        int idx = spherical_index(ew, eh, r.d);
        const float* e = envmap + 4 * (size_t)idx;
        const float ig = 1.f / 2.2f;
        argb[id] = pack(std::pow(e[0], ig), std::pow(e[1], ig), std::pow(e[2], ig), e[3]);
      } else {
        argb[id] = pack(0.f, 0.f, 0.f, 1.f);
      }
      group[id] = -1;
    }
  }
}

// Grid-guided environment sample (illuminate_env_grid) and pdf/radiance
// (radiance_env_grid) for one shading point, FP32. pdf_ref_out: the pdf the
// reference's illuminateEnvironmentLight1 returns (pdfSS / (2 pi^2 sin), no
// tile probability); gidx_out: the grid entry of (cell, tile).
void or_env_grid_illuminate(const float* envmap, const float* lum, const float* sat, int w, int h,
                            const float* gfunc, const float* gsat, int nu, int nv, int rx, int ry, const float* cam4,
                            const float* p4, const float* s4, float* dir_out, float* pdf_out, float* pdf_ref_out,
                            float* contrib_out, int* gidx_out) {
  Env<float> E;
  E.rgb = envmap; E.lum = lum; E.sat = sat; E.w = w; E.h = h; E.present = true;
  E.grid_on = true; E.gfunc = gfunc; E.gsat = gsat; E.nu = nu; E.nv = nv; E.rx = rx; E.ry = ry;
  for (int i = 0; i < 4; ++i) E.cam[i] = cam4[i];
  V4<float> p{p4[0], p4[1], p4[2], p4[3]}, s{s4[0], s4[1], s4[2], s4[3]};
  V4<float> dir{0, 0, 0, 0};
  float dist = 0, pdf = 0;
  V4<float> c = illuminate_env_grid(E, p, s, &dir, &dist, &pdf);
  const size_t base = grid_cell_base(E, grid_cell(E, p));
  const SATRegion rc = grid_cell_region(E);
  float uvLL[2], pdfLL[1];
  int offLL[2];
  sample_continuous<float>(rc, s.x, s.y, uvLL, offLL, pdfLL, gsat + base, gfunc + base);
  *gidx_out = (int)(base + (size_t)offLL[1] * nu + offLL[0]);
  *pdf_ref_out = 0.f;
  if (pdfLL[0] > 0.f) {
    const SATRegion rt = env_tile_region(E, offLL[0], offLL[1]);
    float uv[2], pdfSS[1];
    int off[2];
    sample_continuous<float>(rt, s.z, s.w, uv, off, pdfSS, sat, lum);
    *pdf_ref_out = pdfSS[0] / (2.f * PI_<float>() * PI_<float>() * sin_(uv[1] * PI_<float>()));
  }
  std::memcpy(dir_out, &dir, 16);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
}

void or_env_grid_radiance(const float* envmap, const float* lum, const float* sat, int w, int h, const float* gfunc,
                          const float* gsat, int nu, int nv, int rx, int ry, const float* cam4, const float* p4,
                          const float* d4, float* pdf_out, float* contrib_out, int* gidx_out, float* accum_out) {
  Env<float> E;
  E.rgb = envmap; E.lum = lum; E.sat = sat; E.w = w; E.h = h; E.present = true;
  E.grid_on = true; E.gfunc = gfunc; E.gsat = gsat; E.nu = nu; E.nv = nv; E.rx = rx; E.ry = ry;
  for (int i = 0; i < 4; ++i) E.cam[i] = cam4[i];
  std::vector<float> acc((size_t)nu * nv, 0.f);
  E.gaccum = acc.data();
  V4<float> p{p4[0], p4[1], p4[2], p4[3]}, d{d4[0], d4[1], d4[2], d4[3]};
  float pdf = 0;
  V4<float> c = radiance_env_grid(E, p, d, &pdf, true);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
  *gidx_out = -1;
  *accum_out = 0.f;
  for (size_t i = 0; i < acc.size(); ++i)
    if (acc[i] != 0.f) {
      *gidx_out = (int)i;
      *accum_out = acc[i];
    }
}

// CImage.processImage (CImage.java:124-136, Image.cl:29-118, RGBSpace.cl:9-106):
// averageAccum -> log-average luminance over pixels with Lw > 0 of
// log(0.01 + Lw) -> Reinhard on the exposure-scaled luminance, applied through
// xyY -> gamma -> ARGB. Pixels with Lw <= 0 keep their ARGB value. The total
// is an FP64 sum rounded to FP32 (the reference sums with its float prefix
// scan, whose lane-0 read of aux[-1] and int truncation in GET_FLOAT make the
// total ill-defined) and is recomputed on every call (the reference keeps the
// total of its first two frames). totals_out: {total log luminance, count}.
void or_tonemap_with_total(const float* accum, int n, float frame_count, float exposure, float gamma,
                           const float* totals_in, int* argb, float* framebuf_out, float* totals_out);

void or_tonemap(const float* accum, int n, float frame_count, float exposure, float gamma, int* argb,
                float* framebuf_out, float* totals_out) {
  or_tonemap_with_total(accum, n, frame_count, exposure, gamma, nullptr, argb, framebuf_out, totals_out);
}

// The same with the log-luminance total and count given (totals_in = {total,
// count}), as updateFrameImage receives them from its scans; NULL computes them.
void or_tonemap_with_total(const float* accum, int n, float frame_count, float exposure, float gamma,
                           const float* totals_in, int* argb, float* framebuf_out, float* totals_out) {
  std::vector<float> fb(4 * (size_t)(n > 0 ? n : 1));
  double tot = 0.0;
  int cnt = 0;
  for (int i = 0; i < n; ++i) {
    const float* a = accum + 4 * (size_t)i;
    float* f = fb.data() + 4 * (size_t)i;
    f[0] = a[0] / frame_count;
    f[1] = a[1] / frame_count;
    f[2] = a[2] / frame_count;
    f[3] = 1.f;
    float Lw = luminance(f[0], f[1], f[2]);
    if (Lw > 0.f) {
      tot += (double)std::log(0.01f + Lw);
      ++cnt;
    }
  }
  float total = (float)tot;
  if (totals_in) {
    total = totals_in[0];
    cnt = (int)totals_in[1];
  }
  if (totals_out) {
    totals_out[0] = total;
    totals_out[1] = (float)cnt;
  }
  float logavg = total / (float)cnt;
  logavg = std::exp(logavg);
  const float ig = 1.f / gamma;
  for (int i = 0; i < n; ++i) {
    float* c = fb.data() + 4 * (size_t)i;
    float L = luminance(c[0], c[1], c[2]);
    if (L > 0.f) {
      float scaled = exposure * L / logavg;
      float Y = scaled / (1.f + scaled);  // toneSimpleReinhard
      if (std::isinf(Y) || std::isnan(Y) || Y < 0.000001f) Y = 0.f;  // check, Util.cl:381-387
      float X_ = 0.5893f * c[0] + 0.1789f * c[1] + 0.1831f * c[2];
      float Y_ = 0.2904f * c[0] + 0.6051f * c[1] + 0.1045f * c[2];
      float Z_ = 0.0000f * c[0] + 0.0684f * c[1] + 1.0202f * c[2];
      float x = 0.f, y = 0.f;
      float XYZ = X_ + Y_ + Z_;
      if (!(XYZ < 1e-6f)) {
        float s = 1.f / XYZ;
        x = X_ * s;
        y = Y_ * s;
      }
      float X = y < 1e-6f ? 0.f : Y * (x / y);
      float Z = y < 1e-6f ? 0.f : (Y * (1 - x - y)) / y;
      c[0] = 1.967f * X - 0.548f * Y - 0.297f * Z;
      c[1] = -0.955f * X + 1.938f * Y - 0.027f * Z;
      c[2] = 0.064f * X - 0.130f * Y + 0.982f * Z;
      c[3] = 1.f;
      c[0] = std::pow(c[0], ig);
      c[1] = std::pow(c[1], ig);
      c[2] = std::pow(c[2], ig);
      auto q = [](float v) { return (int)(std::fmin(std::fmax(v, 0.f), 1.f) * 255.0f); };
      argb[i] = (q(c[3]) << 24) | (q(c[0]) << 16) | (q(c[1]) << 8) | q(c[2]);
    }
  }
  if (framebuf_out) std::memcpy(framebuf_out, fb.data(), 16 * (size_t)n);
}

// Initial light-grid func: each cell's tile (tx, ty) holds the map's luminance
// summed over the tile's region, from the FP64 SAT when given, else from the
// FP32 SAT in SAT.cl:149-156's order. The reference fills it from a luminance
// histogram of 500 samples per tile (CAdaptiveEnvironment.java:77, an
// un-vendored library routine); the tile sum is that histogram's expectation.
void or_grid_init_func(const double* sat64, const float* sat32, int w, int h, int nu, int nv, int rx, int ry,
                       float* func) {
  for (int gy = 0; gy < nv; ++gy)
    for (int gx = 0; gx < nu; ++gx) {
      const int tx = gx % rx, ty = gy % ry;
      const int x0 = (int)((float)w * ((float)tx / (float)rx)), y0 = (int)((float)h * ((float)ty / (float)ry));
      const int x1 = (int)((float)w * ((float)(tx + 1) / (float)rx)) - 1;
      const int y1 = (int)((float)h * ((float)(ty + 1) / (float)ry)) - 1;
      float v;
      if (sat64) {
        auto at = [&](int x, int y) { return (x < 0 || y < 0) ? 0.0 : sat64[(size_t)y * w + x]; };
        v = (float)(at(x1, y1) - at(x0 - 1, y1) - at(x1, y0 - 1) + at(x0 - 1, y0 - 1));
      } else {
        auto at = [&](int x, int y) { return (x < 0 || y < 0) ? 0.f : sat32[(size_t)y * w + x]; };
        v = at(x0 - 1, y0 - 1) + at(x1, y1) - at(x1, y0 - 1) - at(x0 - 1, y1);
      }
      func[(size_t)gy * nu + gx] = v;
    }
}

}  // extern "C"
