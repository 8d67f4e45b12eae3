// Device-side arithmetic of the GI path (FP32). Each function keeps the
// reference kernel's operation order so that, with FMA contraction off
// (-fmad=false) and IEEE division/sqrt, results match the reference kernels
// bit for bit on identical inputs; transcendentals are CUDA's (the reference's
// are the OpenCL device's). Citations: mambastudio/MambaTracer file:line.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "mt_common.h"

namespace mt {
namespace dv {

typedef float4 V;

__device__ __forceinline__ V mk(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
__device__ __forceinline__ V add(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ V sub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ V mul(V a, V b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ V muls(V a, float s) { return mk(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ V smul(float s, V a) { return mk(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ V divs(V a, float s) { return mk(a.x / s, a.y / s, a.z / s, a.w / s); }
__device__ __forceinline__ V neg(V a) { return mk(-a.x, -a.y, -a.z, -a.w); }
__device__ __forceinline__ V xyz0(V a) { return mk(a.x, a.y, a.z, 0.0f); }
__device__ __forceinline__ V zero4() { return mk(0.f, 0.f, 0.f, 0.f); }

// dot/cross/normalize with the lane order of the reference oracle
__device__ __forceinline__ float dot4(V a, V b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
__device__ __forceinline__ float dot3(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V cross4(V a, V b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
__device__ __forceinline__ V normalize4(V v) { float l = sqrtf(dot4(v, v)); return divs(v, l); }
__device__ __forceinline__ V normalize3(V v) {
  float l = sqrtf(dot3(v, v));
  return mk(v.x / l, v.y / l, v.z / l, 0.0f);
}
__device__ __forceinline__ float minf_(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float maxf_(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float clampf_(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ bool zero3(V v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
__device__ __forceinline__ bool zero4(V v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f && v.w == 0.f; }
// Util.cl:537-549
__device__ __forceinline__ bool abs_valid4(V v) {
  float a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (isnan(a[i]) || isinf(a[i]) || a[i] < 0.f) return false;
  return true;
}

constexpr float kPi = 3.14159265359f;       // Util.cl:7
constexpr float kEpsCos = 1e-6f;            // Util.cl:5
constexpr float kFloatMax = 3.402823e+38f;  // Util.cl:1

// ------------------------------------------------------------------ RNG
// Sampling.cl:15-23
__device__ __forceinline__ uint32_t wanghash(int32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed = (int32_t)((uint32_t)seed * 9u);
  seed = seed ^ (seed >> 4);
  seed = (int32_t)((uint32_t)seed * 0x27d4eb2du);
  seed = seed ^ (seed >> 15);
  return (uint32_t)seed;
}
struct Seed { int32_t x, y; };
// Sampling.cl:32-40
__device__ __forceinline__ Seed gen_seed(int32_t sx, int32_t sy, float frame_count, int32_t gid) {
  uint32_t fc = (uint32_t)(int32_t)frame_count;
  Seed s;
  s.x = (int32_t)((uint32_t)gid + fc * (uint32_t)sx);
  s.y = (int32_t)((uint32_t)gid + fc * (uint32_t)sy);
  return s;
}
// Sampling.cl:43-59
__device__ __forceinline__ float rnd(Seed& s) {
  s.x = (int32_t)wanghash(s.x);
  s.y = (int32_t)wanghash(s.y);
  uint32_t ires = ((uint32_t)s.x << 16) + (uint32_t)s.y;
  uint32_t bits = (ires & 0x007fffffu) | 0x40000000u;
  return (__uint_as_float(bits) - 2.0f) / 2.0f;
}
// Benchmark-mode seed pair of a (bounce, stage); pixel key pixel ^ 0x9E3779B9.
__host__ __device__ __forceinline__ uint32_t wanghash_hd(int32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed = (int32_t)((uint32_t)seed * 9u);
  seed = seed ^ (seed >> 4);
  seed = (int32_t)((uint32_t)seed * 0x27d4eb2du);
  seed = seed ^ (seed >> 15);
  return (uint32_t)seed;
}
__host__ __device__ __forceinline__ void stage_seed(int bounce, int stage, int32_t* sx, int32_t* sy) {
  *sx = (int32_t)(wanghash_hd((int32_t)(0x5EED0000u + 16u * (uint32_t)bounce + 2u * (uint32_t)stage)) | 1u);
  *sy = (int32_t)(wanghash_hd((int32_t)(0x5EED8000u + 16u * (uint32_t)bounce + 2u * (uint32_t)stage)) | 1u);
}
__device__ __forceinline__ int32_t pixel_gid(int pixel) { return (int32_t)((uint32_t)pixel ^ 0x9E3779B9u); }

// ---------------------------------------------------------------- frame
struct Frame { V mX, mY, mZ; };
// Util.cl:196-211
__device__ __forceinline__ Frame get_frame(V n) {
  Frame f;
  f.mZ = n;
  float a = 1.0f / (1.0f + n.z);
  float b = -n.x * n.y * a;
  f.mX = mk(1.0f - n.x * n.x * a, b, -n.x, 0.0f);
  f.mY = mk(b, 1.0f - n.y * n.y * a, -n.y, 0.0f);
  if (n.z < -0.9999999f) {
    f.mX = mk(0.f, -1.f, 0.f, 0.f);
    f.mY = mk(-1.f, 0.f, 0.f, 0.f);
  }
  return f;
}
// Util.cl:213-221
__device__ __forceinline__ V world_coord(const Frame& f, V a) { return add(add(muls(f.mX, a.x), muls(f.mY, a.y)), muls(f.mZ, a.z)); }
__device__ __forceinline__ V local_coord(const Frame& f, V a) { return mk(dot4(f.mX, a), dot4(f.mY, a), dot4(f.mZ, a), 0.0f); }

// RGBSpace.cl:28-32
__device__ __forceinline__ float luminance(float x, float y, float z) { return (0.2989f * x + 0.5866f * y) + 0.1145f * z; }

// ------------------------------------------------------------ hit record
struct Hit {
  V p, n, ng;
  float u, v;
  int mat;
};
__device__ __forceinline__ V ldg4(const float4* p) { return __ldg(p); }

// NormalBVH.cl:124-221 with Primitive.cl:31-71 (ray direction d, hit distance t)
__device__ __forceinline__ void hit_record(const DevScene& S, V o, V d, float t, int id, Hit& h) {
  Face f;
  const int* fp = reinterpret_cast<const int*>(S.faces + id);
  f.vx = __ldg(fp + 0); f.vy = __ldg(fp + 1); f.vz = __ldg(fp + 2);
  f.uvx = __ldg(fp + 3); f.uvy = __ldg(fp + 4); f.uvz = __ldg(fp + 5);
  f.nx = __ldg(fp + 6); f.ny = __ldg(fp + 7); f.nz = __ldg(fp + 8); f.mat = __ldg(fp + 9);
  V p1 = ldg4(S.points + f.vx), p2 = ldg4(S.points + f.vy), p3 = ldg4(S.points + f.vz);
  V p = mk(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z, 0.0f);
  bool hasTex = f.uvx > -1;
  float tu = 0.f, tv = 0.f;
  if (hasTex) {
    V f1 = xyz0(sub(p1, p)), f2 = xyz0(sub(p2, p)), f3 = xyz0(sub(p3, p));
    V c0 = cross4(xyz0(sub(p1, p2)), xyz0(sub(p1, p3)));
    float a = sqrtf(dot3(c0, c0));
    V c1 = cross4(f2, f3), c2 = cross4(f3, f1), c3 = cross4(f1, f2);
    float a1 = sqrtf(dot3(c1, c1)) / a, a2 = sqrtf(dot3(c2, c2)) / a, a3 = sqrtf(dot3(c3, c3)) / a;
    float2 u1 = __ldg(S.uvs + f.uvx), u2 = __ldg(S.uvs + f.uvy), u3 = __ldg(S.uvs + f.uvz);
    tu = (u1.x * a1 + u2.x * a2) + u3.x * a3;
    tv = (u1.y * a1 + u2.y * a2) + u3.y * a3;
  }
  float u = 0.f, v = 0.f;
  {
    V e1 = xyz0(sub(p2, p1)), e2 = xyz0(sub(p3, p1)), e = xyz0(sub(p, p1));
    float d00 = dot3(e1, e1), d01 = dot3(e1, e2), d11 = dot3(e2, e2), d20 = dot3(e, e1), d21 = dot3(e, e2);
    float denom = d00 * d11 - d01 * d01;
    if (!(denom == 0.f)) {
      float inv = 1.f / denom;
      u = (d11 * d20 - d01 * d21) * inv;
      v = (d00 * d21 - d01 * d20) * inv;
    }
  }
  V n;
  if (f.nx > -1) {
    V n1 = ldg4(S.normals + f.nx), n2 = ldg4(S.normals + f.ny), n3 = ldg4(S.normals + f.nz);
    float s = (1.f - u) - v;
    n = add(add(muls(n1, s), muls(n2, u)), muls(n3, v));
    if (dot4(n, d) > 0.00001f) {
      n = neg(n);
      n1 = neg(n1);
      n2 = neg(n2);
      n3 = neg(n3);
    }
    n = normalize4(n);
    V q1 = xyz0(sub(p, p1)), q2 = xyz0(sub(p, p2)), q3 = xyz0(sub(p, p3));
    V m1 = normalize3(n1), m2 = normalize3(n2), m3 = normalize3(n3);
    float du = minf_(0.f, dot3(q1, m1)), dv_ = minf_(0.f, dot3(q2, m2)), dw = minf_(0.f, dot3(q3, m3));
    q1 = sub(q1, xyz0(smul(du, m1)));
    q2 = sub(q2, xyz0(smul(dv_, m2)));
    q3 = sub(q3, xyz0(smul(dw, m3)));
    p = add(add(add(p, smul(s, q1)), smul(u, q2)), smul(v, q3));
  } else {
    n = normalize4(cross4(sub(p2, p1), sub(p3, p1)));
    if (dot4(n, d) > 0.00001f) n = neg(n);
  }
  V ng = normalize4(cross4(sub(p2, p1), sub(p3, p1)));
  if (dot4(ng, d) > 0.00001f) ng = neg(ng);
  h.p = p;
  h.n = n;
  h.ng = ng;
  h.u = hasTex ? tu : u;
  h.v = hasTex ? tv : v;
  h.mat = f.mat & 0xFFFF;
}

// ------------------------------------------------------------------ BSDF
struct Bsdf {
  Frame frame;
  V fix;          // localDirFix
  int mat;        // -1 = invalid
  float pd, pg;   // diffuse / glossy probabilities
  const Material* pm;  // parameters (the scene's material, or a path's copy of it)
};
__device__ __forceinline__ const Material& matl(const DevScene& S, int m) { return S.materials[m]; }

// Bsdf.cl:70-160
__device__ __forceinline__ Bsdf setup_bsdf(const DevScene& S, V d, V n, int mat) {
  Bsdf b;
  b.frame = get_frame(n);
  b.fix = local_coord(b.frame, neg(d));
  b.pd = b.pg = 0.f;
  if (fabsf(b.fix.z) < kEpsCos) {
    b.mat = -1;
    return b;
  }
  b.mat = mat;
  b.pm = S.materials + mat;
  const Material& M = *b.pm;
  V cd = muls(M.diffuse_color, M.diffuse_param.x);
  V cg = muls(M.glossy_color, M.glossy_param.x);
  float ad = luminance(cd.x, cd.y, cd.z), ag = luminance(cg.x, cg.y, cg.z);
  float total = ad + ag;
  if (total < 1e-9f) {
    b.pd = 0.f;
    b.pg = 0.f;
  } else {
    b.pd = ad / total;
    b.pg = ag / total;
  }
  return b;
}
// ------------------------------------------------------------- textures
// Java's float -> int cast: NaN -> 0, saturating at the int range.
__device__ __forceinline__ int java_f2i(float x) {
  if (x != x) return 0;
  if (x >= 2147483648.f) return 0x7FFFFFFF;
  if (x <= -2147483648.f) return (int)0x80000000;
  return (int)x;
}
// TextureInfoCache.getDomainValue (TextureInfoCache.java:131-136)
__device__ __forceinline__ float tex_domain(float x) {
  return x < 0.f ? (x - (float)java_f2i(x)) + 1.f : x - (float)java_f2i(x);
}
// CTextureApplyPass.process (CTextureApplyPass.java:37-92): the texel at
// ((int)(u' (W - 1)), (int)(v' (H - 1))) of a W x H ARGB image; the index is
// clamped to the image (Java's PixelReader throws beyond it, which only
// infinite or |uv| >= 2^31 coordinates reach).
__device__ __forceinline__ int tex_fetch(const int* __restrict__ texels, int4 ref, float u, float v) {
  const float dx = tex_domain(u) * ((float)ref.y - 1.f);
  const float dy = tex_domain(v) * ((float)ref.z - 1.f);
  const int x = min(max(java_f2i(dx), 0), ref.y - 1), y = min(max(java_f2i(dy), 0), ref.z - 1);
  return __ldg(texels + ref.x + (long long)y * ref.y + x);
}
// getFloat4ARGB (Util.cl:482-493)
__device__ __forceinline__ float4 argb_float4(int c) {
  return make_float4(((c >> 16) & 0xFF) / 255.0f, ((c >> 8) & 0xFF) / 255.0f, (c & 0xFF) / 255.0f,
                     ((c >> 24) & 0xFF) / 255.0f);
}
__device__ __forceinline__ bool has_textures(const Material& M) {
  return M.isDiffuseTexture || M.isGlossyTexture || M.isRoughnessTexture;
}
// texturePassGI + CTextureApplyPass.process + updateToTextureColorGI
// (Render.cl:127-231): a path's copy of its material takes the texel colours at
// the hit's uv (diffuse and glossy colour; roughness from red and green). A
// flagged texture without an image reads ARGB 0. The component probabilities
// stay those of the untextured material, as SetupBSDFPath computed them first.
__device__ __forceinline__ void apply_textures(const DevScene& S, int mat, float u, float v, Material& m) {
  const int4* r = S.tex_ref + 4 * (size_t)mat;
  if (m.isDiffuseTexture) {
    const int4 t = __ldg(r + 0);
    m.diffuse_color = argb_float4(t.y > 0 ? tex_fetch(S.texels, t, u, v) : 0);
  }
  if (m.isGlossyTexture) {
    const int4 t = __ldg(r + 1);
    m.glossy_color = argb_float4(t.y > 0 ? tex_fetch(S.texels, t, u, v) : 0);
  }
  if (m.isRoughnessTexture) {
    const int4 t = __ldg(r + 2);
    const float4 c = argb_float4(t.y > 0 ? tex_fetch(S.texels, t, u, v) : 0);
    m.glossy_param.y = fmaxf(0.001f, c.x);
    m.glossy_param.z = fmaxf(0.001f, c.y);
  }
}

// Bsdf.cl:162-166
__device__ __forceinline__ bool is_emitter(const Material& M) {
  V c = muls(M.emission_color, M.emission_param.x);
  return luminance(c.x, c.y, c.z) != 0.f;
}

// Geometry.cl:1-56
__device__ __forceinline__ float cos2t(V w) { return w.z * w.z; }
__device__ __forceinline__ float sin2t(V w) { return fmaxf(0.f, 1.f - cos2t(w)); }
__device__ __forceinline__ float sint(V w) { return sqrtf(sin2t(w)); }
__device__ __forceinline__ float tant(V w) { return sint(w) / w.z; }
__device__ __forceinline__ float tan2t(V w) { return sin2t(w) / cos2t(w); }
__device__ __forceinline__ float cosp(V w) { float st = sint(w); return st == 0.f ? 1.f : clampf_(w.x / st, -1.f, 1.f); }
__device__ __forceinline__ float sinp(V w) { float st = sint(w); return st == 0.f ? 0.f : clampf_(w.y / st, -1.f, 1.f); }
__device__ __forceinline__ float cos2p(V w) { return cosp(w) * cosp(w); }
__device__ __forceinline__ float sin2p(V w) { return sinp(w) * sinp(w); }

// Bsdf.cl:229-264
__device__ __forceinline__ float alpha_(V w, float ax, float ay) { return sqrtf(cos2p(w) * ax * ax + sin2p(w) * ay * ay); }
__device__ __forceinline__ float lambda_(V w, float ax, float ay) {
  float at = fabsf(tant(w));
  float a = alpha_(w, ax, ay);
  float a2t = (a * at) * (a * at);
  float lam = (-1.f + sqrtf(1.f + a2t)) / 2.f;
  return isinf(at) ? 0.f : lam;
}
__device__ __forceinline__ float D_H(V wh, float ax, float ay) {
  float t2 = tan2t(wh);
  float c4 = cos2t(wh) * cos2t(wh);
  float e = (cos2p(wh) / (ax * ax) + sin2p(wh) / (ay * ay)) * t2;
  float d = 1.f / (kPi * ax * ay * c4 * (1.f + e) * (1.f + e));
  return isinf(t2) ? 0.f : d;
}
__device__ __forceinline__ float G_Atten(V w1, V w2, float ax, float ay) { return 1.f / (1.f + lambda_(w1, ax, ay) + lambda_(w2, ax, ay)); }
__device__ __forceinline__ float G1_(V w, float ax, float ay) { return 1.f / (1.f + lambda_(w, ax, ay)); }
// Bsdf.cl:270-294
__device__ __forceinline__ V sample_vndf(V v, float ax, float ay, float r1, float r2) {
  V Vh = normalize4(mk(ax * v.x, ay * v.y, v.z, 0.f));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  V T1 = mk(1.f, 0.f, 0.f, 0.f);
  if (lensq > 0.f) {
    float rs = 1.f / sqrtf(lensq);
    T1 = muls(mk(-Vh.y, Vh.x, 0.f, 0.f), rs);
  }
  V T2 = cross4(Vh, T1);
  float r = sqrtf(r1);
  float phi = 2.0f * kPi * r2;
  float t1 = r * cosf(phi);
  float t2 = r * sinf(phi);
  float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
  V Nh = add(add(smul(t1, T1), smul(t2, T2)), smul(sqrtf(maxf_(0.f, 1.f - t1 * t1 - t2 * t2)), Vh));
  return normalize4(mk(ax * Nh.x, ay * Nh.y, maxf_(0.f, Nh.z), 0.f));
}
// Bsdf.cl:297-311
__device__ __forceinline__ float pdf_vndf(V v, V ni, float ax, float ay) {
  float Dv = G1_(v, ax, ay) * maxf_(0.001f, dot4(v, ni)) * D_H(ni, ax, ay) / maxf_(0.001f, v.z);
  float VN = dot4(v, ni);
  return Dv / (4.f * VN);
}
// Bsdf.cl:185-189
__device__ __forceinline__ V schlick3(float c, V f0) {
  float ex = powf(1.f - c, 5.0f);
  return mk(f0.x + (1.f - f0.x) * ex, f0.y + (1.f - f0.y) * ex, f0.z + (1.f - f0.z) * ex, 0.f);
}
// Bsdf.cl:380-394 with Sampling.cl:129-148
__device__ __forceinline__ V sample_diffuse(const DevScene& S, const Bsdf& b, float sx, float sy, V* gen, float* pdfW) {
  if (b.fix.z < kEpsCos) return zero4();
  float term1 = 2.f * kPi * sx;
  float term2 = sqrtf(1.f - sy);
  V ret = mk(cosf(term1) * term2, sinf(term1) * term2, sqrtf(sy), 0.f);
  float un = ret.z * 1.f / kPi;
  *gen = ret;
  *pdfW += un * b.pd;
  V c = b.pm->diffuse_color;
  return mk(c.x * 1.f / kPi, c.y * 1.f / kPi, c.z * 1.f / kPi, 1.f);
}
// Bsdf.cl:396-432
__device__ __forceinline__ V sample_glossy(const DevScene& S, const Bsdf& b, float sx, float sy, V* gen, float* pdfW) {
  if (b.fix.z < kEpsCos) return zero4();
  const Material& M = *b.pm;
  float ax = M.glossy_param.y, ay = M.glossy_param.z;
  V wh = sample_vndf(b.fix, ax, ay, sx, sy);
  V wo = add(neg(b.fix), smul(2.f * dot4(b.fix, wh), wh));
  *gen = wo;
  float cI = fabsf(b.fix.z), cO = fabsf(wo.z);
  *pdfW += b.pg * pdf_vndf(wo, wh, ax, ay);
  float fr = G_Atten(b.fix, wo, ax, ay) * D_H(wh, ax, ay) / (4.f * cI * cO);
  float whdot = fabsf(dot4(wh, wo));
  V Fc = schlick3(whdot, M.glossy_color);
  if (cI == 0.f || cO == 0.f) Fc = zero4();
  if (wh.x == 0.f && wh.y == 0.f && wh.z == 0.f) Fc = zero4();
  return mk(Fc.x * fr, Fc.y * fr, Fc.z * fr, 0.f);
}
// Bsdf.cl:452-467
__device__ __forceinline__ V eval_diffuse(const DevScene& S, const Bsdf& b, V gen, float* pdfW) {
  if (b.pd == 0.f) return zero4();
  if (b.fix.z < kEpsCos || gen.z < kEpsCos) return zero4();
  *pdfW += b.pd * fmaxf(0.f, gen.z * 1.f / kPi);
  V c = b.pm->diffuse_color;
  return mk(c.x * 1.f / kPi, c.y * 1.f / kPi, c.z * 1.f / kPi, 1.f);
}
// Bsdf.cl:469-507
__device__ __forceinline__ V eval_glossy(const DevScene& S, const Bsdf& b, V gen, float* pdfW) {
  if (b.pg == 0.f) return zero4();
  if (b.fix.z < kEpsCos || gen.z < kEpsCos) return zero4();
  const Material& M = *b.pm;
  float ax = M.glossy_param.y, ay = M.glossy_param.z;
  V wh = normalize4(add(b.fix, gen));
  float cI = fabsf(b.fix.z), cO = fabsf(gen.z);
  *pdfW += b.pg * pdf_vndf(gen, wh, ax, ay);
  float fr = G_Atten(b.fix, gen, ax, ay) * D_H(wh, ax, ay) / (4.f * cI * cO);
  float whdot = fabsf(dot4(wh, gen));
  V Fc = schlick3(whdot, M.glossy_color);
  if (cI == 0.f || cO == 0.f) Fc = zero4();
  if (wh.x == 0.f && wh.y == 0.f && wh.z == 0.f) Fc = zero4();
  return mk(Fc.x * fr, Fc.y * fr, Fc.z * fr, 0.f);
}
// Bsdf.cl:525-545
__device__ __forceinline__ V eval_bsdf(const DevScene& S, const Bsdf& b, V world, float* pdfW, float* cosGen) {
  V result = mk(0.f, 0.f, 0.f, 1.f);
  V gen = local_coord(b.frame, world);
  if (gen.z * b.fix.z < 0.f) return result;
  *cosGen = gen.z;
  result = add(result, eval_diffuse(S, b, gen, pdfW));
  result = add(result, eval_glossy(S, b, gen, pdfW));
  return result;
}
// Bsdf.cl:555-606 (worldGen is left untouched when the sample is rejected)
__device__ __forceinline__ V sample_bsdf(const DevScene& S, const Bsdf& b, float s0, float s1, float s2, V* world,
                                         float* pdfW, float* cosGen) {
  V result = mk(0.f, 0.f, 0.f, 1.f);
  V gen = zero4();
  if (s2 < b.pd) {
    result = add(result, sample_diffuse(S, b, s0, s1, &gen, pdfW));
    if (zero4(result)) return zero4();
    result = add(result, eval_glossy(S, b, gen, pdfW));
  } else {
    result = add(result, sample_glossy(S, b, s0, s1, &gen, pdfW));
    if (zero4(result)) return zero4();
    result = add(result, eval_diffuse(S, b, gen, pdfW));
  }
  *cosGen = fabsf(gen.z);
  if (*cosGen < kEpsCos) return zero4();
  *world = world_coord(b.frame, gen);
  return result;
}
// Sampling.cl:212-235
__device__ __forceinline__ float mis2(float a, float b) { return a / (a + b); }
__device__ __forceinline__ float pdf_a_to_w(float pdfA, float dist, float c) { return pdfA * (dist * dist) / fabsf(c); }

// ------------------------------------------------------------- lights
struct AreaLight {
  V p1, e1, e2, nz, intensity;
  float invArea;
};
// Light.cl:43-77
__device__ __forceinline__ AreaLight get_area_light(const DevScene& S, const Material& M, int tri) {
  AreaLight L;
  const int* fp = reinterpret_cast<const int*>(S.faces + tri);
  int vx = __ldg(fp + 0), vy = __ldg(fp + 1), vz = __ldg(fp + 2);
  int nx = __ldg(fp + 6), ny = __ldg(fp + 7), nz = __ldg(fp + 8);
  V p1 = ldg4(S.points + vx), p2 = ldg4(S.points + vy), p3 = ldg4(S.points + vz);
  V n;
  if (nx > -1) {
    V n1 = ldg4(S.normals + nx), n2 = ldg4(S.normals + ny), n3 = ldg4(S.normals + nz);
    n = normalize4(divs(add(add(n1, n2), n3), 3.0f));
  } else {
    n = normalize4(cross4(sub(p2, p1), sub(p3, p1)));
  }
  V e1 = xyz0(sub(p2, p1)), e2 = xyz0(sub(p3, p1));
  V nn = cross4(e1, e2);
  L.invArea = 2.f / sqrtf(dot3(nn, nn));
  L.nz = get_frame(n).mZ;
  L.p1 = p1;
  L.e1 = e1;
  L.e2 = e2;
  L.intensity = muls(M.emission_color, M.emission_param.y);
  return L;
}
// Light.cl:85-109
__device__ __forceinline__ V illuminate_area(const AreaLight& L, V recv, float sx, float sy, V* dir, float* dist, float* pdfW) {
  float term = sqrtf(sx);
  float bu = 1.f - term, bv = sy * term;
  V lp = add(add(L.p1, muls(L.e1, bu)), muls(L.e2, bv));
  V dd = sub(lp, recv);
  float d2 = dot4(dd, dd);
  *dist = sqrtf(d2);
  dd = divs(dd, *dist);
  *dir = dd;
  float cN = dot4(L.nz, neg(dd));
  if (cN < kEpsCos) return zero4();
  *pdfW = L.invArea * d2 / cN;
  return L.intensity;
}
// Light.cl:111-127
__device__ __forceinline__ V radiance_area(const AreaLight& L, V rd, float* pdfA) {
  float c = maxf_(0.f, dot4(L.nz, neg(rd)));
  if (c == 0.f) return zero4();
  *pdfA = L.invArea;
  return L.intensity;
}

// ---------------------------------------------------------------- SAT
// SAT.cl: 2-D piecewise-constant sampling off an inclusive SAT.
struct Region { int nu, nv, minX, minY, sx, sy; };
__device__ __forceinline__ int last_x(const Region& r) { return r.minX + r.sx - 1; }
__device__ __forceinline__ int last_y(const Region& r) { return r.minY + r.sy - 1; }
__device__ __forceinline__ float satv(const Region& r, int x, int y, const float* sat) {  // SAT.cl:135-147
  if (x < 0 || y < 0 || x > last_x(r) || y > last_y(r)) return 0.f;
  return __ldg(sat + (size_t)y * r.nu + x);
}
__device__ __forceinline__ float sat_range(const Region& r, int x0, int y0, int x1, int y1, const float* sat) {
  float D1 = satv(r, x1, y1, sat), C1 = satv(r, x0 - 1, y1, sat), B1 = satv(r, x1, y0 - 1, sat),
        A1 = satv(r, x0 - 1, y0 - 1, sat);
  return A1 + D1 - B1 - C1;
}
__device__ __forceinline__ float cond_(const Region& r, int x, int y, const float* sat) {
  float fi = sat_range(r, r.minX, y, last_x(r), y, sat);
  return sat_range(r, r.minX, y, x - 1, y, sat) / fi;
}
__device__ __forceinline__ float marg_(const Region& r, int y, const float* sat) {
  float last = sat_range(r, r.minX, r.minY, last_x(r), last_y(r), sat);
  return sat_range(r, r.minX, r.minY, last_x(r), y - 1, sat) / last;
}
__device__ __forceinline__ float func_at(const Region& r, int x, int y, const float* f) {
  int i = (x < 0 || y < 0 || x > r.nu - 1 || y > r.nv - 1) ? 0 : y * r.nu + x;
  return __ldg(f + i);
}
__device__ __forceinline__ float pdf_cond(const Region& r, int x, int y, const float* sat, const float* f) {
  return func_at(r, x, y, f) / sat_range(r, r.minX, y, last_x(r), y, sat);
}
__device__ __forceinline__ float pdf_marg(const Region& r, int y, const float* sat) {
  float fi = sat_range(r, r.minX, y, last_x(r), y, sat);
  float last = sat_range(r, r.minX, r.minY, last_x(r), last_y(r), sat);
  return (fi * (float)(r.sx * r.sy)) / last;
}
// The values the searches of sample_cont compare: the marginal CDF at row y
// (SAT.cl:190-197) and the conditional CDF at column x of row y (SAT.cl:183-188),
// with the region total `last` and the row integral `fi`.
__device__ __forceinline__ float marg_value(const Region& r, int y, const float* sat, float last) {
  return sat_range(r, r.minX, r.minY, last_x(r), y - 1, sat) / last;
}
__device__ __forceinline__ float cond_value(const Region& r, int x, int y, const float* sat, float fi) {
  return sat_range(r, r.minX, y, x - 1, y, sat) / fi;
}
// SAT.cl:244-259, :275-290, :313-323. The region total and the chosen row's
// integral are read once instead of at every search step (same values, same
// divisions, so the same result as the reference's per-step recomputation).
// marg(y) / cond(x, y, fi) give the CDF values: computed from the SAT, or read
// from tables that hold the same values (RegionTab).
template <class M, class Cd>
__device__ __forceinline__ void sample_cont_with(const Region& r, float u0, float u1, float* uv, int* off, float* pdf,
                                                 const float* sat, const float* f, M marg, Cd cond) {
  float p1, p0;
  const float last = sat_range(r, r.minX, r.minY, last_x(r), last_y(r), sat);
  {
    int b = r.minY, e = r.minY + r.sy;
    while (b != e) {
      int mid = b + (e - b) / 2;
      float mv = marg(mid, last);
      bool right = !(u1 < mv);
      b = right ? mid + 1 : b;
      e = right ? e : mid;
    }
    int o = b - 1 > 0 ? b - 1 : 0;
    off[1] = o;
    float m0 = marg(o, last);
    float du = (u1 - m0) / (marg(o + 1, last) - marg(o, last));
    const float fi = sat_range(r, r.minX, o, last_x(r), o, sat);
    p1 = (fi * (float)(r.sx * r.sy)) / last;  // pdf_marg
    uv[1] = ((float)o + du) / (float)r.nv;
  }
  {
    int y = off[1];
    const float fi = sat_range(r, r.minX, y, last_x(r), y, sat);
    int b = r.minX, e = r.minX + r.sx;
    while (b != e) {
      int mid = b + (e - b) / 2;
      float mv = cond(mid, y, fi);
      bool right = !(u0 < mv);
      b = right ? mid + 1 : b;
      e = right ? e : mid;
    }
    int o = b - 1 > 0 ? b - 1 : 0;
    off[0] = o;
    float c0 = cond(o, y, fi);
    float du = (u0 - c0) / (cond(o + 1, y, fi) - cond(o, y, fi));
    p0 = func_at(r, o, y, f) / fi;  // pdf_cond
    uv[0] = ((float)o + du) / (float)r.nu;
  }
  pdf[0] = p0 * p1;
}
__device__ __forceinline__ void sample_cont(const Region& r, float u0, float u1, float* uv, int* off, float* pdf,
                                            const float* sat, const float* f) {
  sample_cont_with(r, u0, u1, uv, off, pdf, sat, f, [&](int y, float last) { return marg_value(r, y, sat, last); },
                   [&](int x, int y, float fi) { return cond_value(r, x, y, sat, fi); });
}
// Tabulated CDFs of a region, the values marg_value / cond_value give, computed
// once (k_region_tables): marg for rows y = minY-1 .. minY+sy (sy + 2 values),
// cond for rows y = minY-1 .. minY+sy-1, each for columns x = minX-1 .. minX+sx
// (sx + 2 values). The searches then read short contiguous arrays instead of
// four scattered SAT entries per step. Rows and columns one before the region
// serve the searches' edge case (the first row or column chosen, o = b - 1).
struct RegionTab {
  const float* marg;
  const float* cond;
};
__device__ __forceinline__ void sample_cont_tab(const Region& r, float u0, float u1, float* uv, int* off, float* pdf,
                                                const float* sat, const float* f, RegionTab t) {
  const int cw = r.sx + 2;
  sample_cont_with(
      r, u0, u1, uv, off, pdf, sat, f, [&](int y, float) { return __ldg(t.marg + (y - r.minY + 1)); },
      [&](int x, int y, float) { return __ldg(t.cond + (size_t)(y - r.minY + 1) * cw + (x - r.minX + 1)); });
}

// Util.cl:397-439
__device__ __forceinline__ void sph_xy(int w, int h, V d, int* x, int* y) {
  float phi = acosf(d.y);
  float theta = atan2f(d.z, d.x);
  *x = (int)((0.5f - 0.5f * theta / kPi) * (float)w);
  *y = (int)((phi / kPi) * (float)h);
}
__device__ __forceinline__ int sph_index(int w, int h, int x, int y) {
  int idx = (int)((float)x + (float)y * (float)w);
  if (idx < 0) idx = 0;
  if (idx > w * h - 1) idx = w * h - 1;
  return idx;
}
__device__ __forceinline__ V sph_dir(float u, float v) {
  float phi = kPi * v;
  float theta = u * 2.f * kPi;
  return mk(-sinf(phi) * cosf(theta), cosf(phi), sinf(phi) * sinf(theta), 0.f);
}
// Light.cl:195-227
__device__ __forceinline__ V illuminate_env(const DevEnv& E, V s, V* dir, float* dist, float* pdfW) {
  Region r{E.w, E.h, 0, 0, E.w, E.h};
  float uv[2];
  int off[2];
  float pdf;
  if (E.env_marg)  // tables of the map's CDFs
    sample_cont_tab(r, s.x, s.y, uv, off, &pdf, E.sat, E.lum, RegionTab{E.env_marg, E.env_cond});
  else
    sample_cont(r, s.x, s.y, uv, off, &pdf, E.sat, E.lum);
  V d = sph_dir(uv[0], uv[1]);
  *dir = d;
  int x, y;
  sph_xy(E.w, E.h, d, &x, &y);
  V c = ldg4(E.rgb + sph_index(E.w, E.h, x, y));
  float sinT = sinf(uv[1] * kPi);
  *pdfW = pdf / (2.f * kPi * kPi * sinf(uv[1] * kPi));
  *dist = kFloatMax;
  if (sinT == 0.f) *pdfW = 0.f;
  return c;
}
// Light.cl:270-286
__device__ __forceinline__ V radiance_env(const DevEnv& E, V d, float* pdfA) {
  int x, y;
  sph_xy(E.w, E.h, d, &x, &y);
  V c = ldg4(E.rgb + sph_index(E.w, E.h, x, y));
  Region r{E.w, E.h, 0, 0, E.w, E.h};
  int xc = x > E.w - 1 ? E.w - 1 : x, yc = y > E.h - 1 ? E.h - 1 : y;
  float pdfXY = pdf_cond(r, xc, yc, E.sat, E.lum) * pdf_marg(r, yc, E.sat);
  float v = (float)y / (float)r.sy;
  *pdfA = pdfXY / (2.f * kPi * kPi * sinf(v * kPi));
  return c;
}


// ------------------------------------------------------ adaptive light grid
// LightGrid.cl:39-343 and the grid versions of the environment light,
// illuminateEnvironmentLight1 / getRadianceEnvironmentLight1 (Light.cl:140-268).
// The grid holds nu x nv values: (nu/rx) x (nv/ry) cells of rx x ry tiles; a
// shading point's cell is the direction camera -> point, a tile a sub-region of
// the environment map. The tile is drawn from the cell's SAT, then the texel
// from the tile's region of the full-map SAT. The reference leaves the tile's
// probability out of the direction pdf and never calls these versions; here
// the pdf is pdfLL * pdfSS (tile density over the cell's tile square times
// texel density over the tile), the density of the direction over the map's
// uv square when tiles divide the map, which mt_job_create checks.
// Cell lookups take the direction from the xyz lanes.
__device__ __forceinline__ int grid_cell(const DevEnv& E, const float* cam, V p) {
  const int cw = E.nu / E.rx, ch = E.nv / E.ry;
  V d = normalize3(mk(p.x - cam[0], p.y - cam[1], p.z - cam[2], 0.f));
  int x, y;
  sph_xy(cw, ch, d, &x, &y);
  return sph_index(cw, ch, x, y);
}
// Offset of a cell's first tile in the grid arrays (subgridGlobalIndex2,
// LightGrid.cl:107-110: cell (cx, cy) starts at (cx * rx, cy * ry)). Each cell
// holds its own SAT, so a cell is sampled as the region (0, 0, rx, ry) of the
// arrays offset to its first tile with row pitch nu: reads left of or above
// the cell give 0 as getSubgridValueSAT's range check does (LightGrid.cl:142-147).
__device__ __forceinline__ size_t grid_cell_base(const DevEnv& E, int cell) {
  const int cw = E.nu / E.rx;
  return (size_t)((cell / cw) * E.ry) * E.nu + (size_t)((cell % cw) * E.rx);
}
// getSubgridUnitBound + getSubRegionFromUnitBound (LightGrid.cl:157-165,
// SAT.cl:28-44): tile (tx, ty) of rx x ry as a region of the w x h map.
__device__ __forceinline__ Region env_tile_region(const DevEnv& E, int tx, int ty) {
  const float ux0 = (float)tx / (float)E.rx, uy0 = (float)ty / (float)E.ry;
  const float ux1 = (float)(tx + 1) / (float)E.rx, uy1 = (float)(ty + 1) / (float)E.ry;
  const int x0 = (int)((float)E.w * ux0), y0 = (int)((float)E.h * uy0);
  const int x1 = (int)((float)E.w * ux1), y1 = (int)((float)E.h * uy1);
  return Region{E.w, E.h, x0, y0, x1 - x0, y1 - y0};
}
__device__ __forceinline__ V illuminate_env_grid(const DevEnv& E, const float* cam, V p, V s, V* dir, float* dist,
                                                 float* pdfW) {
  const int cell = grid_cell(E, cam, p);
  const size_t base = grid_cell_base(E, cell);
  const Region rc{E.nu, E.nv, 0, 0, E.rx, E.ry};
  float uvLL[2], pdfLL, uvSS[2], pdfSS;
  int offLL[2], offSS[2];
  if (E.cell_marg)  // tables of the cell's CDFs
    sample_cont_tab(rc, s.x, s.y, uvLL, offLL, &pdfLL, E.grid_sat + base, E.grid_func + base,
                    RegionTab{E.cell_marg + (size_t)cell * (E.ry + 2),
                              E.cell_cond + (size_t)cell * (E.ry + 1) * (E.rx + 2)});
  else
    sample_cont(rc, s.x, s.y, uvLL, offLL, &pdfLL, E.grid_sat + base, E.grid_func + base);
  *dist = kFloatMax;
  *pdfW = 0.f;
  if (!(pdfLL > 0.f)) return zero4();  // empty cell: the BSDF sample covers it alone
  const Region rt = env_tile_region(E, offLL[0], offLL[1]);
  if (E.tile_marg) {  // tables of the tile's CDFs (tiles divide the map: every tile is tw x th)
    const int tw = E.w / E.rx, th = E.h / E.ry, tile = offLL[1] * E.rx + offLL[0];
    sample_cont_tab(rt, s.z, s.w, uvSS, offSS, &pdfSS, E.sat, E.lum,
                    RegionTab{E.tile_marg + (size_t)tile * (th + 2), E.tile_cond + (size_t)tile * (th + 1) * (tw + 2)});
  } else {
    sample_cont(rt, s.z, s.w, uvSS, offSS, &pdfSS, E.sat, E.lum);
  }
  if (!(pdfSS > 0.f)) return zero4();
  V d = sph_dir(uvSS[0], uvSS[1]);
  *dir = d;
  int x, y;
  sph_xy(E.w, E.h, d, &x, &y);
  V c = ldg4(E.rgb + sph_index(E.w, E.h, x, y));
  float sinT = sinf(uvSS[1] * kPi);
  *pdfW = (pdfLL * pdfSS) / (2.f * kPi * kPi * sinf(uvSS[1] * kPi));
  if (sinT == 0.f) *pdfW = 0.f;
  return c;
}
// pdf of direction d under illuminate_env_grid from shading point p, and the
// radiance; the tile is the one holding d's texel, and the sine term takes
// v = y / h over the whole map (the reference's unused version divides by the
// tile's height, Light.cl:253). accumulate: add the texel's
// luminance into the grid's accumulation array at (cell, tile)
// (getRadianceEnvironmentLight1 with accumLightGrid, Light.cl:35-38).
__device__ __forceinline__ V radiance_env_grid(const DevEnv& E, const float* cam, V p, V d, float* pdfA,
                                               bool accumulate) {
  int x, y;
  sph_xy(E.w, E.h, d, &x, &y);
  V c = ldg4(E.rgb + sph_index(E.w, E.h, x, y));
  const int xc = x > E.w - 1 ? E.w - 1 : (x < 0 ? 0 : x), yc = y > E.h - 1 ? E.h - 1 : (y < 0 ? 0 : y);
  const int tx = xc / (E.w / E.rx), ty = yc / (E.h / E.ry);
  const size_t base = grid_cell_base(E, grid_cell(E, cam, p));
  const Region rc{E.nu, E.nv, 0, 0, E.rx, E.ry};
  const float pdfLL =
      pdf_cond(rc, tx, ty, E.grid_sat + base, E.grid_func + base) * pdf_marg(rc, ty, E.grid_sat + base);
  const Region rt = env_tile_region(E, tx, ty);
  const float pdfSS = pdf_cond(rt, xc, yc, E.sat, E.lum) * pdf_marg(rt, yc, E.sat);
  const float v = (float)y / (float)E.h;
  float pdf = (pdfLL * pdfSS) / (2.f * kPi * kPi * sinf(v * kPi));
  *pdfA = pdf > 0.f ? pdf : 0.f;  // also maps NaN from an empty cell or tile to 0
  if (accumulate)
    atomicAdd(E.grid_accum + base + (size_t)ty * E.nu + tx, luminance(c.x, c.y, c.z));
  return c;
}

}  // namespace dv
}  // namespace mt
