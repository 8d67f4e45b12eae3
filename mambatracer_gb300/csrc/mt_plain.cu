// The reference's kernel set by name, over the reference's own buffer layouts.
//
// OpenCLConfiguration.createKernel(name, args...) + execute1DKernel(k, global,
// local) is how every MambaTracer host class drives the device
// (CDeviceGI.java:166-179 and :214-271, CCompact.java:55-89, CImage.java:98-136,
// CLightConfiguration.java:43-87, CAdaptiveEnvironment.java:37-145). This file
// gives each of those kernels a CUDA implementation with the same name,
// argument list (buffers in the reference layouts: 80-byte Ray, 96-byte
// Intersection, 304-byte Path, 16-byte State, 28-byte BVHNode, 32-byte
// BoundingBox, 80-byte TextureData, the LightGrid struct) and semantics, so a
// host that keeps its own loop can swap JOCL for this library kernel by kernel.
// It is the plain wavefront: one launch per reference kernel, one thread per
// queue slot, the BVH traversed in the reference's node layout, AoS state
// re-read and re-written by every kernel. The fused path (mt_render_frame) is
// the fast one; this one is the drop-in and the comparison point.
//
// Shading arithmetic is shared with the fused path (mt_device.cuh), so both
// produce the reference's results. Where the reference reads out of bounds
// (lane 0 of its Kogge-Stone scans reads aux[-1]) the value read is 0; the
// group scan writes its first prefix (0), which the reference leaves unset.
// Indices read from buffers (pixel indices, BVH links, face vertices) are
// checked against the buffers' sizes; a bad one latches an error that
// mt_finish returns, and the access is skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "mt_device.cuh"
#include "mt_compact.h"
#include "mt_internal.h"
#include "mt_traverse.cuh"

namespace mt {
namespace plain {

using namespace dv;

struct RRay {  // Util.cl:129-138
  float4 o, d, inv_d;
  int4 sign;
  int2 extra;
  float tMin, tMax;
};
struct RIsect {  // Util.cl:141-151
  float4 p, n, ng, d;
  float2 uv;
  int mat, id, hit;
};
struct RFrame {
  float4 mX, mY, mZ;
};
struct RBsdf {  // Bsdf.cl:52-64
  Material param;
  RFrame frame;
  float4 localDirFix, localGeomN;
  int materialID;
  float diffProb, glossyProb, reflProb, refrProb;
};
struct RPath {  // Path.cl:1-11
  float4 throughput, hitpoint;
  int pathlength, lastSpecular;
  float lastPdfW;
  int active;
  RBsdf bsdf;
};
struct RState {  // Sampling.cl:2-6
  int2 seed;
  float frameCount;
};
struct RTex {  // Material.cl:2-10
  int4 diffuse, glossy, roughness, mirror, parameters;
};
struct RLight {  // Util.cl:160-165
  int faceId, type;
};
struct RNode {  // NormalBVH.cl:1-11
  int bound, sibling, left, right, parent, isLeaf, child;
};
struct RBound {  // Util.cl:116-121
  float4 mn, mx;
};
static_assert(sizeof(RRay) == 80, "Ray");
static_assert(sizeof(RIsect) == 96, "Intersection");
static_assert(sizeof(RBsdf) == 256, "Bsdf");
static_assert(sizeof(RPath) == 304, "Path");
static_assert(sizeof(RState) == 16, "State");
static_assert(sizeof(RTex) == 80, "TextureData");
static_assert(sizeof(RNode) == 28, "BVHNode");
static_assert(sizeof(RBound) == 32, "BoundingBox");

// LightGrid (LightGrid.cl:9-37): header, then accum, func and sat of 2,560,000 floats.
constexpr size_t kGridValues = 2560000;
constexpr size_t kGridHeader = 48;
constexpr size_t kGridBytes = kGridHeader + 3 * kGridValues * 4;
struct GridHdr {
  unsigned char isPresent, pad_[3];
  int sampleTile, width, height, nu, nv, rx, ry;
  float4 cameraPosition;
};
static_assert(sizeof(GridHdr) == kGridHeader, "LightGrid header");

__device__ __forceinline__ void latch(int* err, int code) { atomicCAS(err, 0, code); }

constexpr int kErrIndex = 1;  // an index read from a buffer is out of range
constexpr int kErrStack = 2;  // BVH deeper than the 64-entry stack

// --------------------------------------------------------------- helpers
__device__ __forceinline__ V v4(float4 a) { return mk(a.x, a.y, a.z, a.w); }
__device__ __forceinline__ float4 f4(V a) { return make_float4(a.x, a.y, a.z, a.w); }

// initGlobalRay / initGlobalRayT (Util.cl:577-600)
__device__ __forceinline__ void init_ray(RRay* r, V o, V d, float tmin, float tmax) {
  r->o = f4(o);
  r->d = f4(d);
  r->inv_d = make_float4(1.f / d.x, 1.f / d.y, 1.f / d.z, 0.f);
  r->sign = make_int4(r->inv_d.x < 0 ? 1 : 0, r->inv_d.y < 0 ? 1 : 0, r->inv_d.z < 0 ? 1 : 0, r->sign.w);
  r->tMin = tmin;
  r->tMax = tmax;
}

// initIsect (Initialize.cl:12-22): ng is left as it is
__device__ __forceinline__ void init_isect(RIsect* is) {
  is->p = make_float4(0.f, 0.f, 0.f, 0.f);
  is->n = make_float4(0.f, 0.f, 0.f, 0.f);
  is->d = make_float4(0.f, 0.f, 0.f, 0.f);
  is->uv = make_float2(0.f, 0.f);
  is->id = -1;
  is->hit = 0;
  is->mat = -1;
}

// addAccum (Render.cl:1-7) with atomicAddFloat4's CAS loop replaced by atomics:
// one writer per pixel per launch, so the sums are the same.
__device__ __forceinline__ void add_accum(float4* acc, V v) {
  if (!abs_valid4(v)) return;
  atomicAdd(&acc->x, v.x);
  atomicAdd(&acc->y, v.y);
  atomicAdd(&acc->z, v.z);
  atomicAdd(&acc->w, v.w);
}

struct MeshArgs {
  const float4* points;
  const float2* uvs;
  const float4* normals;
  const Face* faces;
  const Material* materials;
  int npoints, nfaces, nmat, nuvs, nnormals;
};
__device__ __forceinline__ DevScene scene_of(const MeshArgs& m) {
  DevScene S{};
  S.points = m.points;
  S.uvs = m.uvs;
  S.normals = m.normals;
  S.faces = m.faces;
  S.materials = m.materials;
  S.ntri = m.nfaces;
  return S;
}
__device__ __forceinline__ bool face_ok(const MeshArgs& m, int f) {
  if (f < 0 || f >= m.nfaces) return false;
  const Face& F = m.faces[f];
  auto in = [](int i, int n) { return i >= 0 && i < n; };
  // uv and normal indices are used when the first one is > -1 (Util.cl:270-300)
  return in(F.vx, m.npoints) && in(F.vy, m.npoints) && in(F.vz, m.npoints) && (F.mat & 0xFFFF) < m.nmat &&
         (F.uvx <= -1 || (in(F.uvx, m.nuvs) && in(F.uvy, m.nuvs) && in(F.uvz, m.nuvs))) &&
         (F.nx <= -1 || (in(F.nx, m.nnormals) && in(F.ny, m.nnormals) && in(F.nz, m.nnormals)));
}

struct BvhArgs {
  const RNode* nodes;
  const RBound* bounds;
  int nnodes, nbounds;
};

// intersectMesh / testOcclusion (NormalBVH.cl:14-92, :235-317) on the
// reference's node layout, in the reference's visit order: both child boxes
// tested, the nearer entered (the right one only if strictly nearer), the
// other deferred; a leaf is one triangle accepted when tMin < t < tMax. A
// deferred interior node whose entry distance is not below the closest hit is
// dropped (its children cannot be hit), as in the fused traversal.
template <bool ANY>
__device__ int trace_ref(const BvhArgs& B, const MeshArgs& M, tr::RayT& r, int* err) {
  int2 stack[kStackDepth];
  int sp = 0;
  int hit = -1;
  const bool finite = tr::ray_is_finite(r);
  int node = 0;
  if (B.nnodes <= 0) return -1;
  for (;;) {
    const RNode nd = B.nodes[node];
    if (!nd.isLeaf) {
      if (nd.left <= 0 || nd.right <= 0 || nd.left >= B.nnodes || nd.right >= B.nnodes) {
        latch(err, kErrIndex);
        return hit;
      }
      const int bl = B.nodes[nd.left].bound, br = B.nodes[nd.right].bound;
      if (bl < 0 || br < 0 || bl >= B.nbounds || br >= B.nbounds) {
        latch(err, kErrIndex);
        return hit;
      }
      const RBound L = B.bounds[bl], R = B.bounds[br];
      float tl, trr;
      bool hl, hr;
      if (finite) {
        hl = tr::slab_fast(r, r.sx ? L.mx.x : L.mn.x, r.sx ? L.mn.x : L.mx.x, r.sy ? L.mx.y : L.mn.y,
                           r.sy ? L.mn.y : L.mx.y, r.sz ? L.mx.z : L.mn.z, r.sz ? L.mn.z : L.mx.z, &tl);
        hr = tr::slab_fast(r, r.sx ? R.mx.x : R.mn.x, r.sx ? R.mn.x : R.mx.x, r.sy ? R.mx.y : R.mn.y,
                           r.sy ? R.mn.y : R.mx.y, r.sz ? R.mx.z : R.mn.z, r.sz ? R.mn.z : R.mx.z, &trr);
      } else {
        hl = tr::slab(r, L.mn.x, L.mx.x, L.mn.y, L.mx.y, L.mn.z, L.mx.z, &tl);
        hr = tr::slab(r, R.mn.x, R.mx.x, R.mn.y, R.mx.y, R.mn.z, R.mx.z, &trr);
      }
      if (hl && hr) {
        const bool rfirst = trr < tl;
        if (sp >= kStackDepth) {
          latch(err, kErrStack);
          return hit;
        }
        stack[sp++] = make_int2(rfirst ? nd.left : nd.right, __float_as_int(rfirst ? tl : trr));
        node = rfirst ? nd.right : nd.left;
        continue;
      }
      if (hl) {
        node = nd.left;
        continue;
      }
      if (hr) {
        node = nd.right;
        continue;
      }
    } else {
      const int f = nd.child;
      if (!face_ok(M, f)) {
        latch(err, kErrIndex);
        return hit;
      }
      const Face& F = M.faces[f];
      const float4 p1 = M.points[F.vx], p2 = M.points[F.vy], p3 = M.points[F.vz];
      const float4 e1 = make_float4(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z, p2.w - p1.w);
      const float4 e2 = make_float4(p3.x - p1.x, p3.y - p1.y, p3.z - p1.z, p3.w - p1.w);
      const float t = tr::tri_t(r, p1, e1, e2);
      if ((r.tmin < t) && (t < r.tmax)) {
        hit = f;
        if (ANY) return hit;
        r.tmax = t;
      }
    }
    for (;;) {
      if (sp == 0) return hit;
      const int2 e = stack[--sp];
      if (ANY || !finite || B.nodes[e.x].isLeaf || __int_as_float(e.y) < r.tmax) {
        node = e.x;
        break;
      }
    }
  }
}

__device__ __forceinline__ tr::RayT ray_of(const RRay& rr) {
  return tr::make_ray(rr.o, rr.d, rr.tMin, rr.tMax);
}

// Bsdf of a path in the fused path's form, parameters read from the path's copy.
__device__ __forceinline__ Bsdf bsdf_of(const RPath* path) {
  Bsdf b;
  b.frame.mX = v4(path->bsdf.frame.mX);
  b.frame.mY = v4(path->bsdf.frame.mY);
  b.frame.mZ = v4(path->bsdf.frame.mZ);
  b.fix = v4(path->bsdf.localDirFix);
  b.mat = path->bsdf.materialID;
  b.pd = path->bsdf.diffProb;
  b.pg = path->bsdf.glossyProb;
  b.pm = &path->bsdf.param;
  return b;
}

// ------------------------------------------------------------ kernels
// InitCameraRayDataJitter (Initialize.cl:129-172); the camera constants come
// from the host (read from the camera buffer at launch), the seed from State.
__global__ void k_init_camera_rays(PassParams pp, RRay* rays, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = min(*length, cap);
  if (id >= n) return;
  Seed s = gen_seed(pp.seeds[0], pp.seeds[1], pp.frame_count, id);
  const float r0 = rnd(s), r1 = rnd(s);
  const int W = pp.width;
  const float px = (float)(id % W), py = (float)(id / W);
  const float j1 = pp.inv_w * (2.f * r0 - 1.f);
  const float j2 = pp.inv_h * (2.f * r1 - 1.f);
  V d = normalize4(mk(pp.cam_a * (2.f * px / pp.dim_w - 1.f + j1), -2.f * py / pp.dim_h + 1.f + j2, -pp.cam_d, 0.f));
  const float* m = pp.cam_m;
  V z = zero4();
  V m0 = mk(m[0], m[1], m[2], m[3]), m1 = mk(m[4], m[5], m[6], m[7]), m2 = mk(m[8], m[9], m[10], m[11]),
    m3 = mk(m[12], m[13], m[14], m[15]);
  V o = mk(dot3(m0, z) + m0.w, dot3(m1, z) + m1.w, dot3(m2, z) + m2.w, dot3(m3, z) + m3.w);
  if (!(o.w == 1.f)) o = mk(o.x / o.w, o.y / o.w, o.z / o.w, 0.f);
  o.w = 0.f;
  V dw = mk(dot4(m0, d), dot4(m1, d), dot4(m2, d), 0.f);
  init_ray(rays + id, o, dw, 0.001f, CUDART_INF_F);
}

// InitPathData (Initialize.cl:24-45)
__global__ void k_init_path(RPath* paths, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*length, cap)) return;
  RPath* p = paths + id;
  p->throughput = make_float4(1.f, 1.f, 1.f, 1.f);
  p->lastSpecular = 1;
  p->lastPdfW = 1.f;
  p->active = 1;
  p->bsdf.materialID = -1;
  p->bsdf.frame.mX = p->bsdf.frame.mY = p->bsdf.frame.mZ = make_float4(0.f, 0.f, 0.f, 0.f);
  p->bsdf.localDirFix = make_float4(0.f, 0.f, 0.f, 0.f);
  p->hitpoint = make_float4(0.f, 0.f, 0.f, 0.f);
}

// InitIntersection (Initialize.cl:47-56)
__global__ void k_init_isect(RIsect* is, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) init_isect(is + id);
}

// InitIntDataToIndex / InitIntData / InitFloatData / InitFloat4DataXYZ /
// InitIntDataRGB (Initialize.cl:58-98): value per element
__global__ void k_fill_index(int* a, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) a[id] = id;
}
__global__ void k_fill_u32(unsigned* a, unsigned v, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) a[id] = v;
}
__global__ void k_fill_f4(float4* a, float4 v, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) a[id] = v;
}

// IntersectPrimitives (NormalBVH.cl:94-233)
__global__ void k_intersect(RRay* rays, RIsect* isects, const int* count, int cap, MeshArgs M, BvhArgs B, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  RIsect* is = isects + id;
  if (id < *count) {
    RRay* ray = rays + id;
    tr::RayT r = ray_of(*ray);
    const int f = trace_ref<false>(B, M, r, err);
    if (f >= 0) {
      ray->tMax = r.tmax;
      DevScene S = scene_of(M);
      Hit H;
      hit_record(S, v4(ray->o), v4(ray->d), r.tmax, f, H);
      is->p = f4(H.p);
      is->n = f4(H.n);
      is->ng = f4(H.ng);
      is->d = ray->d;
      is->uv = make_float2(H.u, H.v);
      is->id = f;
      is->mat = H.mat;
      is->hit = 1;
      return;
    }
  }
  is->hit = 0;
  is->mat = -1;
}

// SetupBSDFPath (Render.cl:10-40)
__global__ void k_setup_bsdf(RIsect* isects, const RRay* rays, RPath* paths, int npaths, const Material* materials,
                             int nmat, const int* pixels, const int* count, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  RIsect* is = isects + id;
  if (!is->hit) return;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths || is->mat < 0 || is->mat >= nmat) {
    latch(err, kErrIndex);
    return;
  }
  DevScene S{};
  S.materials = materials;
  const Bsdf b = setup_bsdf(S, v4(rays[id].d), v4(is->n), is->mat);
  if (b.mat < 0) {
    is->hit = 0;
    return;
  }
  RBsdf& o = paths[pix].bsdf;
  o.param = materials[b.mat];
  o.frame.mX = f4(b.frame.mX);
  o.frame.mY = f4(b.frame.mY);
  o.frame.mZ = f4(b.frame.mZ);
  o.localDirFix = f4(b.fix);
  o.localGeomN = f4(local_coord(b.frame, v4(is->ng)));
  o.materialID = b.mat;
  o.diffProb = b.pd;
  o.glossyProb = b.pg;
}

struct EnvArgs {
  const float4* rgb;
  const float* lum;
  const float* sat;
  const GridHdr* grid;
};
__device__ __forceinline__ DevEnv env_of(const EnvArgs& A) {
  DevEnv E{};
  E.rgb = A.rgb;
  E.lum = A.lum;
  E.sat = A.sat;
  E.w = A.grid->width;
  E.h = A.grid->height;
  E.present = A.grid->isPresent != 0;
  return E;
}

// LightHitPass (Render.cl:42-125)
__global__ void k_light_hit(RIsect* isects, const RRay* rays, RPath* paths, int npaths, const int* total_lights,
                            MeshArgs M, float4* accum, const int* pixels, const int* count, int cap, EnvArgs A,
                            int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  RIsect* is = isects + id;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths) {
    latch(err, kErrIndex);
    return;
  }
  RPath* path = paths + pix;
  const RRay& ray = rays[id];
  if (is->hit) {
    const Material& P = path->bsdf.param;
    if (!is_emitter(P)) return;
    if (!face_ok(M, is->id)) {
      latch(err, kErrIndex);
      return;
    }
    const float pick = 1.f / (float)*total_lights;
    DevScene S = scene_of(M);
    AreaLight L = get_area_light(S, P, is->id);
    float pdfA = 0.f;
    V c = radiance_area(L, v4(ray.d), &pdfA);
    if (zero3(c)) return;
    float w = 1.f;
    if (!path->lastSpecular) {
      const float pdfW = pdf_a_to_w(pdfA, ray.tMax, path->bsdf.localDirFix.z);
      w = mis2(path->lastPdfW, pdfW * pick);
    }
    add_accum(accum + pix, muls(mul(v4(path->throughput), c), w));
    is->hit = 0;
  } else if (A.grid->isPresent) {
    DevEnv E = env_of(A);
    float pdfW = 0.f;
    V c = radiance_env(E, v4(ray.d), &pdfW);
    if (zero3(c)) return;
    float w = 1.f;
    if (!path->lastSpecular) w = mis2(path->lastPdfW, pdfW);
    add_accum(accum + pix, muls(mul(v4(path->throughput), c), w));
  }
}

// texturePassGI (Render.cl:127-187): the material id is written for every
// work-item, as in the reference; texture flags and uv bits below the count.
__global__ void k_texture_pass(const RPath* paths, int npaths, const RIsect* isects, RTex* tex, const int* pixels,
                               const int* count, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths) {
    latch(err, kErrIndex);
    return;
  }
  const RBsdf& b = paths[pix].bsdf;
  RTex* t = tex + id;
  t->parameters.x = b.materialID;
  if (id < *count) {
    const RIsect& is = isects[id];
    const int ux = __float_as_int(is.uv.x), uy = __float_as_int(is.uv.y);
    if (b.param.isDiffuseTexture) {
      t->diffuse.w = 1;
      t->diffuse.x = ux;
      t->diffuse.y = uy;
    } else {
      t->diffuse.w = 0;
    }
    if (b.param.isGlossyTexture) {
      t->glossy.w = 1;
      t->glossy.x = ux;
      t->glossy.y = uy;
    } else {
      t->glossy.w = 0;
    }
    if (b.param.isRoughnessTexture) {
      t->roughness.w = 1;
      t->roughness.x = ux;
      t->roughness.y = uy;
    } else {
      t->roughness.w = 0;
    }
  }
}

// CTextureApplyPass.process (CTextureApplyPass.java:37-92) on the device, in
// place of the reference's per-bounce copy of TextureData to the host and back:
// below the count, each flagged texture (w > 0) of the slot's material
// (parameters.x) with an image gets its ARGB texel in z; without an image z is
// left as it was, as the host pass leaves it. tex_ref: 4 int4 per material
// (first texel, width, height, 0) for diffuse, glossy, roughness, mirror.
__global__ void k_texture_apply(RTex* tex, const int* count, const int* __restrict__ texels, long long ntexels,
                                const int4* __restrict__ tex_ref, int nref, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  RTex& t = tex[id];
  const int mat = t.parameters.x;
  int4* kinds[3] = {&t.diffuse, &t.glossy, &t.roughness};
  for (int k = 0; k < 3; ++k) {
    int4& e = *kinds[k];
    if (e.w <= 0) continue;
    if (mat < 0 || 4 * (long long)mat + k >= nref) {
      latch(err, kErrIndex);
      return;
    }
    const int4 r = tex_ref[4 * mat + k];
    if (r.y <= 0 || r.z <= 0) continue;
    if (r.x < 0 || (long long)r.x + (long long)r.y * r.z > ntexels) {
      latch(err, kErrIndex);
      return;
    }
    e.z = tex_fetch(texels, r, __int_as_float(e.x), __int_as_float(e.y));
  }
}

// updateToTextureColorGI (Render.cl:189-231)
__global__ void k_texture_color(RPath* paths, int npaths, const RTex* tex, const int* pixels, const int* count,
                                int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths) {
    latch(err, kErrIndex);
    return;
  }
  Material& P = paths[pix].bsdf.param;
  const RTex& t = tex[id];
  if (t.diffuse.w) P.diffuse_color = argb_float4(t.diffuse.z);
  if (t.glossy.w) P.glossy_color = argb_float4(t.glossy.z);
  if (t.roughness.w) {
    const float4 c = argb_float4(t.roughness.z);
    P.glossy_param.y = fmaxf(0.001f, c.x);
    P.glossy_param.z = fmaxf(0.001f, c.y);
  }
}

// SampleBSDFRayDirection (Render.cl:233-285)
__global__ void k_sample_bsdf(RIsect* isects, RRay* rays, RPath* paths, int npaths, const int* pixels,
                              const RState* state, const int* count, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths) {
    latch(err, kErrIndex);
    return;
  }
  RPath* path = paths + pix;
  RIsect* is = isects + id;
  Seed s = gen_seed(state->seed.x, state->seed.y, state->frameCount, id);
  const float s0 = rnd(s), s1 = rnd(s), s2 = rnd(s);
  DevScene S{};
  const Bsdf b = bsdf_of(path);
  V dir = zero4();
  float pdf = 0.f, cosO = 0.f;
  V f = sample_bsdf(S, b, s0, s1, s2, &dir, &pdf, &cosO);
  const float q = cosO / pdf;
  V thr = mul(v4(path->throughput), muls(f, q));
  path->throughput = f4(thr);
  path->lastSpecular = 0;
  path->lastPdfW = pdf;
  path->hitpoint = is->p;
  init_ray(rays + id, v4(is->p), dir, 0.001f, CUDART_INF_F);
  init_isect(is);
}

// DirectLight (Render.cl:377-466) with illuminateLight / illuminateMeshLight
// (:287-375): the light sample and the BSDF sample of a slot share its State
// seed, and the mesh light used is light 0 (Render.cl:305).
__global__ void k_direct_light(const RPath* paths, int npaths, const RIsect* isects, const RLight* lights, int nlights_cap,
                               const int* total_lights, RRay* occlus, float4* accum, const int* pixels,
                               const int* count, int cap, const RState* state, MeshArgs M, BvhArgs B, EnvArgs A,
                               int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*count, cap)) return;
  const int pix = pixels[id];
  if (pix < 0 || pix >= npaths) {
    latch(err, kErrIndex);
    return;
  }
  const RPath* path = paths + pix;
  const RIsect& is = isects[id];
  Seed s = gen_seed(state->seed.x, state->seed.y, state->frameCount, id);
  const int nl = *total_lights;
  const bool env = A.grid->isPresent != 0;
  float pick = 1.f;
  V smp;
  smp.x = rnd(s);
  smp.y = rnd(s);
  smp.z = rnd(s);
  smp.w = rnd(s);
  bool smesh = false, senv = false;
  if (env && nl > 0) {
    const float r = rnd(s);
    pick = pick * 0.5f;
    if (r < 0.5f) smesh = true; else senv = true;
  } else if (env) {
    senv = true;
  } else if (nl > 0) {
    smesh = true;
  }
  V dir = zero4(), rad = zero4();
  float dist = 0.f, pdfW = 0.f;
  DevScene S = scene_of(M);
  if (smesh) {
    (void)rnd(s);  // random_int_range: the index is drawn, light 0 is used
    if (nlights_cap < 1) {
      latch(err, kErrIndex);
      return;
    }
    const int tri = lights[0].faceId;
    if (!face_ok(M, tri)) {
      latch(err, kErrIndex);
      return;
    }
    pick = pick * (1.f / (float)nl);
    const Material& Ml = M.materials[M.faces[tri].mat & 0xFFFF];
    AreaLight L = get_area_light(S, Ml, tri);
    rad = illuminate_area(L, v4(is.p), smp.x, smp.y, &dir, &dist, &pdfW);
  } else if (senv) {
    DevEnv E = env_of(A);
    rad = illuminate_env(E, smp, &dir, &dist, &pdfW);
  }
  if (zero3(rad)) return;
  const Bsdf b = bsdf_of(path);
  float bpdf = 0.f, cosO = 0.f;
  V f = eval_bsdf(S, b, dir, &bpdf, &cosO);
  if (zero3(f)) return;
  const float w = mis2(pdfW, bpdf);
  const float sc = (w * cosO / (pick * pdfW));
  const V thr = v4(path->throughput);
  const V contrib = mk(sc * (rad.x * f.x) * thr.x, sc * (rad.y * f.y) * thr.y, sc * (rad.z * f.z) * thr.z, 1.f);
  RRay* ray = occlus + id;
  init_ray(ray, v4(is.p), dir, 0.0001f, dist - 2.f * 1e-3f);
  tr::RayT r = ray_of(*ray);
  if (trace_ref<true>(B, M, r, err) < 0) add_accum(accum + pix, contrib);
}

// CompactAtomic's transfers (Compact.cl:2-19)
__global__ void k_copy_isects(RIsect* dst, const RIsect* src, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) dst[id] = src[id];
}
__global__ void k_copy_ints(int* dst, const int* src, const int* length, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < min(*length, cap)) dst[id] = src[id];
}

// averageAccum (Image.cl:29-67)
__global__ void k_average_accum(const float4* accum, const float* fc, float4* fb, float* loglw, int* cnt,
                                const int* size, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  loglw[id] = 0.f;
  cnt[id] = 0;
  if (id < *size) {
    const float4 a = accum[id];
    const float4 f = make_float4(a.x / fc[0], a.y / fc[0], a.z / fc[0], 1.f);
    fb[id] = f;
    const float Lw = luminance(f.x, f.y, f.z);
    if (Lw > 0.f) {
      loglw[id] = logf(0.01f + Lw);
      cnt[id] = 1;
    }
  }
}

__device__ __forceinline__ int argb_int(float r, float g, float b, float a) {  // getIntARGB, Util.cl:469-480
  auto q = [](float v) { return (int)(fminf(fmaxf(v, 0.f), 1.f) * 255.0f); };
  return (q(a) << 24) | (q(r) << 16) | (q(g) << 8) | q(b);
}

// updateFrameImage (Image.cl:70-118)
__global__ void k_update_frame_image(float4* fb, int* argb, const float* total_log, const int* total_n,
                                     const int* size, const float* exposure, const float* gamma, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  float logavg = total_log[0] / (float)total_n[0];
  logavg = expf(logavg);
  if (id >= min(*size, cap)) return;
  float4 c = fb[id];
  const float L = luminance(c.x, c.y, c.z);
  if (!(L > 0.f)) return;
  const float scaled = (*exposure) * L / logavg;
  float Y = scaled / (1.f + scaled);
  if (isinf(Y) || isnan(Y) || Y < 0.000001f) Y = 0.f;
  const float X_ = 0.5893f * c.x + 0.1789f * c.y + 0.1831f * c.z;
  const float Y_ = 0.2904f * c.x + 0.6051f * c.y + 0.1045f * c.z;
  const float Z_ = 0.0000f * c.x + 0.0684f * c.y + 1.0202f * c.z;
  float x = 0.f, y = 0.f;
  const float XYZ = X_ + Y_ + Z_;
  if (!(XYZ < 1e-6f)) {
    const float s = 1.f / XYZ;
    x = X_ * s;
    y = Y_ * s;
  }
  const float X = y < 1e-6f ? 0.f : Y * (x / y);
  const float Z = y < 1e-6f ? 0.f : (Y * (1 - x - y)) / y;
  c.x = 1.967f * X - 0.548f * Y - 0.297f * Z;
  c.y = -0.955f * X + 1.938f * Y - 0.027f * Z;
  c.z = 0.064f * X - 0.130f * Y + 0.982f * Z;
  c.w = 1.f;
  const float ig = 1.f / (*gamma);
  c.x = powf(c.x, ig);
  c.y = powf(c.y, ig);
  c.z = powf(c.z, ig);
  fb[id] = c;
  argb[id] = argb_int(c.x, c.y, c.z, c.w);
}

// UpdateImage (Image.cl:1-27)
__global__ void k_update_image(const float4* accum, const float* fc, int* argb, const int* size, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*size, cap)) return;
  const float4 a = accum[id];
  float4 c = make_float4(a.x / fc[0], a.y / fc[0], a.z / fc[0], 1.f);
  if (luminance(c.x, c.y, c.z) > 0.f) {
    c.x = powf(c.x, 1.f / 2.2f);
    c.y = powf(c.y, 1.f / 2.2f);
    c.z = powf(c.z, 1.f / 2.2f);
    argb[id] = argb_int(c.x, c.y, c.z, c.w);
  }
}

// Kogge-Stone group scans (Util.cl:917-1043): localScanInteger / localScanFloat.
// The float variant reads through GET_FLOAT, which returns int (values are
// truncated), as the reference does; lane 0 reads aux[-1] = 0.
template <typename T, bool TRUNC>
__global__ void k_local_scan(const T* in, T* out, T* group_sum, const int* length) {
  extern __shared__ unsigned char sh_raw[];
  T* aux = reinterpret_cast<T*>(sh_raw) + 1;
  const int idl = threadIdx.x, idg = blockIdx.x * blockDim.x + threadIdx.x, ls = blockDim.x;
  const int n = *length;
  if (idl == 0) aux[-1] = (T)0;
  T v = idg < n ? in[idg] : (T)0;
  if (TRUNC) v = (T)(int)v;
  aux[idl] = v;
  __syncthreads();
  for (int off = 1; off < ls; off *= 2) {
    T t = (T)0;
    if (idl >= off) t = aux[idl - off];
    __syncthreads();
    if (idl >= off) aux[idl] = t + aux[idl];
    __syncthreads();
  }
  if (idl == ls - 1) group_sum[blockIdx.x] = aux[idl];
  const T o = aux[idl] > (T)0 ? aux[idl - 1] : aux[0];
  if (idg < n) out[idg] = o;
}
// groupScanInteger / groupScanFloat (global 1, local 1): sequential
template <typename T>
__global__ void k_group_scan(const T* group_sum, T* group_prefix, const int* ngroups) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  group_prefix[0] = (T)0;
  for (int i = 1; i < *ngroups; ++i) group_prefix[i] = group_prefix[i - 1] + group_sum[i - 1];
}
// globalScanInteger / globalScanFloat (the float one through int, as the reference)
template <typename T, bool TRUNC>
__global__ void k_global_scan(T* out, const T* group_prefix, const int* length) {
  const int idg = blockIdx.x * blockDim.x + threadIdx.x;
  if (idg >= *length) return;
  if (TRUNC) {
    const int v = (int)out[idg];
    const int s = (int)(group_prefix[blockIdx.x] + (T)v);
    out[idg] = (T)s;
  } else {
    out[idg] = group_prefix[blockIdx.x] + out[idg];
  }
}
// globalTotalInteger / globalTotalFloat
template <typename T>
__global__ void k_global_total(const T* in, const T* out, T* total, const int* length) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int n = *length;
  *total = n > 0 ? in[n - 1] + out[n - 1] : (T)0;
}

// identifyMeshLights / prepareLightInfo (LightConfiguration.cl:1-55)
__global__ void k_identify_lights(const Face* faces, const int* size, const Material* materials, int nmat,
                                  int* predicate, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*size, cap)) return;
  const int m = faces[id].mat & 0xFFFF;
  if (m >= nmat) {
    latch(err, kErrIndex);
    return;
  }
  predicate[id] = is_emitter(materials[m]) ? 1 : 0;
}
__global__ void k_prepare_lights(const int* predicate, const int* prefix, const int* total, RLight* lights, int lcap,
                                 int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*total, cap)) return;
  if (!predicate[id]) return;
  const int k = prefix[id];
  if (k < 0 || k >= lcap) {
    latch(err, kErrIndex);
    return;
  }
  lights[k].faceId = id;
  lights[k].type = 0;  // AREA_LIGHT
}

// Light grid (LightGrid.cl:347-423) on the LightGrid struct
__device__ __forceinline__ float* gv(GridHdr* g, int which) {
  return reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(g) + kGridHeader) + (size_t)which * kGridValues;
}
__global__ void k_grid_row_scan(GridHdr* g, int gsz) {  // prefixSumRowSubgrid, group = rx
  extern __shared__ float auxf[];
  const int idl = threadIdx.x, idg = blockIdx.x * blockDim.x + threadIdx.x;
  if (idg >= (int)kGridValues) return;
  auxf[idl] = gv(g, 1)[idg];
  __syncthreads();
  for (int off = 1; off < gsz; off *= 2) {
    float t = 0.f;
    if (idl >= off) t = auxf[idl - off];
    __syncthreads();
    if (idl >= off) auxf[idl] = t + auxf[idl];
    __syncthreads();
  }
  gv(g, 2)[idg] = auxf[idl];
}
__global__ void k_grid_col_scan(GridHdr* g, int gsz) {  // prefixSumColSubgrid, group = ry
  extern __shared__ float auxf[];
  const int idl = threadIdx.x;
  const int i = gsz * blockIdx.x;
  const int nu = g->nu, nv = g->nv;
  if (nu <= 0 || nv <= 0) return;
  const int xi = i / nv, yi = i % nv + idl;
  const long long index = (long long)xi + (long long)yi * nu;
  const bool ok = index >= 0 && index < (long long)kGridValues;
  auxf[idl] = ok ? gv(g, 2)[index] : 0.f;
  __syncthreads();
  for (int off = 1; off < gsz; off *= 2) {
    float t = 0.f;
    if (idl >= off) t = auxf[idl - off];
    __syncthreads();
    if (idl >= off) auxf[idl] = t + auxf[idl];
    __syncthreads();
  }
  if (ok) gv(g, 2)[index] = auxf[idl];
}
__global__ void k_grid_init(GridHdr* g, int which_mask, int copy_func) {  // initLightGrid / initFuncAndSat / calculateFunc
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= kGridValues) return;
  if (copy_func) {
    gv(g, 1)[id] = gv(g, 0)[id];
    return;
  }
  for (int w = 0; w < 3; ++w)
    if (which_mask & (1 << w)) gv(g, w)[id] = 0.f;
}

// ---------------------------------------------------------- preview device
// Raytrace.cl (CDeviceRT): unjittered camera rays, a BSDF per pixel, quick
// shading, the environment as background, the material group per pixel.

// InitCameraRayData (Raytrace.cl:1-31): no jitter, no length check
__global__ void k_rt_camera_rays(PassParams pp, RRay* rays, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  const int W = pp.width;
  const float px = (float)(id % W), py = (float)(id / W);
  V d = normalize4(mk(pp.cam_a * (2.f * px / pp.dim_w - 1.f), -2.f * py / pp.dim_h + 1.f, -pp.cam_d, 0.f));
  const float* m = pp.cam_m;
  V z = zero4();
  V m0 = mk(m[0], m[1], m[2], m[3]), m1 = mk(m[4], m[5], m[6], m[7]), m2 = mk(m[8], m[9], m[10], m[11]),
    m3 = mk(m[12], m[13], m[14], m[15]);
  V o = mk(dot3(m0, z) + m0.w, dot3(m1, z) + m1.w, dot3(m2, z) + m2.w, dot3(m3, z) + m3.w);
  if (!(o.w == 1.f)) o = mk(o.x / o.w, o.y / o.w, o.z / o.w, 0.f);
  o.w = 0.f;
  V dw = mk(dot4(m0, d), dot4(m1, d), dot4(m2, d), 0.f);
  init_ray(rays + id, o, dw, 0.001f, CUDART_INF_F);
}

// SetupBSDFRaytrace (Raytrace.cl:34-50): the whole Bsdf per pixel; an invalid
// one keeps materialID -1 with its material's parameters
__global__ void k_rt_setup_bsdf(const RIsect* isects, const RRay* rays, RBsdf* bsdfs, const Material* materials,
                                int nmat, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  const RIsect& is = isects[id];
  if (!is.hit) return;
  if (is.mat < 0 || is.mat >= nmat) {
    latch(err, kErrIndex);
    return;
  }
  DevScene S{};
  S.materials = materials;
  const Bsdf b = setup_bsdf(S, v4(rays[id].d), v4(is.n), is.mat);
  RBsdf& o = bsdfs[id];
  o.param = materials[is.mat];
  o.frame.mX = f4(b.frame.mX);
  o.frame.mY = f4(b.frame.mY);
  o.frame.mZ = f4(b.frame.mZ);
  o.localDirFix = f4(b.fix);
  o.localGeomN = f4(local_coord(b.frame, v4(is.ng)));
  o.materialID = b.mat;
  o.diffProb = b.pd;
  o.glossyProb = b.pg;
}

// textureInitPassRT / updateToTextureColorRT (Raytrace.cl:52-145)
__global__ void k_rt_texture_pass(const RBsdf* bsdfs, const RIsect* isects, RTex* tex, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  const RBsdf& b = bsdfs[id];
  if (is_emitter(b.param)) return;
  RTex* t = tex + id;
  t->parameters.x = b.materialID;
  const int ux = __float_as_int(isects[id].uv.x), uy = __float_as_int(isects[id].uv.y);
  t->diffuse = b.param.isDiffuseTexture ? make_int4(ux, uy, t->diffuse.z, 1) : make_int4(t->diffuse.x, t->diffuse.y, t->diffuse.z, 0);
  t->glossy = b.param.isGlossyTexture ? make_int4(ux, uy, t->glossy.z, 1) : make_int4(t->glossy.x, t->glossy.y, t->glossy.z, 0);
  t->roughness = b.param.isRoughnessTexture ? make_int4(ux, uy, t->roughness.z, 1)
                                            : make_int4(t->roughness.x, t->roughness.y, t->roughness.z, 0);
}
__global__ void k_rt_texture_color(RBsdf* bsdfs, const RTex* tex, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  Material& P = bsdfs[id].param;
  const RTex& t = tex[id];
  if (t.diffuse.w) P.diffuse_color = argb_float4(t.diffuse.z);
  if (t.glossy.w) P.glossy_color = argb_float4(t.glossy.z);
  if (t.roughness.w) {
    const float4 c = argb_float4(t.roughness.z);
    P.glossy_param.y = c.x;
    P.glossy_param.z = c.y;
  }
}

// getQuickSurfaceColor (Material.cl:33-43) packed by getIntARGB with w = 1
__device__ __forceinline__ int quick_argb(const Material& P, float coeff) {
  V c = is_emitter(P) ? v4(P.emission_color) : muls(v4(P.diffuse_color), coeff);
  return argb_int(c.x, c.y, c.z, 1.f);
}
// backgroundShade's colour (Raytrace.cl:175-204): the texel with gamma 2.2
__device__ __forceinline__ int background_argb(const float4* env, int w, int h, V d) {
  int x, y;
  sph_xy(w, h, d, &x, &y);
  const float4 e = env[sph_index(w, h, x, y)];
  const float ig = 1.f / 2.2f;
  return argb_int(powf(e.x, ig), powf(e.y, ig), powf(e.z, ig), e.w);
}

// fastShade (Raytrace.cl:147-173)
__global__ void k_rt_fast_shade(const RIsect* isects, const RBsdf* bsdfs, int* argb, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap || !isects[id].hit) return;
  argb[id] = quick_argb(bsdfs[id].param, bsdfs[id].localDirFix.z);
}
// backgroundShade (Raytrace.cl:175-204)
__global__ void k_rt_background(const RIsect* isects, int* argb, const RRay* rays, const float4* env,
                                const GridHdr* grid, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap || isects[id].hit) return;
  argb[id] = grid->isPresent ? background_argb(env, grid->width, grid->height, v4(rays[id].d))
                             : argb_int(0.f, 0.f, 0.f, 1.f);
}
// updateGroupbufferShadeImage (Raytrace.cl:206-220)
__global__ void k_rt_group(const RIsect* isects, int* group, int cap) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= cap) return;
  group[id] = isects[id].hit ? (isects[id].mat & 0xFFFF) : -1;
}
// findBound (Util.cl:830-884): bound of the faces whose material index is the
// group's; float min/max through ordered integer atomics (one atomic per lane)
__device__ __forceinline__ void atomic_min_f(float* a, float v) {
  if (v >= 0.f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
  if (v >= 0.f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__global__ void k_find_bound(const int* group, MeshArgs M, const int* size, float* bound, int cap, int* err) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= min(*size, cap)) return;
  if (!face_ok(M, id)) {
    latch(err, kErrIndex);
    return;
  }
  const Face& F = M.faces[id];
  if ((F.mat & 0xFFFF) != group[0]) return;
  const float4 p1 = M.points[F.vx], p2 = M.points[F.vy], p3 = M.points[F.vz];
  atomic_min_f(bound + 0, fminf(fminf(p1.x, p2.x), p3.x));
  atomic_min_f(bound + 1, fminf(fminf(p1.y, p2.y), p3.y));
  atomic_min_f(bound + 2, fminf(fminf(p1.z, p2.z), p3.z));
  atomic_max_f(bound + 3, fmaxf(fmaxf(p1.x, p2.x), p3.x));
  atomic_max_f(bound + 4, fmaxf(fmaxf(p1.y, p2.y), p3.y));
  atomic_max_f(bound + 5, fmaxf(fmaxf(p1.z, p2.z), p3.z));
}

}  // namespace plain
}  // namespace mt

// ------------------------------------------------------------------ host side
namespace {

using namespace mt::plain;

enum KernelId {
  kInitCameraRays, kInitPath, kInitIsect, kInitIndex, kInitInt, kInitFloat, kInitF4XYZ, kInitRGB,
  kIntersect, kSetupBsdf, kLightHit, kTexturePass, kTextureColor, kSampleBsdf, kDirectLight,
  kCompactAtomic, kTransferIsect, kTransferPixels,
  kAverageAccum, kUpdateFrameImage, kUpdateImage,
  kLocalScanInt, kGroupScanInt, kGlobalScanInt, kGlobalTotalInt,
  kLocalScanFloat, kGroupScanFloat, kGlobalScanFloat, kGlobalTotalFloat,
  kIdentifyLights, kPrepareLights,
  kGridRowScan, kGridColScan, kGridInit, kGridInitFuncSat, kGridCalcFunc,
  kRtCameraRays, kRtSetupBsdf, kRtTexturePass, kRtTextureColor, kRtFastShade, kRtBackground, kRtGroup, kFindBound,
  kTextureApply,
  kNumKernels
};

struct Spec {
  const char* name;
  int nargs;
};
// names and argument counts of the reference's __kernel functions
const Spec kSpecs[kNumKernels] = {
    {"InitCameraRayDataJitter", 4}, {"InitPathData", 2}, {"InitIntersection", 2}, {"InitIntDataToIndex", 2},
    {"InitIntData", 2}, {"InitFloatData", 2}, {"InitFloat4DataXYZ", 2}, {"InitIntDataRGB", 2},
    {"IntersectPrimitives", 10}, {"SetupBSDFPath", 6}, {"LightHitPass", 17}, {"texturePassGI", 5},
    {"updateToTextureColorGI", 4}, {"SampleBSDFRayDirection", 7}, {"DirectLight", 21},
    {"CompactAtomic", 6}, {"TransferIntersection", 3}, {"TransferPixels", 3},
    {"averageAccum", 6}, {"updateFrameImage", 7}, {"UpdateImage", 4},
    {"localScanInteger", 5}, {"groupScanInteger", 3}, {"globalScanInteger", 3}, {"globalTotalInteger", 4},
    {"localScanFloat", 5}, {"groupScanFloat", 3}, {"globalScanFloat", 3}, {"globalTotalFloat", 4},
    {"identifyMeshLights", 4}, {"prepareLightInfo", 4},
    {"prefixSumRowSubgrid", 2}, {"prefixSumColSubgrid", 2}, {"initLightGrid", 1}, {"initFuncAndSat", 1},
    {"calculateFunc", 1},
    {"InitCameraRayData", 2}, {"SetupBSDFRaytrace", 4}, {"textureInitPassRT", 3}, {"updateToTextureColorRT", 2},
    {"fastShade", 3}, {"backgroundShade", 6}, {"updateGroupbufferShadeImage", 3}, {"findBound", 7},
    {"textureApplyPass", 4},
};

std::string names_list() {
  std::string out;
  for (const Spec& sp : kSpecs) {
    if (!out.empty()) out += ",";
    out += sp.name;
  }
  return out;
}

}  // namespace

struct mt_kernel {
  mt_context* ctx = nullptr;
  int id = 0;
  std::vector<mt_buffer*> args;
  std::vector<size_t> local_bytes;
};

extern "C" const char* mt_kernel_names(void) {
  static const std::string names = names_list();
  return names.c_str();
}

extern "C" int mt_kernel_create(mt_context* ctx, const char* name, mt_kernel** out) {
  if (!ctx || !name || !out) return fail(MT_ERR_INVALID, "NULL argument");
  *out = nullptr;
  for (int i = 0; i < kNumKernels; ++i)
    if (std::strcmp(kSpecs[i].name, name) == 0) {
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      CU(cudaSetDevice(ctx->device));
      if (!ctx->d_plain_err) {
        int r = dalloc(&ctx->d_plain_err, 1);
        if (r) return r;
        CU(cudaMemset(ctx->d_plain_err, 0, 4));
      }
      auto* k = new mt_kernel();
      k->ctx = ctx;
      k->id = i;
      k->args.assign(kSpecs[i].nargs, nullptr);
      k->local_bytes.assign(kSpecs[i].nargs, 0);
      *out = k;
      return MT_OK;
    }
  return fail(MT_ERR_INVALID, "unknown kernel '%s' (known: %s)", name, mt_kernel_names());
}

extern "C" int mt_kernel_set_arg_buf(mt_kernel* k, int index, mt_buffer* buf) {
  if (!k || !buf) return fail(MT_ERR_INVALID, "NULL argument");
  if (index < 0 || index >= (int)k->args.size())
    return fail(MT_ERR_INVALID, "%s takes %d arguments, not index %d", kSpecs[k->id].name, (int)k->args.size(), index);
  if (buf->ctx != k->ctx) return fail(MT_ERR_INVALID, "buffer of another context");
  k->args[index] = buf;
  return MT_OK;
}

extern "C" int mt_kernel_set_arg_local(mt_kernel* k, int index, size_t bytes) {
  if (!k) return fail(MT_ERR_INVALID, "NULL kernel");
  if (index < 0 || index >= (int)k->args.size()) return fail(MT_ERR_INVALID, "argument index %d", index);
  k->local_bytes[index] = bytes;  // the kernels size their own shared memory from the group size
  return MT_OK;
}

extern "C" int mt_kernel_destroy(mt_kernel* k) {
  delete k;
  return MT_OK;
}

namespace {

template <class T>
T* ptr(mt_kernel* k, int i) {
  return static_cast<T*>(k->args[i]->ptr);
}
template <class T>
int count_of(mt_kernel* k, int i) {
  size_t n = k->args[i]->bytes / sizeof(T);
  return n > (size_t)INT32_MAX ? INT32_MAX : (int)n;
}

int read_host(mt_context* ctx, void* dst, const mt_buffer* b, size_t bytes) {
  if (b->bytes < bytes) return fail(MT_ERR_INVALID, "buffer of %zu B, %zu needed", b->bytes, bytes);
  CU(cudaMemcpyAsync(dst, b->ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return MT_OK;
}

MeshArgs mesh_args(mt_kernel* k, int points, int uvs, int normals, int faces, int materials) {
  MeshArgs m;
  m.points = ptr<float4>(k, points);
  m.uvs = ptr<float2>(k, uvs);
  m.normals = ptr<float4>(k, normals);
  m.faces = ptr<Face>(k, faces);
  m.materials = materials >= 0 ? ptr<Material>(k, materials) : nullptr;
  m.npoints = count_of<float4>(k, points);
  m.nfaces = count_of<Face>(k, faces);
  m.nmat = materials >= 0 ? count_of<Material>(k, materials) : 65536;
  m.nuvs = count_of<float2>(k, uvs);
  m.nnormals = count_of<float4>(k, normals);
  return m;
}

}  // namespace

extern "C" int mt_launch_1d(mt_kernel* k, size_t global, size_t local) {
  if (!k) return fail(MT_ERR_INVALID, "NULL kernel");
  for (size_t i = 0; i < k->args.size(); ++i)
    if (!k->args[i] && !k->local_bytes[i])
      return fail(MT_ERR_INVALID, "%s: argument %zu is not set", kSpecs[k->id].name, i);
  if (global == 0) return MT_OK;
  if (global > (size_t)INT32_MAX) return fail(MT_ERR_INVALID, "global size %zu", global);
  mt_context* ctx = k->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  join_jobs(ctx);
  cudaStream_t st = ctx->stream;
  int* err = ctx->d_plain_err;
  const int G = (int)global;
  const int T = 128;
  const unsigned B = (unsigned)((G + T - 1) / T);
  auto capn = [&](int i, size_t elem) { return std::min(G, (int)std::min<size_t>(k->args[i]->bytes / elem, INT32_MAX)); };
  auto grid_of = [&](int i) -> int {
    if (k->args[i]->bytes < kGridBytes) return fail(MT_ERR_INVALID, "LightGrid buffer of %zu B, %zu needed",
                                                     k->args[i]->bytes, kGridBytes);
    return MT_OK;
  };
  // the environment arrays must hold the width x height the LightGrid header names
  auto env_of_args = [&](int rgb, int lum, int sat, int grid) -> int {
    if (int r = grid_of(grid)) return r;
    GridHdr h;
    if (int r = read_host(ctx, &h, k->args[grid], sizeof(h))) return r;
    if (!h.isPresent) return MT_OK;
    const long long n = (long long)h.width * h.height;
    if (h.width <= 0 || h.height <= 0 || (size_t)n * 16 > k->args[rgb]->bytes || (size_t)n * 4 > k->args[lum]->bytes ||
        (size_t)n * 4 > k->args[sat]->bytes)
      return fail(MT_ERR_INVALID, "environment of %d x %d does not fit its buffers", h.width, h.height);
    return MT_OK;
  };
  switch (k->id) {
    case kInitCameraRays: {
      unsigned char cam[64];
      RState stt;
      int r = read_host(ctx, cam, k->args[0], 64);
      if (!r) r = read_host(ctx, &stt, k->args[2], sizeof(RState));
      if (r) return r;
      float dim[2];
      std::memcpy(dim, cam + 48, 8);
      const int W = (int)dim[0], H = (int)dim[1];
      if (W <= 0 || H <= 0) return fail(MT_ERR_INVALID, "camera dimension %g x %g", dim[0], dim[1]);
      PassParams pp{};
      camera_constants(cam, W, H, pp);
      pp.width = W;
      pp.height = H;
      pp.frame_count = stt.frameCount;
      pp.seeds[0] = stt.seed.x;
      pp.seeds[1] = stt.seed.y;
      k_init_camera_rays<<<B, T, 0, st>>>(pp, ptr<RRay>(k, 1), ptr<int>(k, 3), capn(1, sizeof(RRay)));
      break;
    }
    case kInitPath:
      k_init_path<<<B, T, 0, st>>>(ptr<RPath>(k, 0), ptr<int>(k, 1), capn(0, sizeof(RPath)));
      break;
    case kInitIsect:
      k_init_isect<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<int>(k, 1), capn(0, sizeof(RIsect)));
      break;
    case kInitIndex:
      k_fill_index<<<B, T, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), capn(0, 4));
      break;
    case kInitInt:
    case kInitFloat:
      k_fill_u32<<<B, T, 0, st>>>(ptr<unsigned>(k, 0), 0u, ptr<int>(k, 1), capn(0, 4));
      break;
    case kInitF4XYZ:
      k_fill_f4<<<B, T, 0, st>>>(ptr<float4>(k, 0), make_float4(0.f, 0.f, 0.f, 1.f), ptr<int>(k, 1), capn(0, 16));
      break;
    case kInitRGB:
      k_fill_u32<<<B, T, 0, st>>>(ptr<unsigned>(k, 0), 0xFF000000u, ptr<int>(k, 1), capn(0, 4));
      break;
    case kIntersect: {
      BvhArgs bv{ptr<RNode>(k, 8), ptr<RBound>(k, 9), count_of<RNode>(k, 8), count_of<RBound>(k, 9)};
      const int cap = std::min(capn(0, sizeof(RRay)), capn(1, sizeof(RIsect)));
      k_intersect<<<B, T, 0, st>>>(ptr<RRay>(k, 0), ptr<RIsect>(k, 1), ptr<int>(k, 2), cap,
                                   mesh_args(k, 3, 4, 5, 6, -1), bv, err);
      break;
    }
    case kSetupBsdf: {
      const int cap = std::min({capn(0, sizeof(RIsect)), capn(1, sizeof(RRay)), capn(4, 4)});
      k_setup_bsdf<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RRay>(k, 1), ptr<RPath>(k, 2), count_of<RPath>(k, 2),
                                    ptr<Material>(k, 3), count_of<Material>(k, 3), ptr<int>(k, 4), ptr<int>(k, 5),
                                    cap, err);
      break;
    }
    case kLightHit: {
      if (int r = env_of_args(13, 14, 15, 16)) return r;
      const int cap = std::min({capn(0, sizeof(RIsect)), capn(1, sizeof(RRay)), capn(11, 4)});
      EnvArgs A{ptr<float4>(k, 13), ptr<float>(k, 14), ptr<float>(k, 15), ptr<GridHdr>(k, 16)};
      k_light_hit<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RRay>(k, 1), ptr<RPath>(k, 2), count_of<RPath>(k, 2),
                                   ptr<int>(k, 3), mesh_args(k, 5, 6, 7, 8, 4), ptr<float4>(k, 10), ptr<int>(k, 11),
                                   ptr<int>(k, 12), cap, A, err);
      break;
    }
    case kTexturePass: {
      const int cap = std::min({capn(1, sizeof(RIsect)), capn(2, sizeof(RTex)), capn(3, 4)});
      k_texture_pass<<<B, T, 0, st>>>(ptr<RPath>(k, 0), count_of<RPath>(k, 0), ptr<RIsect>(k, 1), ptr<RTex>(k, 2),
                                      ptr<int>(k, 3), ptr<int>(k, 4), cap, err);
      break;
    }
    case kTextureApply: {
      if (k->args[1]->bytes < 4) return fail(MT_ERR_INVALID, "count buffer too small");
      long long ntexels = (long long)(k->args[2]->bytes / 4);
      k_texture_apply<<<B, T, 0, st>>>(ptr<RTex>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2), ntexels, ptr<int4>(k, 3),
                                       count_of<int4>(k, 3), capn(0, sizeof(RTex)), err);
      break;
    }
    case kTextureColor: {
      const int cap = std::min(capn(1, sizeof(RTex)), capn(2, 4));
      k_texture_color<<<B, T, 0, st>>>(ptr<RPath>(k, 0), count_of<RPath>(k, 0), ptr<RTex>(k, 1), ptr<int>(k, 2),
                                       ptr<int>(k, 3), cap, err);
      break;
    }
    case kSampleBsdf: {
      if (k->args[5]->bytes < sizeof(RState)) return fail(MT_ERR_INVALID, "State buffer too small");
      const int cap = std::min({capn(0, sizeof(RIsect)), capn(1, sizeof(RRay)), capn(4, 4)});
      k_sample_bsdf<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RRay>(k, 1), ptr<RPath>(k, 2), count_of<RPath>(k, 2),
                                     ptr<int>(k, 4), ptr<RState>(k, 5), ptr<int>(k, 6), cap, err);
      break;
    }
    case kDirectLight: {
      if (int r = env_of_args(17, 18, 19, 20)) return r;
      if (k->args[8]->bytes < sizeof(RState)) return fail(MT_ERR_INVALID, "State buffer too small");
      const int cap = std::min({capn(1, sizeof(RIsect)), capn(4, sizeof(RRay)), capn(6, 4)});
      BvhArgs bv{ptr<RNode>(k, 15), ptr<RBound>(k, 16), count_of<RNode>(k, 15), count_of<RBound>(k, 16)};
      EnvArgs A{ptr<float4>(k, 17), ptr<float>(k, 18), ptr<float>(k, 19), ptr<GridHdr>(k, 20)};
      k_direct_light<<<B, T, 0, st>>>(ptr<RPath>(k, 0), count_of<RPath>(k, 0), ptr<RIsect>(k, 1), ptr<RLight>(k, 2),
                                      count_of<RLight>(k, 2), ptr<int>(k, 3), ptr<RRay>(k, 4), ptr<float4>(k, 5),
                                      ptr<int>(k, 6), ptr<int>(k, 7), cap, ptr<RState>(k, 8),
                                      mesh_args(k, 10, 11, 12, 13, 9), bv, A, err);
      break;
    }
    case kCompactAtomic: {
      // CompactAtomic (Compact.cl:21-40) in the serial order: kept records and
      // their pixel ids at count, count + 1, ... (the stable compaction)
      int n = 0;
      if (int r = read_host(ctx, &n, k->args[5], 4)) return r;
      n = std::min({n, G, capn(0, sizeof(RIsect)), capn(1, sizeof(RIsect)), capn(2, 4), capn(3, 4)});
      if (n <= 0) break;
      const size_t tiles = ((size_t)n + kCompactThreads - 1) / kCompactThreads;
      if (tiles > ctx->cs_tiles) {
        dfree(ctx->cs_status);
        dfree(ctx->cs_words);
        ctx->cs_tiles = 0;
        int r = dalloc(&ctx->cs_status, tiles);
        if (!r) r = dalloc(&ctx->cs_words, 4);
        if (r) return r;
        ctx->cs_tiles = tiles;
      }
      const cudaError_t le = launch_compact_isects(st, ptr<void>(k, 0), ptr<int>(k, 2), n, ptr<void>(k, 1),
                                                   ptr<int>(k, 3), ptr<int>(k, 4),
                                                   CompactScratch{ctx->cs_status, ctx->cs_words});
      if (le != cudaSuccess) return fail(MT_ERR_CUDA, "compaction launch: %s", cudaGetErrorString(le));
      break;
    }
    case kTransferIsect:
      k_copy_isects<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RIsect>(k, 1), ptr<int>(k, 2),
                                     std::min(capn(0, sizeof(RIsect)), capn(1, sizeof(RIsect))));
      break;
    case kTransferPixels:
      k_copy_ints<<<B, T, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2), std::min(capn(0, 4), capn(1, 4)));
      break;
    case kAverageAccum: {
      const int cap = std::min({capn(0, 16), capn(2, 16), capn(3, 4), capn(4, 4)});
      k_average_accum<<<B, T, 0, st>>>(ptr<float4>(k, 0), ptr<float>(k, 1), ptr<float4>(k, 2), ptr<float>(k, 3),
                                       ptr<int>(k, 4), ptr<int>(k, 5), cap);
      break;
    }
    case kUpdateFrameImage: {
      const int cap = std::min(capn(0, 16), capn(1, 4));
      k_update_frame_image<<<B, T, 0, st>>>(ptr<float4>(k, 0), ptr<int>(k, 1), ptr<float>(k, 2), ptr<int>(k, 3),
                                            ptr<int>(k, 4), ptr<float>(k, 5), ptr<float>(k, 6), cap);
      break;
    }
    case kUpdateImage:
      k_update_image<<<B, T, 0, st>>>(ptr<float4>(k, 0), ptr<float>(k, 1), ptr<int>(k, 2), ptr<int>(k, 3),
                                      std::min(capn(0, 16), capn(2, 4)));
      break;
    case kLocalScanInt:
    case kLocalScanFloat: {
      // the group size is the scan's segment: the launch's local size (128 in PrefixSum*)
      const int L = (int)std::max<size_t>(1, std::min<size_t>(local ? local : 128, 1024));
      if (L & (L - 1)) return fail(MT_ERR_INVALID, "local size %d is not a power of two", L);
      const unsigned nb = (unsigned)((G + L - 1) / L);
      int len = 0;
      if (int r = read_host(ctx, &len, k->args[3], 4)) return r;
      if ((size_t)std::min(len, G) * 4 > std::min(k->args[0]->bytes, k->args[1]->bytes) ||
          (size_t)nb * 4 > k->args[2]->bytes)
        return fail(MT_ERR_INVALID, "scan buffers smaller than the launch");
      if (k->id == kLocalScanInt)
        k_local_scan<int, false><<<nb, L, (L + 1) * 4, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2),
                                                             ptr<int>(k, 3));
      else
        k_local_scan<float, true><<<nb, L, (L + 1) * 4, st>>>(ptr<float>(k, 0), ptr<float>(k, 1), ptr<float>(k, 2),
                                                              ptr<int>(k, 3));
      break;
    }
    case kGroupScanInt:
    case kGroupScanFloat: {
      int ng = 0;
      if (int r = read_host(ctx, &ng, k->args[2], 4)) return r;
      if ((size_t)std::max(ng, 0) * 4 > std::min(k->args[0]->bytes, k->args[1]->bytes))
        return fail(MT_ERR_INVALID, "group buffers smaller than %d groups", ng);
      if (k->id == kGroupScanInt)
        k_group_scan<int><<<1, 1, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2));
      else
        k_group_scan<float><<<1, 1, 0, st>>>(ptr<float>(k, 0), ptr<float>(k, 1), ptr<int>(k, 2));
      break;
    }
    case kGlobalScanInt:
    case kGlobalScanFloat: {
      const int L = (int)std::max<size_t>(1, std::min<size_t>(local ? local : 128, 1024));
      const unsigned nb = (unsigned)((G + L - 1) / L);
      int len = 0;
      if (int r = read_host(ctx, &len, k->args[2], 4)) return r;
      if ((size_t)std::min(len, G) * 4 > k->args[0]->bytes || (size_t)nb * 4 > k->args[1]->bytes)
        return fail(MT_ERR_INVALID, "scan buffers smaller than the launch");
      if (k->id == kGlobalScanInt)
        k_global_scan<int, false><<<nb, L, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2));
      else
        k_global_scan<float, true><<<nb, L, 0, st>>>(ptr<float>(k, 0), ptr<float>(k, 1), ptr<int>(k, 2));
      break;
    }
    case kGlobalTotalInt:
    case kGlobalTotalFloat: {
      int len = 0;
      if (int r = read_host(ctx, &len, k->args[3], 4)) return r;
      if (len > 0 && (size_t)len * 4 > std::min(k->args[0]->bytes, k->args[1]->bytes))
        return fail(MT_ERR_INVALID, "scan buffers smaller than the length %d", len);
      if (k->id == kGlobalTotalInt)
        k_global_total<int><<<1, 1, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2), ptr<int>(k, 3));
      else
        k_global_total<float><<<1, 1, 0, st>>>(ptr<float>(k, 0), ptr<float>(k, 1), ptr<float>(k, 2), ptr<int>(k, 3));
      break;
    }
    case kIdentifyLights:
      k_identify_lights<<<B, T, 0, st>>>(ptr<Face>(k, 0), ptr<int>(k, 1), ptr<Material>(k, 2),
                                         count_of<Material>(k, 2), ptr<int>(k, 3),
                                         std::min(capn(0, sizeof(Face)), capn(3, 4)), err);
      break;
    case kPrepareLights:
      k_prepare_lights<<<B, T, 0, st>>>(ptr<int>(k, 0), ptr<int>(k, 1), ptr<int>(k, 2), ptr<RLight>(k, 3),
                                        count_of<RLight>(k, 3), std::min(capn(0, 4), capn(1, 4)), err);
      break;
    case kGridRowScan:
    case kGridColScan: {
      if (int r = grid_of(0)) return r;
      const int L = (int)local;
      if (L < 1 || L > 1024 || (L & (L - 1))) return fail(MT_ERR_INVALID, "local size %zu", local);
      const unsigned nb = (unsigned)((std::min<size_t>(global, kGridValues) + L - 1) / L);
      if (k->id == kGridRowScan)
        k_grid_row_scan<<<nb, L, L * 4, st>>>(ptr<GridHdr>(k, 0), L);
      else
        k_grid_col_scan<<<nb, L, L * 4, st>>>(ptr<GridHdr>(k, 0), L);
      break;
    }
    case kGridInit:
    case kGridInitFuncSat:
    case kGridCalcFunc: {
      if (int r = grid_of(0)) return r;
      const unsigned nb = (unsigned)((std::min<size_t>(global, kGridValues) + 255) / 256);
      k_grid_init<<<nb, 256, 0, st>>>(ptr<GridHdr>(k, 0), k->id == kGridInit ? 7 : 6, k->id == kGridCalcFunc);
      break;
    }
    case kRtCameraRays: {
      unsigned char cam[64];
      if (int r = read_host(ctx, cam, k->args[0], 64)) return r;
      float dim[2];
      std::memcpy(dim, cam + 48, 8);
      const int W = (int)dim[0], H = (int)dim[1];
      if (W <= 0 || H <= 0) return fail(MT_ERR_INVALID, "camera dimension %g x %g", dim[0], dim[1]);
      PassParams pp{};
      camera_constants(cam, W, H, pp);
      pp.width = W;
      pp.height = H;
      k_rt_camera_rays<<<B, T, 0, st>>>(pp, ptr<RRay>(k, 1), capn(1, sizeof(RRay)));
      break;
    }
    case kRtSetupBsdf:
      k_rt_setup_bsdf<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RRay>(k, 1), ptr<RBsdf>(k, 2), ptr<Material>(k, 3),
                                       count_of<Material>(k, 3),
                                       std::min({capn(0, sizeof(RIsect)), capn(1, sizeof(RRay)), capn(2, sizeof(RBsdf))}),
                                       err);
      break;
    case kRtTexturePass:
      k_rt_texture_pass<<<B, T, 0, st>>>(ptr<RBsdf>(k, 0), ptr<RIsect>(k, 1), ptr<RTex>(k, 2),
                                         std::min({capn(0, sizeof(RBsdf)), capn(1, sizeof(RIsect)), capn(2, sizeof(RTex))}));
      break;
    case kRtTextureColor:
      k_rt_texture_color<<<B, T, 0, st>>>(ptr<RBsdf>(k, 0), ptr<RTex>(k, 1),
                                          std::min(capn(0, sizeof(RBsdf)), capn(1, sizeof(RTex))));
      break;
    case kRtFastShade:
      k_rt_fast_shade<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<RBsdf>(k, 1), ptr<int>(k, 2),
                                       std::min({capn(0, sizeof(RIsect)), capn(1, sizeof(RBsdf)), capn(2, 4)}));
      break;
    case kRtBackground: {
      if (int r = grid_of(5)) return r;
      GridHdr h;
      if (int r = read_host(ctx, &h, k->args[5], sizeof(h))) return r;
      if (h.isPresent && (h.width <= 0 || h.height <= 0 || (size_t)h.width * h.height * 16 > k->args[4]->bytes))
        return fail(MT_ERR_INVALID, "environment of %d x %d does not fit its buffer", h.width, h.height);
      k_rt_background<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<int>(k, 2), ptr<RRay>(k, 3), ptr<float4>(k, 4),
                                       ptr<GridHdr>(k, 5),
                                       std::min({capn(0, sizeof(RIsect)), capn(2, 4), capn(3, sizeof(RRay))}));
      break;
    }
    case kRtGroup:
      k_rt_group<<<B, T, 0, st>>>(ptr<RIsect>(k, 0), ptr<int>(k, 2), std::min(capn(0, sizeof(RIsect)), capn(2, 4)));
      break;
    case kFindBound:
      if (k->args[6]->bytes < 24) return fail(MT_ERR_INVALID, "group bound buffer holds 6 floats");
      k_find_bound<<<B, T, 0, st>>>(ptr<int>(k, 0), mesh_args(k, 1, 2, 3, 4, -1), ptr<int>(k, 5), ptr<float>(k, 6),
                                    capn(4, sizeof(Face)), err);
      break;
    default:
      return fail(MT_ERR_INVALID, "kernel id %d", k->id);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MT_ERR_CUDA, "%s launch: %s", kSpecs[k->id].name, cudaGetErrorString(e));
  return MT_OK;
}

