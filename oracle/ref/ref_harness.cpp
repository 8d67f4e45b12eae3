// Drives MambaTracer's own kernels (compiled as C++ through clshim.h) on the CPU.
// Test infrastructure only: the parity reference for the CPU restatement in
// oracle/ and for golden fixtures. Built into oracle/_ref/ by make_ref.py.
//
// Barrier-free kernels run one work-item after another in id order, which is
// a legal OpenCL schedule; for CompactAtomic (src/cl/kernel/Compact.cl:21-40)
// it is the stable order. Kernels with barrier() (the Kogge-Stone scans,
// src/cl/kernel/Util.cl:917-1043, src/cl/kernel/LightGrid.cl:347-400) run each
// work-group's items as fibers that yield at every barrier.
#include <ucontext.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <type_traits>
#include <vector>

#include "clshim.h"
#include "ref_tu.inc"
#undef A
#undef B
#undef C
#undef D
#undef E
#undef F
#undef W

namespace {

void set_item(int gid, int lid, int grp, int lsz, int gsz) {
  clshim::wi.global_id = gid;
  clshim::wi.local_id = lid;
  clshim::wi.group_id = grp;
  clshim::wi.local_size = lsz;
  clshim::wi.global_size = gsz;
  clshim::wi.barrier_fn = nullptr;
  clshim::wi.barrier_ctx = nullptr;
}

template <class F>
void run_serial(int nglobal, F&& body) {
  for (int id = 0; id < nglobal; ++id) {
    set_item(id, 0, 0, 1, nglobal);
    body();
  }
}

// --- fiber work-group executor ------------------------------------------
struct GroupExec {
  ucontext_t sched;
  std::vector<ucontext_t> ctx;
  std::vector<std::vector<char>> stacks;
  std::vector<char> done;
  std::function<void()> body;
  int cur = 0, nlocal = 0, group = 0, nglobal = 0;
};
GroupExec* g_exec = nullptr;

void fiber_yield(void*) {
  GroupExec* e = g_exec;
  swapcontext(&e->ctx[e->cur], &e->sched);
}

void fiber_entry() {
  GroupExec* e = g_exec;
  int l = e->cur;
  clshim::wi.global_id = e->group * e->nlocal + l;
  clshim::wi.local_id = l;
  clshim::wi.group_id = e->group;
  clshim::wi.local_size = e->nlocal;
  clshim::wi.global_size = e->nglobal;
  clshim::wi.barrier_fn = fiber_yield;
  e->body();
  e->done[l] = 1;
}

void run_groups(int nglobal, int nlocal, const std::function<void()>& body) {
  GroupExec e;
  e.nlocal = nlocal;
  e.nglobal = nglobal;
  e.body = body;
  e.ctx.resize(nlocal);
  e.stacks.assign(nlocal, std::vector<char>(256 * 1024));
  e.done.assign(nlocal, 0);
  g_exec = &e;
  for (int g = 0; g * nlocal < nglobal; ++g) {
    e.group = g;
    for (int l = 0; l < nlocal; ++l) {
      e.done[l] = 0;
      getcontext(&e.ctx[l]);
      e.ctx[l].uc_stack.ss_sp = e.stacks[l].data();
      e.ctx[l].uc_stack.ss_size = e.stacks[l].size();
      e.ctx[l].uc_link = &e.sched;
      makecontext(&e.ctx[l], fiber_entry, 0);
    }
    bool all_done = false;
    while (!all_done) {
      all_done = true;
      for (int l = 0; l < nlocal; ++l) {
        if (e.done[l]) continue;
        e.cur = l;
        swapcontext(&e.sched, &e.ctx[l]);
        // barrier: every item must have reached it (or finished) before any resumes
        if (!e.done[l]) all_done = false;
      }
    }
  }
  g_exec = nullptr;
  set_item(0, 0, 0, 1, 1);
}

LightGrid* new_light_grid() {
  LightGrid* g = static_cast<LightGrid*>(std::calloc(1, sizeof(LightGrid)));
  // defaults of src/cl/struct/CLightGrid.java:331-342
  g->nu = 1600;
  g->nv = 1600;
  g->subgridRangeX = 16;
  g->subgridRangeY = 32;
  return g;
}

// Texture images for ref_render_frame: an ARGB texel pool and 4 entries per
// material (first texel, width, height, 0) for diffuse, glossy, roughness,
// mirror; width 0 = no image.
struct RefTextures {
  const int* texels = nullptr;
  const int* ref = nullptr;
  int nref = 0;
};
RefTextures g_ref_tex;

// Java's (int) cast of a float: NaN -> 0, saturating at the int range.
int jcast(float x) {
  if (x != x) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return -2147483647 - 1;
  return (int)x;
}

// CTextureApplyPass.process (src/cl/algorithms/CTextureApplyPass.java:37-92),
// the Java host pass between texturePassGI and updateToTextureColorGI, with
// TextureInfoCache.getDomainValue (TextureInfoCache.java:131-136). The texel
// index is clamped to the image where Java's PixelReader would throw.
void texture_apply_process(TextureData* tex, int count, const RefTextures& T) {
  auto dom = [](float x) { return x < 0 ? x - (float)jcast(x) + 1 : x - (float)jcast(x); };
  for (int index = 0; index < count; ++index) {
    TextureData& t = tex[index];
    int4* kinds[3] = {&t.diffuseTexture, &t.glossyTexture, &t.roughnessTexture};
    for (int k = 0; k < 3; ++k) {
      if (!(kinds[k]->w > 0)) continue;
      const int entry = 4 * t.parameters.x + k;
      if (t.parameters.x < 0 || entry >= T.nref) continue;
      const int* r = T.ref + 4 * (size_t)entry;
      if (r[1] <= 0) continue;  // image == null
      float x, y;
      std::memcpy(&x, &kinds[k]->x, 4);
      std::memcpy(&y, &kinds[k]->y, 4);
      x = dom(x);
      y = dom(y);
      float dx = (float)x * ((float)r[1] - 1);
      float dy = (float)y * ((float)r[2] - 1);
      int ix = std::min(std::max(jcast(dx), 0), r[1] - 1), iy = std::min(std::max(jcast(dy), 0), r[2] - 1);
      kinds[k]->z = T.texels[r[0] + (size_t)iy * r[1] + ix];
    }
  }
}

}  // namespace

extern "C" {

int ref_sizeof(int which) {
  switch (which) {
    case 0: return (int)sizeof(Ray);
    case 1: return (int)sizeof(Intersection);
    case 2: return (int)sizeof(BVHNode);
    case 3: return (int)sizeof(BoundingBox);
    case 4: return (int)sizeof(Face);
    case 5: return (int)sizeof(Material);
    case 6: return (int)sizeof(Bsdf);
    case 7: return (int)sizeof(Path);
    case 8: return (int)sizeof(TextureData);
    case 9: return (int)sizeof(State);
    case 10: return (int)sizeof(CameraStruct);
    case 11: return (int)sizeof(LightInfo);
    case 12: return (int)sizeof(LightGrid);
    default: return -1;
  }
}

// IntersectPrimitives (NormalBVH.cl:94-233) over `launch` work-items with *count = count.
void ref_intersect(void* rays, void* isects, int count, int launch, const float* points,
                   const float* uvs, const float* normals, const int* faces, int nfaces,
                   const int* nodes, const float* bounds) {
  int cnt = count, size = nfaces;
  run_serial(launch, [&] {
    IntersectPrimitives((Ray*)rays, (Intersection*)isects, &cnt, (const float4*)points,
                        (const float2*)uvs, (const float4*)normals, (const Face*)faces, &size,
                        (const BVHNode*)nodes, (const BoundingBox*)bounds);
  });
}

// testOcclusion (NormalBVH.cl:235-317), the shadow test DirectLight calls.
void ref_occlusion(void* rays, int* occluded, int count, const float* points, const float* uvs,
                   const float* normals, const int* faces, int nfaces, const int* nodes,
                   const float* bounds) {
  TriangleMesh mesh = {(const float4*)points, (const float2*)uvs, (const float4*)normals,
                       (const Face*)faces, nfaces};
  for (int i = 0; i < count; ++i) {
    set_item(i, 0, 0, 1, count);
    occluded[i] = testOcclusion((Ray*)rays + i, mesh, (const BVHNode*)nodes,
                                (const BoundingBox*)bounds)
                      ? 1
                      : 0;
  }
}

// InitCameraRayDataJitter (Initialize.cl:129-172).
void ref_raygen(const void* camera, void* rays, const int* seed, float frame_count, int length) {
  State st;
  std::memset(&st, 0, sizeof(st));
  st.seed.x = seed[0];
  st.seed.y = seed[1];
  st.frameCount = frame_count;
  int len = length;
  CameraStruct cam = *(const CameraStruct*)camera;
  run_serial(length, [&] { InitCameraRayDataJitter(&cam, (Ray*)rays, &st, &len); });
}

// WangHash / generate_seed / get_random (Sampling.cl:15-59): n draws for work-item gid.
void ref_random(const int* seed, float frame_count, int gid, int n, float* out) {
  State st;
  std::memset(&st, 0, sizeof(st));
  st.seed.x = seed[0];
  st.seed.y = seed[1];
  st.frameCount = frame_count;
  set_item(gid, 0, 0, 1, gid + 1);
  int2 s = generate_seed(&st);
  for (int i = 0; i < n; ++i) out[i] = get_random(&s);
}

unsigned int ref_wanghash(int seed) { return WangHash(seed); }

// Mesh-light list: identifyMeshLights + PrefixSumInteger + prepareLightInfo
// (CLightConfiguration.java:43-87). Returns the light count.
int ref_light_list(const int* faces, int nfaces, const float* materials, int* light_info /*2*nfaces*/) {
  int size = nfaces;
  std::vector<int> predicate(nfaces, 0), prefix(nfaces, 0);
  const int nlocal = 100;
  int nglobal = ((nfaces + nlocal - 1) / nlocal) * nlocal;
  run_serial(nglobal, [&] {
    identifyMeshLights((const Face*)faces, &size, (Material*)materials, predicate.data());
  });
  // PrefixSumInteger.java:80-88 with LOCALSIZE 128
  const int lsz = 128;
  int gsz = ((nfaces + lsz - 1) / lsz) * lsz;
  int groups = gsz / lsz;
  std::vector<int> group_sum(groups, 0), group_prefix(groups, 0), aux(lsz + 1, 0);
  int len = nfaces, gcount = groups, total = 0;
  run_groups(gsz, lsz, [&] {
    localScanInteger(predicate.data(), prefix.data(), group_sum.data(), &len, aux.data() + 1);
  });
  run_serial(1, [&] { groupScanInteger(group_sum.data(), group_prefix.data(), &gcount); });
  for (int g = 0; g < groups; ++g) {
    for (int l = 0; l < lsz; ++l) {
      set_item(g * lsz + l, l, g, lsz, gsz);
      globalScanInteger(prefix.data(), group_prefix.data(), &len);
    }
  }
  run_serial(1, [&] { globalTotalInteger(predicate.data(), prefix.data(), &total, &len); });
  if (total > 0) {
    run_serial(nglobal, [&] {
      prepareLightInfo(predicate.data(), prefix.data(), &size, (LightInfo*)light_info);
    });
  }
  return total;
}

// PrefixSumInteger (PrefixSumInteger.java:80-88) on an arbitrary int array.
int ref_scan_int(const int* in, int n, int* out, int lsz) {
  int gsz = ((n + lsz - 1) / lsz) * lsz;
  int groups = gsz / lsz;
  std::vector<int> data(in, in + n), group_sum(groups, 0), group_prefix(groups, 0), aux(lsz + 1, 0);
  int len = n, gcount = groups, total = 0;
  run_groups(gsz, lsz, [&] {
    localScanInteger(data.data(), out, group_sum.data(), &len, aux.data() + 1);
  });
  run_serial(1, [&] { groupScanInteger(group_sum.data(), group_prefix.data(), &gcount); });
  for (int g = 0; g < groups; ++g)
    for (int l = 0; l < lsz; ++l) {
      set_item(g * lsz + l, l, g, lsz, gsz);
      globalScanInteger(out, group_prefix.data(), &len);
    }
  run_serial(1, [&] { globalTotalInteger(data.data(), out, &total, &len); });
  return total;
}

// InitEnvironmentLum + InitEnvironmentSAT (Initialize.cl:100-127): luminance and
// the serial FP32 inclusive SAT (SAT.cl:113-133, :304-311) of an env map.
void ref_env_lum_sat(const float* envmap, int w, int h, float* lum, float* sat) {
  EnvironmentGrid* eg = static_cast<EnvironmentGrid*>(std::calloc(1, sizeof(EnvironmentGrid)));
  eg->width = w;
  eg->height = h;
  run_serial(w * h, [&] { InitEnvironmentLum((float4*)envmap, lum, sat, eg); });
  run_serial(1, [&] { InitEnvironmentSAT(eg, sat); });
  std::free(eg);
}

// sampleContinuous (SAT.cl:313-323) over a region of a full-map SAT.
void ref_sat_sample(const float* sat, const float* func, const int* region6, float u0, float u1,
                    float* uv, int* offset, float* pdf) {
  SATRegion r;
  r.nu = region6[0];
  r.nv = region6[1];
  r.minX = region6[2];
  r.minY = region6[3];
  r.strideX = region6[4];
  r.strideY = region6[5];
  sampleContinuous(r, u0, u1, uv, offset, pdf, (float*)sat, (float*)func);
}

void ref_sat_sample_discrete(const float* sat, const float* func, const int* region6, float u0,
                             float u1, int* offset, float* pdf) {
  SATRegion r;
  r.nu = region6[0];
  r.nv = region6[1];
  r.minX = region6[2];
  r.minY = region6[3];
  r.strideX = region6[4];
  r.strideY = region6[5];
  sampleDiscrete(r, u0, u1, offset, pdf, (float*)sat, (float*)func);
}

float ref_sat_pdf(const float* sat, const float* func, const int* region6, int x, int y) {
  SATRegion r;
  r.nu = region6[0];
  r.nv = region6[1];
  r.minX = region6[2];
  r.minY = region6[3];
  r.strideX = region6[4];
  r.strideY = region6[5];
  return getPdfSAT(r, x, y, (float*)sat, (float*)func);
}

// Full-map environment light: illuminateEnvironmentLight (Light.cl:195-227) and
// getRadianceEnvironmentLight (Light.cl:270-286).
void ref_env_illuminate(const float* envmap, const float* lum, const float* sat, int w, int h,
                        const float* sample4, float* dir_out, float* pdf_out, float* contrib_out) {
  LightGrid* lg = new_light_grid();
  lg->isPresent = true;
  lg->width = w;
  lg->height = h;
  EnvironmentLight el = getEnvironmentLight(lg, (float4*)envmap, (float*)lum, (float*)sat);
  float4 s = clv_float4(sample4[0], sample4[1], sample4[2], sample4[3]);
  float4 p = clv_float4(0.f);
  float4 dir;
  float dist = 0, pdf = 0, lumv = 0;
  int idx = 0;
  float4 c = illuminateEnvironmentLight(el, p, s, &dir, &dist, &pdf, &lumv, &idx);
  std::memcpy(dir_out, &dir, 16);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
  std::free(lg);
}

void ref_env_radiance(const float* envmap, const float* lum, const float* sat, int w, int h,
                      const float* dir4, float* pdf_out, float* contrib_out) {
  LightGrid* lg = new_light_grid();
  lg->isPresent = true;
  lg->width = w;
  lg->height = h;
  EnvironmentLight el = getEnvironmentLight(lg, (float4*)envmap, (float*)lum, (float*)sat);
  float4 d = clv_float4(dir4[0], dir4[1], dir4[2], dir4[3]);
  float pdf = 0;
  float4 c = getRadianceEnvironmentLight(el, d, clv_float4(0.f), &pdf);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
  std::free(lg);
}

// Grid versions of the environment light: illuminateEnvironmentLight1 and
// getRadianceEnvironmentLight1 (Light.cl:140-268) on a grid whose func and SAT
// are given, camera at cam4, shading point p4. The radiance call's
// accumLightGrid is read back as the one accumulation entry it touched.
void ref_env_grid_illuminate(const float* envmap, const float* lum, const float* sat, int w, int h,
                             const float* gfunc, const float* gsat, int nu, int nv, int rx, int ry,
                             const float* cam4, const float* p4, const float* sample4, float* dir_out,
                             float* pdf_out, float* contrib_out, float* lum_out, int* gidx_out) {
  LightGrid* lg = new_light_grid();
  lg->isPresent = true;
  lg->width = w;
  lg->height = h;
  lg->nu = nu;
  lg->nv = nv;
  lg->subgridRangeX = rx;
  lg->subgridRangeY = ry;
  lg->cameraPosition = clv_float4(cam4[0], cam4[1], cam4[2], cam4[3]);
  std::memcpy(lg->func, gfunc, sizeof(float) * (size_t)nu * nv);
  std::memcpy(lg->sat, gsat, sizeof(float) * (size_t)nu * nv);
  EnvironmentLight el = getEnvironmentLight(lg, (float4*)envmap, (float*)lum, (float*)sat);
  float4 s = clv_float4(sample4[0], sample4[1], sample4[2], sample4[3]);
  float4 p = clv_float4(p4[0], p4[1], p4[2], p4[3]);
  float4 dir;
  float dist = 0, pdf = 0, lumv = 0;
  int idx = 0;
  float4 c = illuminateEnvironmentLight1(el, p, s, &dir, &dist, &pdf, &lumv, &idx);
  std::memcpy(dir_out, &dir, 16);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
  *lum_out = lumv;
  *gidx_out = idx;
  std::free(lg);
}

void ref_env_grid_radiance(const float* envmap, const float* lum, const float* sat, int w, int h,
                           const float* gfunc, const float* gsat, int nu, int nv, int rx, int ry, const float* cam4,
                           const float* p4, const float* dir4, float* pdf_out, float* contrib_out, int* gidx_out,
                           float* accum_out) {
  LightGrid* lg = new_light_grid();
  lg->isPresent = true;
  lg->width = w;
  lg->height = h;
  lg->nu = nu;
  lg->nv = nv;
  lg->subgridRangeX = rx;
  lg->subgridRangeY = ry;
  lg->cameraPosition = clv_float4(cam4[0], cam4[1], cam4[2], cam4[3]);
  std::memcpy(lg->func, gfunc, sizeof(float) * (size_t)nu * nv);
  std::memcpy(lg->sat, gsat, sizeof(float) * (size_t)nu * nv);
  EnvironmentLight el = getEnvironmentLight(lg, (float4*)envmap, (float*)lum, (float*)sat);
  float4 d = clv_float4(dir4[0], dir4[1], dir4[2], dir4[3]);
  float4 p = clv_float4(p4[0], p4[1], p4[2], p4[3]);
  float pdf = 0;
  float4 c = getRadianceEnvironmentLight1(el, d, p, &pdf);
  *pdf_out = pdf;
  std::memcpy(contrib_out, &c, 16);
  *gidx_out = -1;
  *accum_out = 0.f;
  for (size_t i = 0; i < (size_t)nu * nv; ++i)
    if (lg->accum[i] != 0.f) {
      *gidx_out = (int)i;
      *accum_out = lg->accum[i];
    }
  std::free(lg);
}

// CImage.processImage's per-pixel kernels (Image.cl:29-118): averageAccum
// (frame buffer, log luminance and its predicate per pixel) and
// updateFrameImage with given totals (the reference computes them with its
// float prefix sum, whose defects are left out here).
void ref_average_accum(const float* accum, float frame_count, int n, float* framebuf_out, float* loglw_out,
                       int* count_out) {
  float fc = frame_count;
  int len = n;
  run_serial(n, [&] {
    averageAccum((float4*)accum, &fc, (float4*)framebuf_out, loglw_out, count_out, &len);
  });
}

void ref_update_frame_image(float* framebuf, int* argb, float total_log, int total_number, int n, float exposure,
                            float gamma) {
  int len = n;
  float tl = total_log, ex = exposure, ga = gamma;
  int tn = total_number;
  run_serial(n, [&] { updateFrameImage((float4*)framebuf, argb, &tl, &tn, &len, &ex, &ga); });
}

// The preview device's frame (CDeviceRT.loop, src/cl/device/CDeviceRT.java:176-197):
// InitCameraRayData, IntersectPrimitives, SetupBSDFRaytrace, backgroundShade,
// fastShade, updateGroupbufferShadeImage (Raytrace.cl) without the texture pass.
void ref_preview(const void* camera, int width, int height, const float* points, const float* uvs,
                 const float* normals, const int* faces, int nfaces, const float* materials, const int* nodes,
                 const float* bounds, const float* envmap, int ew, int eh, int env_present, int* argb, int* group) {
  CameraStruct cam = *(const CameraStruct*)camera;
  cam.dimension.x = (float)width;
  cam.dimension.y = (float)height;
  const int n = width * height;
  std::vector<Ray> rays(n);
  std::vector<Intersection> isects(n);
  std::vector<Bsdf> bsdfs(n);
  int count = n, size = nfaces;
  LightGrid* lg = new_light_grid();
  lg->isPresent = env_present != 0;
  lg->width = ew;
  lg->height = eh;
  run_serial(n, [&] { InitCameraRayData(&cam, rays.data()); });
  run_serial(n, [&] {
    IntersectPrimitives(rays.data(), isects.data(), &count, (float4*)points, (float2*)uvs, (float4*)normals,
                        (Face*)faces, &size, (BVHNode*)nodes, (BoundingBox*)bounds);
  });
  run_serial(n, [&] { SetupBSDFRaytrace(isects.data(), rays.data(), bsdfs.data(), (Material*)materials); });
  if (g_ref_tex.nref > 0) {  // the texture pass of CDeviceRT.loop (CDeviceRT.java:179-182)
    std::vector<TextureData> texd(n);
    std::memset(texd.data(), 0, sizeof(TextureData) * (size_t)n);
    run_serial(n, [&] { textureInitPassRT(bsdfs.data(), isects.data(), texd.data()); });
    texture_apply_process(texd.data(), n, g_ref_tex);
    run_serial(n, [&] { updateToTextureColorRT(bsdfs.data(), texd.data()); });
  }
  run_serial(n, [&] { backgroundShade(isects.data(), &cam, argb, rays.data(), (float4*)envmap, lg); });
  run_serial(n, [&] { fastShade(isects.data(), bsdfs.data(), argb); });
  run_serial(n, [&] { updateGroupbufferShadeImage(isects.data(), &cam, group); });
  std::free(lg);
}

// Light-grid per-cell SAT: prefixSumRowSubgrid then prefixSumColSubgrid
// (LightGrid.cl:347-400), launched as CAdaptiveEnvironment.java:86-87 does.
void ref_lightgrid_sat(const float* func, float* sat_out, int nu, int nv, int rx, int ry) {
  LightGrid* lg = new_light_grid();
  lg->nu = nu;
  lg->nv = nv;
  lg->subgridRangeX = rx;
  lg->subgridRangeY = ry;
  std::memcpy(lg->func, func, sizeof(float) * (size_t)nu * nv);
  std::vector<float> aux(64 + 1, 0.f);
  run_groups(nu * nv, rx, [&] { prefixSumRowSubgrid(lg, aux.data() + 1); });
  run_groups(nu * nv, ry, [&] { prefixSumColSubgrid(lg, aux.data() + 1); });
  std::memcpy(sat_out, lg->sat, sizeof(float) * (size_t)nu * nv);
  std::free(lg);
}

// sampleSubgridContinuous / getSubgridPdfContinuous (LightGrid.cl:310-343) of cell `cell`
// on a grid whose func and SAT are given.
void ref_lightgrid_sample(const float* func, const float* sat, int nu, int nv, int rx, int ry,
                          int cell, float u0, float u1, float* uv, int* offset, float* pdf) {
  LightGrid* lg = new_light_grid();
  lg->nu = nu;
  lg->nv = nv;
  lg->subgridRangeX = rx;
  lg->subgridRangeY = ry;
  std::memcpy(lg->func, func, sizeof(float) * (size_t)nu * nv);
  std::memcpy(lg->sat, sat, sizeof(float) * (size_t)nu * nv);
  sampleSubgridContinuous(lg, cell, u0, u1, uv, offset, pdf);
  std::free(lg);
}

int ref_lightgrid_global_index(int nu, int nv, int rx, int ry, int cell, int lx, int ly) {
  LightGrid* lg = new_light_grid();
  lg->nu = nu;
  lg->nv = nv;
  lg->subgridRangeX = rx;
  lg->subgridRangeY = ry;
  int r = globalIndexInSubgrid(lg, cell, lx, ly);
  std::free(lg);
  return r;
}

// setupBsdf + SampleBsdf / EvaluateBsdf (Bsdf.cl:130-160, :525-606) for one
// shading point: n, ng, ray direction d (float4 each), material (144 B).
int ref_bsdf_sample(const float* material, const float* n, const float* ng, const float* d,
                    const float* sample3, float* dir_out, float* pdf_out, float* cos_out,
                    float* factor_out, float* probs_out) {
  Ray ray;
  std::memset(&ray, 0, sizeof(ray));
  std::memcpy(&ray.d, d, 16);
  Intersection is;
  std::memset(&is, 0, sizeof(is));
  std::memcpy(&is.n, n, 16);
  std::memcpy(&is.ng, ng, 16);
  is.mat = 0;
  Bsdf b = setupBsdf(&ray, &is, (Material*)material);
  if (isBsdfInvalid(b)) return 0;
  float3 s = clv_float3(sample3[0], sample3[1], sample3[2]);
  float4 dir = clv_float4(0.f);
  float pdf = 0, cosg = 0;
  float4 f = SampleBsdf(b, s, &dir, &pdf, &cosg);
  std::memcpy(dir_out, &dir, 16);
  *pdf_out = pdf;
  *cos_out = cosg;
  std::memcpy(factor_out, &f, 16);
  probs_out[0] = b.probabilities.diffProb;
  probs_out[1] = b.probabilities.glossyProb;
  return 1;
}

int ref_bsdf_eval(const float* material, const float* n, const float* ng, const float* d,
                  const float* wgen, float* pdf_out, float* cos_out, float* factor_out) {
  Ray ray;
  std::memset(&ray, 0, sizeof(ray));
  std::memcpy(&ray.d, d, 16);
  Intersection is;
  std::memset(&is, 0, sizeof(is));
  std::memcpy(&is.n, n, 16);
  std::memcpy(&is.ng, ng, 16);
  is.mat = 0;
  Bsdf b = setupBsdf(&ray, &is, (Material*)material);
  if (isBsdfInvalid(b)) return 0;
  float4 w = clv_float4(wgen[0], wgen[1], wgen[2], wgen[3]);
  float pdf = 0, cosg = 0;
  float4 f = EvaluateBsdf(b, w, &pdf, &cosg);
  *pdf_out = pdf;
  *cos_out = cosg;
  std::memcpy(factor_out, &f, 16);
  return 1;
}

// Textures for ref_render_frame (NULL / 0 entries: none, and the texture pass
// is skipped).
void ref_set_textures(const int* texels, const int* tex_ref, int nentries) {
  g_ref_tex.texels = texels;
  g_ref_tex.ref = tex_ref;
  g_ref_tex.nref = texels && tex_ref ? nentries : 0;
}

// The texture pass on one path: a Path whose Bsdf holds `material` (144 B) and
// material id `mat`, an Intersection with uv (u, v), through texturePassGI,
// CTextureApplyPass.process and updateToTextureColorGI; the Bsdf's parameters
// after the pass go to material_out.
void ref_texture_apply(const float* material, int mat, float u, float v, const int* texels, const int* tex_ref,
                       int nentries, float* material_out) {
  Path path;
  Intersection isect;
  TextureData tex;
  std::memset(&path, 0, sizeof(path));
  std::memset(&isect, 0, sizeof(isect));
  std::memset(&tex, 0, sizeof(tex));
  std::memcpy(&path.bsdf.param, material, sizeof(SurfaceParameter));
  path.bsdf.materialID = mat;
  isect.uv.x = u;
  isect.uv.y = v;
  int pixel = 0, count = 1;
  RefTextures T{texels, tex_ref, nentries};
  run_serial(1, [&] { texturePassGI(&path, &isect, &tex, &pixel, &count); });
  texture_apply_process(&tex, count, T);
  run_serial(1, [&] { updateToTextureColorGI(&path, &tex, &pixel, &count); });
  std::memcpy(material_out, &path.bsdf.param, sizeof(SurfaceParameter));
}

// One progressive GI frame, restating CDeviceGI.loop (CDeviceGI.java:214-271):
// raygen and path/queue init, then `max_depth` bounces of IntersectPrimitives,
// SetupBSDFPath, LightHitPass, CCompact.execute (CCompact.java:79-89), the
// texture pass (when textures are set), DirectLight, SampleBSDFRayDirection.
// seeds: the State seed pair of each allocateState() call in launch order
// (1 + 2*max_depth pairs). Film accumulates into accum (float4 per pixel).
// counts_out[b] = live queue length after bounce b's compaction.
int ref_render_frame(const void* camera, int width, int height, int max_depth, const int* seeds,
                     float frame_count, const float* points, const float* uvs,
                     const float* normals, const int* faces, int nfaces, const float* materials,
                     const int* nodes, const float* bounds, const float* envmap,
                     const float* env_lum, const float* env_sat, int env_w, int env_h,
                     int env_present, float* accum, int* counts_out) {
  const int N = width * height;
  CameraStruct cam = *(const CameraStruct*)camera;
  cam.dimension.x = (float)width;
  cam.dimension.y = (float)height;

  std::vector<Ray> rays(N), occl(N);
  std::vector<Intersection> isects(N), tmp_isects(N);
  std::vector<Path> paths(N);
  std::vector<int> pixels(N), tmp_pixels(N);
  std::vector<TextureData> texd(N);
  std::memset(texd.data(), 0, sizeof(TextureData) * (size_t)N);
  int length = N, count = N, size = nfaces;

  // lights (CDeviceGI.initLight, CDeviceGI.java:293-306)
  std::vector<int> linfo(2 * (nfaces > 0 ? nfaces : 1), 0);
  int total_lights = ref_light_list(faces, nfaces, materials, linfo.data());

  LightGrid* lg = new_light_grid();
  lg->isPresent = env_present ? true : false;
  lg->width = env_w;
  lg->height = env_h;
  lg->cameraPosition = cam.position;

  State st;
  std::memset(&st, 0, sizeof(st));
  int k = 0;
  auto allocate_state = [&] {
    st.seed.x = seeds[2 * k];
    st.seed.y = seeds[2 * k + 1];
    st.frameCount = frame_count;
    ++k;
  };

  const float4* P = (const float4*)points;
  const float2* UV = (const float2*)uvs;
  const float4* NN = (const float4*)normals;
  const Face* FF = (const Face*)faces;
  Material* M = (Material*)materials;
  const BVHNode* ND = (const BVHNode*)nodes;
  const BoundingBox* BD = (const BoundingBox*)bounds;
  float4* ACC = (float4*)accum;

  allocate_state();
  run_serial(N, [&] { InitCameraRayDataJitter(&cam, rays.data(), &st, &length); });
  run_serial(N, [&] { InitPathData(paths.data(), &length); });
  run_serial(N, [&] { InitIntersection(isects.data(), &length); });
  run_serial(N, [&] { InitIntDataToIndex(pixels.data(), &length); });
  count = N;
  for (int pathLength = 1; pathLength <= max_depth; ++pathLength) {
    run_serial(N, [&] {
      IntersectPrimitives(rays.data(), isects.data(), &count, P, UV, NN, FF, &size, ND, BD);
    });
    allocate_state();
    run_serial(N, [&] { SetupBSDFPath(isects.data(), rays.data(), paths.data(), M, pixels.data(), &count); });
    run_serial(N, [&] {
      LightHitPass(isects.data(), rays.data(), paths.data(), &total_lights, M, P, UV, NN, FF, &size,
                   ACC, pixels.data(), &count, (float4*)envmap, (float*)env_lum, (float*)env_sat, lg);
    });
    // CCompact.execute
    count = 0;
    run_serial(N, [&] { InitIntersection(tmp_isects.data(), &length); });
    run_serial(N, [&] { InitIntData(tmp_pixels.data(), &length); });
    run_serial(N, [&] {
      CompactAtomic(isects.data(), tmp_isects.data(), pixels.data(), tmp_pixels.data(), &count, &length);
    });
    run_serial(N, [&] { InitIntersection(isects.data(), &length); });
    run_serial(N, [&] { InitIntData(pixels.data(), &length); });
    run_serial(N, [&] { TransferIntersection(isects.data(), tmp_isects.data(), &length); });
    run_serial(N, [&] { TransferPixels(pixels.data(), tmp_pixels.data(), &length); });
    if (counts_out) counts_out[pathLength - 1] = count;
    // texture pass (CDeviceGI.java:241-244)
    if (g_ref_tex.nref > 0) {
      run_serial(N, [&] { texturePassGI(paths.data(), isects.data(), texd.data(), pixels.data(), &count); });
      texture_apply_process(texd.data(), count, g_ref_tex);
      run_serial(N, [&] { updateToTextureColorGI(paths.data(), texd.data(), pixels.data(), &count); });
    }
    // directLightEvaluation (CDeviceGI.java:273-277)
    allocate_state();
    run_serial(N, [&] {
      DirectLight(paths.data(), isects.data(), (LightInfo*)linfo.data(), &total_lights, occl.data(),
                  ACC, pixels.data(), &count, &st, M, P, UV, NN, FF, &size, ND, BD,
                  (float4*)envmap, (float*)env_lum, (float*)env_sat, lg);
    });
    run_serial(N, [&] {
      SampleBSDFRayDirection(isects.data(), rays.data(), paths.data(), M, pixels.data(), &st, &count);
    });
  }
  std::free(lg);
  return total_lights;
}

}  // extern "C"
