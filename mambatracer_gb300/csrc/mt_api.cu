// C-ABI of the GB300 wavefront path tracer (see include/mambatracer.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "mt_compact.h"
#include "mt_device.cuh"
#include "mt_internal.h"

// ------------------------------------------------------------------ context
namespace {
thread_local std::string g_err;
}

extern "C" const char* mt_last_error(void) { return g_err.c_str(); }

namespace mt {
__attribute__((visibility("hidden"))) void set_last_error(const char* msg) { g_err = msg; }
__attribute__((visibility("hidden"))) int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
}  // namespace mt

int quiesce(mt_context* ctx) {
  join_jobs(ctx);
  CU(cudaStreamSynchronize(ctx->stream));
  servers_sync(ctx);
  return MT_OK;
}

void join_jobs(mt_context* ctx) {
  for (mt_job* j : ctx->jobs) {
    for (JobSlot& s : j->slots)
      if (s.done) cudaStreamWaitEvent(ctx->stream, s.done, 0);
    if (j->rdone) cudaStreamWaitEvent(ctx->stream, j->rdone, 0);
  }
}

extern "C" const char* mt_version(void) {
  return "mambatracer-gb300 sm_103a fmad=false prec-div prec-sqrt";
}

extern "C" int mt_ctx_create(int device, mt_context** out) {
  if (!out) return fail(MT_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int n = 0;
  CU(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(MT_ERR_INVALID, "device %d of %d", device, n);
  CU(cudaSetDevice(device));
  auto* c = new mt_context();
  c->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    return fail(MT_ERR_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
  }
  c->num_sms = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(MT_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  if (dalloc(&c->d_scratch, 4) != MT_OK) {
    cudaStreamDestroy(c->stream);
    delete c;
    return MT_ERR_NOMEM;
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  *out = c;
  return MT_OK;
}

extern "C" int mt_ctx_destroy(mt_context* ctx) {
  if (!ctx) return fail(MT_ERR_INVALID, "ctx is NULL");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  dfree(ctx->d_scratch);
  dfree(ctx->cs_status);
  dfree(ctx->cs_words);
  dfree(ctx->d_plain_err);
  for (auto& ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MT_OK;
}

extern "C" int mt_ctx_event_record(mt_context* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 8) return fail(MT_ERR_INVALID, "bad event slot");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  join_jobs(ctx);
  CU(cudaEventRecord(ctx->ev[slot], ctx->stream));
  return MT_OK;
}

extern "C" int mt_ctx_event_elapsed(mt_context* ctx, int a, int b, float* ms) {
  if (!ctx || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return fail(MT_ERR_INVALID, "bad event slot");
  CU(cudaSetDevice(ctx->device));
  CU(cudaEventSynchronize(ctx->ev[b]));
  CU(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
  return MT_OK;
}

extern "C" int mt_finish(mt_context* ctx) {
  if (!ctx) return fail(MT_ERR_INVALID, "ctx is NULL");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  join_jobs(ctx);
  CU(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_plain_err) {
    int e = 0;
    CU(cudaMemcpy(&e, ctx->d_plain_err, 4, cudaMemcpyDeviceToHost));
    if (e) {
      CU(cudaMemset(ctx->d_plain_err, 0, 4));
      return fail(MT_ERR_DEVICE, "a kernel launched by name met %s", e == 1 ? "an index out of range in its buffers"
                                                                           : "a BVH deeper than 64 levels");
    }
  }
  return MT_OK;
}

// ------------------------------------------------------------------ buffers
extern "C" int mt_buf_alloc(mt_context* ctx, size_t bytes, mt_buffer** out) {
  if (!ctx || !out) return fail(MT_ERR_INVALID, "NULL argument");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(MT_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  CU(cudaMemsetAsync(p, 0, bytes ? bytes : 1, ctx->stream));
  *out = new mt_buffer{ctx, p, bytes};
  return MT_OK;
}

extern "C" int mt_buf_create_from(mt_context* ctx, const void* host, size_t bytes, mt_buffer** out) {
  int r = mt_buf_alloc(ctx, bytes, out);
  if (r != MT_OK) return r;
  return mt_buf_write(*out, 0, host, bytes);
}

extern "C" int mt_buf_write(mt_buffer* b, size_t off, const void* host, size_t bytes) {
  if (!b || (!host && bytes)) return fail(MT_ERR_INVALID, "NULL argument");
  if (off > b->bytes || bytes > b->bytes - off) return fail(MT_ERR_INVALID, "write [%zu,+%zu) past %zu B", off, bytes, b->bytes);
  std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
  CU(cudaSetDevice(b->ctx->device));
  CU(cudaMemcpyAsync((char*)b->ptr + off, host, bytes, cudaMemcpyHostToDevice, b->ctx->stream));
  CU(cudaStreamSynchronize(b->ctx->stream));
  return MT_OK;
}

extern "C" int mt_buf_read(mt_buffer* b, size_t off, void* host, size_t bytes) {
  if (!b || (!host && bytes)) return fail(MT_ERR_INVALID, "NULL argument");
  if (off > b->bytes || bytes > b->bytes - off) return fail(MT_ERR_INVALID, "read [%zu,+%zu) past %zu B", off, bytes, b->bytes);
  std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
  CU(cudaSetDevice(b->ctx->device));
  CU(cudaMemcpyAsync(host, (char*)b->ptr + off, bytes, cudaMemcpyDeviceToHost, b->ctx->stream));
  CU(cudaStreamSynchronize(b->ctx->stream));
  return MT_OK;
}

namespace {
__global__ void k_fill32(uint32_t* p, uint32_t v, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}
}  // namespace

extern "C" int mt_buf_fill32(mt_buffer* b, uint32_t pattern, size_t off, size_t bytes) {
  if (!b) return fail(MT_ERR_INVALID, "NULL buffer");
  if ((off | bytes) & 3) return fail(MT_ERR_INVALID, "offset and size must be multiples of 4");
  if (off > b->bytes || bytes > b->bytes - off) return fail(MT_ERR_INVALID, "fill past the end");
  std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
  CU(cudaSetDevice(b->ctx->device));
  size_t n = bytes / 4;
  if (n) k_fill32<<<(unsigned)((n + 255) / 256), 256, 0, b->ctx->stream>>>((uint32_t*)((char*)b->ptr + off), pattern, n);
  CU(cudaGetLastError());
  return MT_OK;
}

extern "C" size_t mt_buf_size(const mt_buffer* b) { return b ? b->bytes : 0; }

extern "C" int mt_buf_free(mt_buffer* b) {
  if (!b) return fail(MT_ERR_INVALID, "NULL buffer");
  {
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    cudaFree(b->ptr);
  }
  delete b;
  return MT_OK;
}

// ------------------------------------------------------------------- scene
namespace {

bool emitter_host(const Material& m) {
  float s = m.emission_param.x;
  float x = m.emission_color.x * s, y = m.emission_color.y * s, z = m.emission_color.z * s;
  return (0.2989f * x + 0.5866f * y) + 0.1145f * z != 0.0f;
}

int upload_lights(mt_scene* s) {
  // identifyMeshLights + prefix scan + prepareLightInfo (CLightConfiguration.java:43-87):
  // the faces whose material emits, in face order.
  std::vector<int> lf;
  const Face* F = reinterpret_cast<const Face*>(s->h_faces.data());
  const Material* M = reinterpret_cast<const Material*>(s->h_materials.data());
  for (int i = 0; i < s->ntri; ++i) {
    int m = F[i].mat & 0xFFFF;
    if (emitter_host(M[m])) lf.push_back(i);
  }
  dfree(s->d_light_faces);
  s->nlights = (int)lf.size();
  int r = dalloc(&s->d_light_faces, lf.size());
  if (r) return r;
  if (!lf.empty()) CU(cudaMemcpy(s->d_light_faces, lf.data(), lf.size() * 4, cudaMemcpyHostToDevice));
  return MT_OK;
}

template <class T>
int upload(T** d, const void* h, size_t count) {
  dfree(*d);
  int r = dalloc(d, count);
  if (r) return r;
  if (h && count) CU(cudaMemcpy(*d, h, count * sizeof(T), cudaMemcpyHostToDevice));
  return MT_OK;
}

void free_scene(mt_scene* s) {
  dfree(s->d_points);
  dfree(s->d_uvs);
  dfree(s->d_normals);
  dfree(s->d_faces);
  dfree(s->d_materials);
  dfree(s->d_light_faces);
  dfree(s->d_nodes);
  dfree(s->d_tris);
  dfree(s->d_qnodes);
  dfree(s->d_wnodes);
  dfree(s->d_wtris);
  dfree(s->d_quad);
  dfree(s->d_up);
  dfree(s->d_env_rgb);
  dfree(s->d_env_lum);
  dfree(s->d_env_sat);
  dfree(s->d_env_sat64);
  dfree(s->d_env_marg);
  dfree(s->d_env_cond);
  dfree(s->d_texels);
  dfree(s->d_tex_ref);
}

// CDF tables of the whole map for full-map environment sampling, from its FP32 SAT.
int build_env_tables(mt_scene* s) {
  dfree(s->d_env_marg);
  dfree(s->d_env_cond);
  if (!cdf_tables_enabled()) return MT_OK;
  size_t m = 0;
  const size_t c = map_table_floats(s->env_w, s->env_h, &m);
  int r = dalloc(&s->d_env_marg, m);
  if (!r) r = dalloc(&s->d_env_cond, c);
  if (!r && launch_map_tables(s->ctx->stream, s->d_env_sat, s->env_w, s->env_h, s->d_env_marg, s->d_env_cond))
    r = fail(MT_ERR_CUDA, "environment tables: %s", cudaGetErrorString(cudaGetLastError()));
  if (r) {
    dfree(s->d_env_marg);
    dfree(s->d_env_cond);
  }
  return r;
}

// Texel pool (all images back to back) and the per-material table of
// (first texel, width, height, 0) for diffuse, glossy, roughness and mirror.
int upload_textures(mt_scene* s) {
  s->h_tex.resize(4 * (size_t)s->nmat);
  size_t total = 0;
  for (const auto& t : s->h_tex) total += t.argb.size();
  if (total > 0x7FFFFFFFu) return fail(MT_ERR_INVALID, "textures hold %zu texels (at most 2^31 - 1)", total);
  dfree(s->d_texels);
  dfree(s->d_tex_ref);
  s->tex_on = 0;
  if (total == 0) return MT_OK;
  std::vector<int32_t> pool;
  pool.reserve(total);
  std::vector<int4> ref(s->h_tex.size());
  for (size_t i = 0; i < s->h_tex.size(); ++i) {
    const auto& t = s->h_tex[i];
    ref[i] = make_int4(t.argb.empty() ? 0 : (int)pool.size(), t.argb.empty() ? 0 : t.w, t.argb.empty() ? 0 : t.h, 0);
    pool.insert(pool.end(), t.argb.begin(), t.argb.end());
  }
  int r = upload(&s->d_texels, pool.data(), pool.size());
  if (!r) r = upload(&s->d_tex_ref, ref.data(), ref.size());
  if (r) return r;
  s->tex_on = 1;
  return MT_OK;
}

}  // namespace

extern "C" int mt_scene_create(mt_context* ctx, const float* points, int npoints, const float* uvs, int nuvs,
                               const float* normals, int nnormals, const int32_t* faces, int nfaces,
                               const void* materials, int nmaterials, mt_scene** out) {
  if (!ctx || !out || !points || !faces || !materials) return fail(MT_ERR_INVALID, "NULL argument");
  if (npoints <= 0 || nfaces <= 0 || nmaterials <= 0) return fail(MT_ERR_INVALID, "empty scene");
  if (nmaterials > 65536) return fail(MT_ERR_INVALID, "more than 65536 materials (16-bit material index)");
  *out = nullptr;
  const Face* F = reinterpret_cast<const Face*>(faces);
  for (int i = 0; i < nfaces; ++i) {
    const Face& f = F[i];
    if (f.vx < 0 || f.vy < 0 || f.vz < 0 || f.vx >= npoints || f.vy >= npoints || f.vz >= npoints)
      return fail(MT_ERR_INVALID, "face %d: vertex index out of range", i);
    if ((f.mat & 0xFFFF) >= nmaterials) return fail(MT_ERR_INVALID, "face %d: material %d of %d", i, f.mat & 0xFFFF, nmaterials);
    if (f.uvx > -1 && (!uvs || f.uvx >= nuvs || f.uvy < 0 || f.uvy >= nuvs || f.uvz < 0 || f.uvz >= nuvs))
      return fail(MT_ERR_INVALID, "face %d: uv index out of range", i);
    if (f.nx > -1 && (!normals || f.nx >= nnormals || f.ny < 0 || f.ny >= nnormals || f.nz < 0 || f.nz >= nnormals))
      return fail(MT_ERR_INVALID, "face %d: normal index out of range", i);
  }
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  auto* s = new mt_scene();
  s->ctx = ctx;
  s->npoints = npoints;
  s->nuvs = nuvs;
  s->nnormals = nnormals;
  s->ntri = nfaces;
  s->nmat = nmaterials;
  s->h_points.assign(points, points + 4 * (size_t)npoints);
  s->h_faces.assign(faces, faces + 10 * (size_t)nfaces);
  s->h_materials.assign((const uint8_t*)materials, (const uint8_t*)materials + 144 * (size_t)nmaterials);
  int r = upload(&s->d_points, points, (size_t)npoints);
  if (!r) r = upload(&s->d_uvs, uvs, uvs ? (size_t)nuvs : 1);
  if (!r) r = upload(&s->d_normals, normals, normals ? (size_t)nnormals : 1);
  if (!r) r = upload(&s->d_faces, faces, (size_t)nfaces);
  if (!r) r = upload(&s->d_materials, materials, (size_t)nmaterials);
  if (!r) r = upload_lights(s);
  if (r) {
    std::string keep = g_err;
    free_scene(s);
    delete s;
    g_err = keep;
    return r;
  }
  *out = s;
  return MT_OK;
}

extern "C" int mt_scene_set_materials(mt_scene* s, const void* materials, int nmaterials) {
  if (!s || !materials || nmaterials <= 0) return fail(MT_ERR_INVALID, "bad argument");
  const Face* F = reinterpret_cast<const Face*>(s->h_faces.data());
  for (int i = 0; i < s->ntri; ++i)
    if ((F[i].mat & 0xFFFF) >= nmaterials) return fail(MT_ERR_INVALID, "face %d needs material %d", i, F[i].mat & 0xFFFF);
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  s->h_materials.assign((const uint8_t*)materials, (const uint8_t*)materials + 144 * (size_t)nmaterials);
  s->nmat = nmaterials;
  int r = upload(&s->d_materials, materials, (size_t)nmaterials);
  if (!r) r = upload_lights(s);
  if (!r) r = upload_textures(s);
  return r;
}

extern "C" int mt_scene_set_texture(mt_scene* s, int material, int kind, const int32_t* argb, int width,
                                    int height) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  if (material < 0 || material >= s->nmat) return fail(MT_ERR_INVALID, "material %d of %d", material, s->nmat);
  if (kind < 0 || kind > 3) return fail(MT_ERR_INVALID, "texture kind %d (0 diffuse, 1 glossy, 2 roughness, 3 mirror)", kind);
  if (argb && (width <= 0 || height <= 0 || (long long)width * height > 0x7FFFFFFFll))
    return fail(MT_ERR_INVALID, "texture of %d x %d", width, height);
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  s->h_tex.resize(4 * (size_t)s->nmat);
  auto& t = s->h_tex[4 * (size_t)material + kind];
  if (argb) {
    t.argb.assign(argb, argb + (size_t)width * height);
    t.w = width;
    t.h = height;
  } else {
    t = mt_scene::HostTex{};
  }
  return upload_textures(s);
}

bool cdf_tables_enabled() {
  const char* v = std::getenv("MT_CDF_TABLES");
  return !(v && std::atoi(v) == 0);
}

extern "C" int mt_scene_light_count(const mt_scene* s) { return s ? s->nlights : -1; }

extern "C" int mt_scene_destroy(mt_scene* s) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  if (s->refs.load() > 0) return fail(MT_ERR_BUSY, "scene used by %d served requests", s->refs.load());
  {
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    cudaSetDevice(s->ctx->device);
    quiesce(s->ctx);
    free_scene(s);
  }
  delete s;
  return MT_OK;
}

// ---------------------------------------------------------------- BVH build
// CNormalBVH.build (src/cl/scene/CNormalBVH.java:45-148): recursive split at the
// centre of the centroid bound's longest axis, one triangle per leaf, children
// allocated as adjacent pairs in preorder, node.bound = node index. The
// partition (CNormalBVH.java:132) is an un-vendored library routine; this builder
// uses a stable split "centroid[dim] < split", falling back to the middle index
// when one side would be empty (CNormalBVH.java:135-136).
namespace {
struct Builder {
  const float* pts;
  const Face* faces;
  int n;
  std::vector<int> obj, tmp;
  std::vector<float> tb, cen;
  int32_t* nodes;   // 7 per node
  float* bounds;    // 8 per node
  int ptr = 1, max_depth = 0;

  void init() {
    obj.resize(n);
    tb.resize(6 * (size_t)n);
    cen.resize(3 * (size_t)n);
    for (int t = 0; t < n; ++t) {
      obj[t] = t;
      const Face& f = faces[t];
      const float* p[3] = {pts + 4 * (size_t)f.vx, pts + 4 * (size_t)f.vy, pts + 4 * (size_t)f.vz};
      for (int a = 0; a < 3; ++a) {
        float lo = INFINITY, hi = -INFINITY;
        for (int k = 0; k < 3; ++k) {
          if (p[k][a] < lo) lo = p[k][a];
          if (p[k][a] > hi) hi = p[k][a];
        }
        tb[6 * (size_t)t + a] = lo;
        tb[6 * (size_t)t + 3 + a] = hi;
        cen[3 * (size_t)t + a] = 0.5f * (lo + hi);
      }
    }
  }
  void subdivide(int parent, int start, int end, int depth) {
    // iterative on the right child to bound the C++ stack on deep trees
    for (;;) {
      max_depth = std::max(max_depth, depth);
      float bmn[3] = {INFINITY, INFINITY, INFINITY}, bmx[3] = {-INFINITY, -INFINITY, -INFINITY};
      float cmn[3] = {INFINITY, INFINITY, INFINITY}, cmx[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (int p = start; p < end; ++p) {
        int t = obj[p];
        for (int a = 0; a < 3; ++a) {
          float lo = tb[6 * (size_t)t + a], hi = tb[6 * (size_t)t + 3 + a], c = cen[3 * (size_t)t + a];
          bmn[a] = std::min(bmn[a], lo);
          bmx[a] = std::max(bmx[a], hi);
          cmn[a] = std::min(cmn[a], c);
          cmx[a] = std::max(cmx[a], c);
        }
      }
      int32_t* nd = nodes + 7 * (size_t)parent;
      float* bd = bounds + 8 * (size_t)parent;
      nd[0] = parent;  // bound
      for (int a = 0; a < 3; ++a) {
        bd[a] = bmn[a];
        bd[4 + a] = bmx[a];
      }
      bd[3] = bd[7] = 0.f;
      if (end - start < 2) {
        nd[6] = obj[start];  // child
        nd[5] = 1;           // isLeaf
        return;
      }
      int li = ptr++, ri = ptr++;
      int32_t* ln = nodes + 7 * (size_t)li;
      int32_t* rn = nodes + 7 * (size_t)ri;
      std::memset(ln, 0, 28);
      std::memset(rn, 0, 28);
      ln[4] = parent;  // parent
      rn[4] = parent;
      ln[1] = ri;      // sibling
      rn[1] = li;
      nd[2] = li;      // left
      nd[3] = ri;      // right
      float ex = cmx[0] - cmn[0], ey = cmx[1] - cmn[1], ez = cmx[2] - cmn[2];
      int dim = (ex > ey && ex > ez) ? 0 : (ey > ez ? 1 : 2);
      float split = 0.5f * (cmn[dim] + cmx[dim]);
      int nl = 0;
      for (int p = start; p < end; ++p) nl += cen[3 * (size_t)obj[p] + dim] < split;
      int mid = start + nl;
      if (mid != start && mid != end) {
        tmp.resize(end - start);
        int a = start, b = 0;
        for (int p = start; p < end; ++p) {
          int t = obj[p];
          if (cen[3 * (size_t)t + dim] < split) obj[a++] = t;
          else tmp[b++] = t;
        }
        std::memcpy(obj.data() + mid, tmp.data(), sizeof(int) * (size_t)b);
      } else {
        mid = start + (end - start) / 2;
      }
      subdivide(li, start, mid, depth + 1);
      parent = ri;
      start = mid;
      depth = depth + 1;
    }
  }
};

// Convert the reference node layout into the traversal layout and upload it.
int import_bvh(mt_scene* s, const int32_t* nodes, const float* bounds, int nnodes) {
  const int n = s->ntri;
  if (nnodes != 2 * n - 1) return fail(MT_ERR_INVALID, "%d nodes for %d triangles (want 2N-1)", nnodes, n);
  auto node = [&](int i) { return nodes + 7 * (size_t)i; };
  // A breadth-first pass checks the tree and its depth; a depth-first pass (left
  // before right) numbers the interior records in preorder and the leaf slots
  // in leaf order.
  std::vector<int> rec(nnodes, -1), slot(nnodes, -1), level(nnodes, 0);
  std::vector<int> order;
  order.reserve(n);
  const int32_t* root = node(0);
  int max_level = 0;
  if (!root[5]) {
    std::deque<int> q;
    q.push_back(0);
    int k = 0;
    std::vector<char> seen(nnodes, 0);
    seen[0] = 1;
    while (!q.empty()) {
      int i = q.front();
      q.pop_front();
      const int32_t* nd = node(i);
      for (int c : {nd[2], nd[3]}) {
        if (c <= 0 || c >= nnodes || seen[c]) return fail(MT_ERR_INVALID, "node %d: bad child %d", i, c);
        seen[c] = 1;
        const int32_t* cn = node(c);
        if (cn[0] < 0 || cn[0] >= nnodes) return fail(MT_ERR_INVALID, "node %d: bad bound index %d", c, cn[0]);
        level[c] = level[i] + 1;
        max_level = std::max(max_level, level[c]);
        if (!cn[5]) q.push_back(c);
        else if (cn[6] < 0 || cn[6] >= n) return fail(MT_ERR_INVALID, "leaf %d: bad triangle %d", c, cn[6]);
      }
    }
    std::vector<int> st{0};
    while (!st.empty()) {
      int i = st.back();
      st.pop_back();
      const int32_t* nd = node(i);
      if (nd[5]) {
        slot[i] = (int)order.size();
        order.push_back(nd[6]);
        continue;
      }
      rec[i] = k++;
      st.push_back(nd[3]);
      st.push_back(nd[2]);
    }
  } else {
    if (root[6] < 0 || root[6] >= n) return fail(MT_ERR_INVALID, "root leaf: bad triangle");
    slot[0] = 0;
    order.push_back(root[6]);
  }
  // Deferred-node stack depth needed <= tree depth; the reference's bitstack holds 64 levels.
  if (max_level > kStackDepth) return fail(MT_ERR_DEPTH, "BVH depth %d exceeds %d", max_level, kStackDepth);
  const int nrec = root[5] ? 0 : n - 1;
  std::vector<float4> hn(4 * (size_t)std::max(nrec, 1));
  auto ref_of = [&](int c) { return node(c)[5] ? ~slot[c] : rec[c]; };
  for (int i = 0; i < nnodes; ++i) {
    if (rec[i] < 0) continue;
    const int32_t* nd = node(i);
    const float* bl = bounds + 8 * (size_t)node(nd[2])[0];
    const float* br = bounds + 8 * (size_t)node(nd[3])[0];
    float4* r = hn.data() + 4 * (size_t)rec[i];
    r[0] = make_float4(bl[0], bl[4], bl[1], bl[5]);
    r[1] = make_float4(br[0], br[4], br[1], br[5]);
    r[2] = make_float4(bl[2], bl[6], br[2], br[6]);
    int lr = ref_of(nd[2]), rr = ref_of(nd[3]);
    float lf, rf;
    std::memcpy(&lf, &lr, 4);
    std::memcpy(&rf, &rr, 4);
    r[3] = make_float4(lf, rf, 0.f, 0.f);
  }
  if ((int)order.size() != n) return fail(MT_ERR_INVALID, "BVH reaches %zu of %d triangles", order.size(), n);
  std::vector<float4> ht(3 * (size_t)n);
  const Face* F = reinterpret_cast<const Face*>(s->h_faces.data());
  const float* P = s->h_points.data();
  for (int k = 0; k < n; ++k) {
    int f = order[k];
    const float* p1 = P + 4 * (size_t)F[f].vx;
    const float* p2 = P + 4 * (size_t)F[f].vy;
    const float* p3 = P + 4 * (size_t)F[f].vz;
    float fid;
    std::memcpy(&fid, &f, 4);
    ht[3 * (size_t)k + 0] = make_float4(p1[0], p1[1], p1[2], fid);
    ht[3 * (size_t)k + 1] = make_float4(p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2], 0.f);
    ht[3 * (size_t)k + 2] = make_float4(p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2], 0.f);
  }
  int r = upload(&s->d_nodes, hn.data(), hn.size());
  if (!r) r = upload(&s->d_tris, ht.data(), ht.size());
  if (r) return r;
  s->nrec = nrec;
  s->root_ref = root[5] ? ~0 : 0;
  s->depth = max_level;
  s->has_bvh = 1;
  return MT_OK;
}
}  // namespace

extern "C" int mt_bvh_build(mt_scene* s, int32_t* nodes_out, float* bounds_out, int* depth_out) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  const int n = s->ntri;
  std::vector<int32_t> nodes(7 * (size_t)(2 * n - 1), 0);
  std::vector<float> bounds(8 * (size_t)(2 * n - 1), 0.f);
  Builder b;
  b.pts = s->h_points.data();
  b.faces = reinterpret_cast<const Face*>(s->h_faces.data());
  b.n = n;
  b.nodes = nodes.data();
  b.bounds = bounds.data();
  b.init();
  b.subdivide(0, 0, n, 0);
  if (nodes_out) std::memcpy(nodes_out, nodes.data(), nodes.size() * 4);
  if (bounds_out) std::memcpy(bounds_out, bounds.data(), bounds.size() * 4);
  if (depth_out) *depth_out = b.max_depth;
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  int r = import_bvh(s, nodes.data(), bounds.data(), 2 * n - 1);
  return r ? r : refresh_qnodes(s);
}

extern "C" int mt_bvh_build_host(const float* points, int npoints, const int32_t* faces, int nfaces,
                                 int32_t* nodes_out, float* bounds_out, int* depth_out) {
  if (!points || !faces || !nodes_out || !bounds_out || npoints <= 0 || nfaces <= 0)
    return fail(MT_ERR_INVALID, "bad argument");
  const Face* F = reinterpret_cast<const Face*>(faces);
  for (int i = 0; i < nfaces; ++i)
    if (F[i].vx < 0 || F[i].vy < 0 || F[i].vz < 0 || F[i].vx >= npoints || F[i].vy >= npoints || F[i].vz >= npoints)
      return fail(MT_ERR_INVALID, "face %d: vertex index out of range", i);
  std::memset(nodes_out, 0, 28 * (size_t)(2 * nfaces - 1));
  std::memset(bounds_out, 0, 32 * (size_t)(2 * nfaces - 1));
  Builder b;
  b.pts = points;
  b.faces = F;
  b.n = nfaces;
  b.nodes = nodes_out;
  b.bounds = bounds_out;
  b.init();
  b.subdivide(0, 0, nfaces, 0);
  if (depth_out) *depth_out = b.max_depth;
  return MT_OK;
}

extern "C" int mt_scene_layout_read(mt_scene* s, void* records_out, void* tris_out, int* nrec_out,
                                    int* root_ref_out) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  if (!s->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  CU(cudaStreamSynchronize(s->ctx->stream));
  if (records_out && s->nrec) CU(cudaMemcpy(records_out, s->d_nodes, 64 * (size_t)s->nrec, cudaMemcpyDeviceToHost));
  if (tris_out) CU(cudaMemcpy(tris_out, s->d_tris, 48 * (size_t)s->ntri, cudaMemcpyDeviceToHost));
  if (nrec_out) *nrec_out = s->nrec;
  if (root_ref_out) *root_ref_out = s->root_ref;
  return MT_OK;
}

extern "C" int mt_bvh_import(mt_scene* s, const int32_t* nodes, const float* bounds, int nnodes) {
  if (!s || !nodes || !bounds) return fail(MT_ERR_INVALID, "NULL argument");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  int r = import_bvh(s, nodes, bounds, nnodes);
  return r ? r : refresh_qnodes(s);
}

extern "C" int mt_scene_set_bvh_precision(mt_scene* s, int precision) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  if (precision < 0 || precision > 3)
    return fail(MT_ERR_INVALID, "BVH precision %d (0 FP32, 1 FP16, 2 wide 8-bit, 3 4-wide FP16)", precision);
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  s->precision = precision;
  return refresh_qnodes(s);
}

// -------------------------------------------------------------- environment
extern "C" int mt_env_set(mt_scene* s, const float* rgb, int w, int h) {
  if (!s || !rgb || w <= 0 || h <= 0) return fail(MT_ERR_INVALID, "bad environment map");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  size_t n = (size_t)w * h;
  int r = upload(&s->d_env_rgb, rgb, n);
  if (!r) { dfree(s->d_env_lum); r = dalloc(&s->d_env_lum, n); }
  if (!r) { dfree(s->d_env_sat); r = dalloc(&s->d_env_sat, n); }
  if (!r) { dfree(s->d_env_sat64); r = dalloc(&s->d_env_sat64, n); }
  if (r) return r;
  if (launch_env_build(s->ctx->stream, s->d_env_rgb, w, h, s->d_env_lum, s->d_env_sat64, s->d_env_sat))
    return fail(MT_ERR_CUDA, "environment build launch: %s", cudaGetErrorString(cudaGetLastError()));
  s->env_w = w;
  s->env_h = h;
  if ((r = build_env_tables(s))) return r;
  CU(cudaStreamSynchronize(s->ctx->stream));
  s->env_present = 1;
  return MT_OK;
}

extern "C" int mt_env_set_with_sat(mt_scene* s, const float* rgb, const float* lum, const float* sat, int w, int h) {
  if (!s || !rgb || !lum || !sat || w <= 0 || h <= 0) return fail(MT_ERR_INVALID, "bad environment map");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  size_t n = (size_t)w * h;
  int r = upload(&s->d_env_rgb, rgb, n);
  if (!r) r = upload(&s->d_env_lum, lum, n);
  if (!r) r = upload(&s->d_env_sat, sat, n);
  if (r) return r;
  dfree(s->d_env_sat64);
  s->env_w = w;
  s->env_h = h;
  if ((r = build_env_tables(s))) return r;
  CU(cudaStreamSynchronize(s->ctx->stream));
  s->env_present = 1;
  return MT_OK;
}

extern "C" int mt_env_clear(mt_scene* s) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  s->env_present = 0;
  return MT_OK;
}

extern "C" int mt_env_read(mt_scene* s, float* lum, double* sat64, float* sat32) {
  if (!s || !s->env_present) return fail(MT_ERR_INVALID, "no environment map");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  CU(cudaStreamSynchronize(s->ctx->stream));
  size_t n = (size_t)s->env_w * s->env_h;
  if (lum) CU(cudaMemcpy(lum, s->d_env_lum, n * 4, cudaMemcpyDeviceToHost));
  if (sat32) CU(cudaMemcpy(sat32, s->d_env_sat, n * 4, cudaMemcpyDeviceToHost));
  if (sat64) {
    if (!s->d_env_sat64) return fail(MT_ERR_INVALID, "the SAT was given, not built in FP64");
    CU(cudaMemcpy(sat64, s->d_env_sat64, n * 8, cudaMemcpyDeviceToHost));
  }
  return MT_OK;
}

extern "C" int mt_env_grid_config(mt_scene* s, int nu, int nv, int rx, int ry, int enable) {
  if (!s || nu <= 0 || nv <= 0 || nu % rx || nv % ry || enable < 0 || enable > 2) return fail(MT_ERR_INVALID, "bad grid");
  if (!((rx == 8 || rx == 16 || rx == 32) && (ry == 8 || ry == 16 || ry == 32)))
    return fail(MT_ERR_INVALID, "tiles per cell must be 8, 16 or 32 along each axis");
  if ((long long)nu * nv > (1ll << 28)) return fail(MT_ERR_INVALID, "grid of %d x %d is too large", nu, nv);
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CU(cudaSetDevice(s->ctx->device));
  int q = quiesce(s->ctx);
  if (q) return q;
  ++s->version;
  s->grid_nu = nu;
  s->grid_nv = nv;
  s->grid_rx = rx;
  s->grid_ry = ry;
  s->grid_on = enable;
  return MT_OK;
}

extern "C" int mt_env_grid_sat(mt_context* ctx, const float* func, float* sat_out, int nu, int nv, int rx, int ry,
                               int fp64) {
  if (!ctx || !func || !sat_out || nu <= 0 || nv <= 0) return fail(MT_ERR_INVALID, "bad argument");
  if (!((rx == 8 || rx == 16 || rx == 32) && (ry == 8 || ry == 16 || ry == 32)) || nu % rx || nv % ry)
    return fail(MT_ERR_INVALID, "tiles per cell must be 8, 16 or 32 and divide the grid");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  size_t n = (size_t)nu * nv;
  float *d_func = nullptr, *d_sat = nullptr;
  double* d_sat64 = nullptr;
  int r = dalloc(&d_func, n);
  if (!r) r = dalloc(&d_sat, n);
  if (!r && fp64) r = dalloc(&d_sat64, n);
  if (!r) {
    cudaMemcpyAsync(d_func, func, n * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (launch_grid_sat(ctx->stream, d_func, d_sat, d_sat64, nu, nv, rx, ry, fp64))
      r = fail(MT_ERR_CUDA, "grid SAT launch failed");
    else if (cudaMemcpyAsync(sat_out, d_sat, n * 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
             cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      r = fail(MT_ERR_CUDA, "grid SAT copy: %s", cudaGetErrorString(cudaGetLastError()));
  }
  dfree(d_func);
  dfree(d_sat);
  dfree(d_sat64);
  return r;
}

// ------------------------------------------------------------- ray queries
namespace {
int query(mt_scene* s, const void* rays, int n, int any, float* t_out, int32_t* prim_out,
          int32_t* counts_out = nullptr) {
  if (!s || (!rays && n) || !prim_out || (!any && !t_out) || n < 0) return fail(MT_ERR_INVALID, "bad argument");
  if (!s->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH");
  if (n == 0) return MT_OK;
  mt_context* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  float4* d_rays = nullptr;
  float* d_t = nullptr;
  int* d_p = nullptr;
  int* d_c = nullptr;
  int r = dalloc(&d_rays, 5 * (size_t)n);
  if (!r) r = dalloc(&d_t, (size_t)n);
  if (!r) r = dalloc(&d_p, (size_t)n);
  if (!r && counts_out) r = dalloc(&d_c, 2 * (size_t)n);
  if (!r) {
    cudaMemcpyAsync(d_rays, rays, 80 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(ctx->d_scratch, 0, 8, ctx->stream);
    const int lr = counts_out ? launch_count(ctx->stream, s->view(), d_rays, n, any, d_t, d_p, d_c, ctx->d_scratch + 1)
                              : launch_query(ctx->stream, s->view(), d_rays, n, any, d_t, d_p, ctx->d_scratch,
                                             ctx->d_scratch + 1, ctx->num_sms);
    if (lr) r = fail(MT_ERR_CUDA, "query launch: %s", cudaGetErrorString(cudaGetLastError()));
  }
  int err = 0;
  if (!r) {
    if (!any) cudaMemcpyAsync(t_out, d_t, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(prim_out, d_p, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (counts_out) cudaMemcpyAsync(counts_out, d_c, 8 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&err, ctx->d_scratch + 1, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) r = fail(MT_ERR_CUDA, "query: %s", cudaGetErrorString(e));
    else if (err) r = fail(MT_ERR_DEVICE, "device error %d", err);
  }
  dfree(d_rays);
  dfree(d_t);
  dfree(d_p);
  dfree(d_c);
  return r;
}
}  // namespace

extern "C" int mt_trace_counts(mt_scene* s, const void* rays, int n, int any, float* t_out, int32_t* prim_out,
                               int32_t* counts_out) {
  if (!counts_out) return fail(MT_ERR_INVALID, "NULL counts");
  return query(s, rays, n, any ? 1 : 0, any ? nullptr : t_out, prim_out, counts_out);
}

extern "C" int mt_trace_closest(mt_scene* s, const void* rays, int n, float* t_out, int32_t* prim_out) {
  return query(s, rays, n, 0, t_out, prim_out);
}

extern "C" int mt_tuning_get(mt_tuning* out) {
  if (!out) return fail(MT_ERR_INVALID, "NULL argument");
  const Tuning t = get_tuning();
  *out = mt_tuning{t.closest_minb, t.shadow_minb, t.closest_grid, t.shadow_grid, t.shade_minb, t.refill_steps,
                   t.shadow_stream};
  return MT_OK;
}

extern "C" int mt_tuning_set(const mt_tuning* in) {
  if (!in) return fail(MT_ERR_INVALID, "NULL argument");
  const Tuning t{in->closest_minb, in->shadow_minb, in->closest_grid, in->shadow_grid,
                 in->shade_minb,   in->refill_steps, in->shadow_stream};
  if (!set_tuning(t))
    return fail(MT_ERR_INVALID, "tuning out of range: minb %d/%d (8, 12, 16), grids %d/%d (0..32), shade %d (3..5), "
                                "steps %d (4..1024), shadow_stream %d (0, 1)",
                t.closest_minb, t.shadow_minb, t.closest_grid, t.shadow_grid, t.shade_minb, t.refill_steps,
                t.shadow_stream);
  return MT_OK;
}

extern "C" int mt_trace_any(mt_scene* s, const void* rays, int n, int32_t* occluded_out) {
  return query(s, rays, n, 1, nullptr, occluded_out);
}

extern "C" int mt_trace_closest_dev(mt_scene* s, mt_buffer* rays, int n, mt_buffer* t_out, mt_buffer* prim_out,
                                    float* ms_out) {
  if (!s || !rays || !t_out || !prim_out || n < 0) return fail(MT_ERR_INVALID, "bad argument");
  if (rays->bytes < 80 * (size_t)n || t_out->bytes < 4 * (size_t)n || prim_out->bytes < 4 * (size_t)n)
    return fail(MT_ERR_INVALID, "buffers too small for %d rays", n);
  mt_context* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  cudaMemsetAsync(ctx->d_scratch, 0, 8, ctx->stream);
  cudaEventRecord(a, ctx->stream);
  int r = launch_query(ctx->stream, s->view(), (const float4*)rays->ptr, n, 0, (float*)t_out->ptr, (int*)prim_out->ptr,
                       ctx->d_scratch, ctx->d_scratch + 1, ctx->num_sms);
  cudaEventRecord(b, ctx->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (r || e != cudaSuccess) return fail(MT_ERR_CUDA, "trace: %s", cudaGetErrorString(cudaGetLastError()));
  if (ms_out) *ms_out = ms;
  return MT_OK;
}

// ------------------------------------------------- kernels by name (stubs)
// ------------------------------------------------------------- compaction
extern "C" int mt_compact_isects(mt_context* ctx, const void* isects_in, const int32_t* pixels_in, int n,
                                 void* isects_out, int32_t* pixels_out, int32_t* count_io) {
  if (!ctx || n < 0 || (n > 0 && (!isects_in || !pixels_in || !isects_out || !pixels_out)) || !count_io)
    return fail(MT_ERR_INVALID, "bad argument");
  if (n > (1 << 30)) return fail(MT_ERR_INVALID, "n = %d exceeds 2^30", n);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  const size_t tiles = (size_t)(n + kCompactThreads - 1) / kCompactThreads;
  if (tiles > ctx->cs_tiles || !ctx->cs_words) {
    CU(cudaStreamSynchronize(ctx->stream));
    dfree(ctx->cs_status);
    dfree(ctx->cs_words);
    ctx->cs_tiles = 0;
    int r = dalloc(&ctx->cs_status, tiles ? tiles : 1);
    if (!r) r = dalloc(&ctx->cs_words, 4);
    if (r) return r;
    ctx->cs_tiles = tiles ? tiles : 1;
  }
  const cudaError_t le = launch_compact_isects(ctx->stream, isects_in, pixels_in, n, isects_out, pixels_out,
                                               count_io, CompactScratch{ctx->cs_status, ctx->cs_words});
  if (le != cudaSuccess) return fail(MT_ERR_CUDA, "compaction launch: %s", cudaGetErrorString(le));
  int err = 0;
  CU(cudaMemcpyAsync(&err, ctx->cs_words + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (err) return fail(MT_ERR_DEVICE, "compaction: device error %d", err);
  return MT_OK;
}

extern "C" void* mt_buf_device_ptr(mt_buffer* b) { return b ? b->ptr : nullptr; }
