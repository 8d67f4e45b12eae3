// Internal definitions shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mambatracer.h"
#include "mt_common.h"
#include "mt_kernels.h"

using namespace mt;

struct mt_job;
struct mt_server;

// ------------------------------------------------------------------ errors
namespace mt {
// Records the message mt_last_error() returns on this thread; returns code.
__attribute__((visibility("hidden"))) int fail(int code, const char* fmt, ...);
}  // namespace mt
using mt::fail;

namespace {
#define CU(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return fail(MT_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(MT_ERR_NOMEM, "cudaMalloc(%zu B): %s", count * sizeof(T), cudaGetErrorString(e));
  }
  return MT_OK;
}
template <class T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}
}  // namespace

// ----------------------------------------------------------------- structs
struct mt_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::recursive_mutex mu;
  int* d_scratch = nullptr;  // [0] work counter, [1] error for ray queries
  cudaEvent_t ev[8] = {};
  // compaction scratch, grown on demand
  unsigned long long* cs_status = nullptr;
  int* cs_words = nullptr;
  size_t cs_tiles = 0;
  std::vector<mt_job*> jobs;  // jobs whose streams join into `stream`
  std::vector<mt_server*> servers;  // served-mode schedulers on this context
  int* d_plain_err = nullptr;       // error latched by kernels launched by name
};

struct mt_buffer {
  mt_context* ctx;
  void* ptr;
  size_t bytes;
};

// MT_TRAVERSAL=bitstack (read once per process): the binary formats traverse
// without a deferred-node stack, as the reference does (bitstack_steps).
bool traversal_bitstack();

struct mt_scene {
  mt_context* ctx;
  int npoints = 0, nuvs = 0, nnormals = 0, ntri = 0, nmat = 0;
  std::vector<float> h_points;
  std::vector<int32_t> h_faces;
  std::vector<uint8_t> h_materials;
  float4* d_points = nullptr;
  float2* d_uvs = nullptr;
  float4* d_normals = nullptr;
  Face* d_faces = nullptr;
  Material* d_materials = nullptr;
  int* d_light_faces = nullptr;
  int nlights = 0;
  // traversal layout
  float4* d_nodes = nullptr;
  float4* d_tris = nullptr;
  uint4* d_qnodes = nullptr;  // FP16 records (precision 1)
  uint4* d_wnodes = nullptr;  // wide BVH with 8-bit child boxes (precision 2)
  uint4* d_quad = nullptr;    // 4-wide FP16 nodes (precision 3)
  int2* d_up = nullptr;       // parent links of the records (the stackless traversal)
  float4* d_wtris = nullptr;
  int nwide = 0, wdepth = 0;
  int nrec = 0, root_ref = 0, depth = 0, has_bvh = 0, precision = 0;
  // environment
  float4* d_env_rgb = nullptr;
  float* d_env_lum = nullptr;
  float* d_env_sat = nullptr;
  double* d_env_sat64 = nullptr;
  float* d_env_marg = nullptr;  // CDF tables of the whole map (dv::RegionTab)
  float* d_env_cond = nullptr;
  int env_w = 0, env_h = 0, env_present = 0;
  int grid_nu = 1600, grid_nv = 1600, grid_rx = 16, grid_ry = 32, grid_on = 0;  // grid_on: 0, 1 FP32, 2 FP64 SAT
  // textures: host images per (material, kind), the device pool and table
  struct HostTex {
    std::vector<int32_t> argb;
    int w = 0, h = 0;
  };
  std::vector<HostTex> h_tex;  // 4 per material: diffuse, glossy, roughness, mirror
  int* d_texels = nullptr;
  int4* d_tex_ref = nullptr;
  int tex_on = 0;
  unsigned version = 0;  // bumped when device arrays or the grid configuration change
  std::atomic<int> refs{0};  // served requests queued or running on this scene

  DevScene view() const {
    DevScene s{};
    s.nodes = d_nodes;
    s.qnodes = reinterpret_cast<const float4*>(d_qnodes);
    s.tris = d_tris;
    s.root_ref = root_ref;
    s.ntri = ntri;
    s.nrec = nrec;
    s.wnodes = d_wnodes;
    s.wtris = d_wtris;
    s.quad = d_quad;
    s.up = d_up;
    s.bitstack = d_up && traversal_bitstack();
    s.precision = (precision == 1 && d_qnodes) ? 1
                  : (precision == 2 && d_wnodes) ? 2
                  : (precision == 3 && d_quad)   ? 3
                                                 : 0;
    s.points = d_points;
    s.uvs = d_uvs;
    s.normals = d_normals;
    s.faces = d_faces;
    s.materials = d_materials;
    s.light_faces = d_light_faces;
    s.nlights = nlights;
    s.texels = d_texels;
    s.tex_ref = d_tex_ref;
    s.tex_on = tex_on;
    return s;
  }
  DevEnv env_view() const {
    DevEnv e{};
    e.rgb = d_env_rgb;
    e.lum = d_env_lum;
    e.sat = d_env_sat;
    e.w = env_w;
    e.h = env_h;
    e.present = env_present;
    e.grid_on = 0;
    e.env_marg = d_env_marg;
    e.env_cond = d_env_cond;
    return e;
  }
};

// One in-flight frame's resources: path state, queues, film, parameters,
// control blocks, and the stream its frames run on.
struct JobSlot {
  FrameBufs fb{};
  Ctrl* d_ctrl = nullptr;                  // one per pass
  unsigned long long* d_status = nullptr;  // compaction tile status, per pass and bounce
  PassParams* h_pp = nullptr;              // pinned, one per pass
  PassParams* d_pp = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // shadow rays beside the next bounce's extension rays
  cudaEvent_t sfork = nullptr, sjoin = nullptr;
  cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr, done = nullptr;
  cudaGraphExec_t graphs[2] = {nullptr, nullptr};  // per shading form: one launch, two launches
  unsigned graph_version = 0;  // scene version the graph was captured against
  bool ran = false;            // a frame has run on this slot (its control blocks hold its counts)
};

struct mt_job {
  mt_context* ctx;
  mt_scene* scene;
  mt_render_config cfg;
  int nslots = 1;
  std::vector<JobSlot> slots;
  int next = 0;   // slot of the next frame
  int last = -1;  // slot of the last frame
  size_t status_stride = 0;
  unsigned char camera[64];
  int has_camera = 0;
  double frames = 0;                       // passes accumulated in the film
  // nslots > 1: each frame renders into its slot's film from zero, and a merge
  // on the slot's stream adds it into this film in frame order
  float4* d_film = nullptr;
  float4* d_film_c = nullptr;
  std::vector<cudaEvent_t> kev;            // profile: 2 + 3 * max_depth per pass
  unsigned long long* d_totals = nullptr;  // running [primary, extension, shadow, error]
  std::vector<Ctrl> h_ctrl;
  // asynchronous film reads
  static constexpr int kMaxReads = 8;
  struct Read {
    float* host = nullptr;
    int resolve = 0;
    double frames = 0;
    cudaEvent_t ev = nullptr;
  };
  cudaStream_t rstream = nullptr;
  cudaEvent_t rfork = nullptr;
  cudaEvent_t rdone = nullptr;  // the latest read's event: one of reads[].ev
  Read reads[kMaxReads];        // pending reads, oldest at r_head
  int r_head = 0, r_count = 0;
  const float4* film() const { return nslots > 1 ? d_film : slots[0].fb.film; }
  // adaptive light grid (mode 1, scene grid on, environment present)
  unsigned scene_version = 0;
  unsigned tune_version = 0;  // launch-shape version the graphs were captured with
  // benchmark-semantics shading form of the next frames (1 two launches, 0 one),
  // chosen from the last finished frame's bounce-1 survivors; -1 not yet known
  int shade_split = -1;
  int64_t launches = 0;  // kernels of the render passes and film merges issued (mt_job_launches)
  int grid_on = 0, grid_fp64 = 0;
  int nu = 0, nv = 0, rx = 0, ry = 0;
  float* d_grid_func = nullptr;
  float* d_grid_sat = nullptr;
  float* d_grid_accum = nullptr;
  double* d_grid_sat64 = nullptr;
  // CDF tables of the grid-guided sampling: per cell (rebuilt with the cells'
  // SATs) and per tile of the map
  float *d_cell_marg = nullptr, *d_cell_cond = nullptr, *d_tile_marg = nullptr, *d_tile_cond = nullptr;
  int grid_tables = 1;
  int grid_frames = 0;           // frames that have accumulated into the grid since it was set up
  cudaEvent_t grid_ev = nullptr;  // recorded after the last grid update
  // displayed image (mt_image_argb), allocated on first use
  int32_t* d_argb = nullptr;
  float4* d_fb = nullptr;
  double* d_tone_part = nullptr;
  int* d_tone_cnt = nullptr;
  float* d_tone_tot = nullptr;
};

// Resets the job's ARGB image to opaque black (InitIntDataRGB), on the context stream.
void image_reset(mt_job* j);

// Per-pass camera constants of InitCameraRayDataJitter from a 64-byte
// CameraStruct, for a width x height frame.
void camera_constants(const void* cam64, int W, int H, PassParams& pp);

// Makes the context stream wait for every job stream's submitted work.
void join_jobs(mt_context* ctx);
// Waits for all work on the context and its jobs' streams, before device arrays
// that frames read are freed or rewritten.
int quiesce(mt_context* ctx);
// Waits for the requests running on the context's servers' lanes.
void servers_sync(mt_context* ctx);
// Rebuild or drop the scene's derived traversal formats from its FP32 records:
// FP16 records (precision 1), 4-wide FP16 nodes (precision 3), and the wide BVH
// (precision 2, refresh_wide).
int refresh_qnodes(mt_scene* s);
int refresh_wide(mt_scene* s);
// MT_CDF_TABLES=0 turns the CDF tables of environment sampling off (the samplers
// then search the SATs directly; the tables hold the same values).
bool cdf_tables_enabled();
