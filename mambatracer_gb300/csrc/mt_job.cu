// Render jobs: film and path state resident on the device, frames enqueued on
// one stream per in-flight slot (see mt_render_config.inflight).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>

#include "mt_internal.h"

namespace {
struct CamF {  // CameraStruct, Util.cl:78-85
  float position[4], lookat[4], up[4], dimension[2], fov, pad;
};
}  // namespace

// Camera constants of InitCameraRayDataJitter (Initialize.cl:129-172) and
// camera_transform (Matrix.cl:216-241), computed once per pass on the host in
// FP32 with the reference's operation order.
void camera_constants(const void* cam64, int W, int H, PassParams& pp) {
  CamF c;
  std::memcpy(&c, cam64, sizeof(CamF));
  auto dot4 = [](const float* a, const float* b) { return ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]) + a[3] * b[3]; };
  auto norm4 = [&](float* v) {
    float l = std::sqrt(dot4(v, v));
    for (int i = 0; i < 4; ++i) v[i] = v[i] / l;
  };
  auto cross4 = [](const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
    o[3] = 0.f;
  };
  float d[4], r[4], u[4];
  for (int i = 0; i < 4; ++i) d[i] = c.lookat[i] - c.position[i];
  norm4(d);
  cross4(d, c.up, r);
  norm4(r);
  cross4(r, d, u);
  float eInv[4][4] = {{1, 0, 0, c.position[0]}, {0, 1, 0, c.position[1]}, {0, 0, 1, c.position[2]}, {0, 0, 0, 1}};
  float nd[4] = {d[0] * -1.f, d[1] * -1.f, d[2] * -1.f, d[3] * -1.f};
  float v2w[4][4];
  for (int row = 0; row < 4; ++row) {
    v2w[row][0] = r[row];
    v2w[row][1] = u[row];
    v2w[row][2] = nd[row];
    v2w[row][3] = row == 3 ? 1.f : 0.f;
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float col[4] = {v2w[0][j], v2w[1][j], v2w[2][j], v2w[3][j]};
      pp.cam_m[4 * i + j] = dot4(eInv[i], col);
    }
  float dimx = (float)W, dimy = (float)H;
  float fov_rad = c.fov * 0.017453292519943295f;
  pp.cam_d = 1.f / std::tan(fov_rad / 2.f);
  pp.cam_a = dimx / dimy;
  pp.inv_w = 1.f / dimx;
  pp.inv_h = 1.f / dimy;
  pp.dim_w = dimx;
  pp.dim_h = dimy;
  for (int i = 0; i < 4; ++i) pp.cam_pos[i] = c.position[i];
}

namespace {

// Adds one frame's film (rendered from zero into its slot's film) into the
// job's film. With Kahan adds on, the slot film's value is film - film_c and
// the add into the job's film is compensated too.
__global__ void k_film_merge(const float4* __restrict__ f, const float4* __restrict__ fc, int kahan, size_t n,
                             float4* __restrict__ acc, float4* __restrict__ comp) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 v = f[i];
  float4 a = acc[i];
  if (!kahan) {
    acc[i] = make_float4(a.x + v.x, a.y + v.y, a.z + v.z, a.w + v.w);
    return;
  }
  const float4 vc = fc[i];
  v = make_float4(v.x - vc.x, v.y - vc.y, v.z - vc.z, v.w - vc.w);
  const float4 c = comp[i];
  const float4 y = make_float4(v.x - c.x, v.y - c.y, v.z - c.z, v.w - c.w);
  const float4 t = make_float4(a.x + y.x, a.y + y.y, a.z + y.z, a.w + y.w);
  comp[i] = make_float4((t.x - a.x) - y.x, (t.y - a.y) - y.y, (t.z - a.z) - y.z, (t.w - a.w) - y.w);
  acc[i] = t;
}

void free_slot(JobSlot& s) {
  for (int k = 0; k < 2; ++k) {
    dfree(s.fb.q_o[k]);
    dfree(s.fb.q_d[k]);
  }
  dfree(s.fb.hit_t);
  dfree(s.fb.hit_prim);
  dfree(s.fb.thr);
  dfree(s.fb.ps);
  dfree(s.fb.flag);
  dfree(s.fb.s_o);
  dfree(s.fb.s_d);
  dfree(s.fb.s_c);
  dfree(s.fb.film);
  dfree(s.fb.film_c);
  dfree(s.fb.live);
  dfree(s.d_ctrl);
  dfree(s.d_status);
  dfree(s.d_pp);
  if (s.h_pp) cudaFreeHost(s.h_pp);
  s.h_pp = nullptr;
  for (cudaGraphExec_t& g : s.graphs) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  for (cudaEvent_t* e : {&s.fork, &s.ev0, &s.ev1, &s.done, &s.sfork, &s.sjoin}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  if (s.stream) cudaStreamDestroy(s.stream);
  s.stream = nullptr;
  if (s.side) cudaStreamDestroy(s.side);
  s.side = nullptr;
}

void free_job(mt_job* j) {
  for (JobSlot& s : j->slots) free_slot(s);
  j->slots.clear();
  dfree(j->d_totals);
  dfree(j->d_film);
  dfree(j->d_film_c);
  dfree(j->d_grid_func);
  dfree(j->d_grid_sat);
  dfree(j->d_grid_accum);
  dfree(j->d_grid_sat64);
  dfree(j->d_cell_marg);
  dfree(j->d_cell_cond);
  dfree(j->d_tile_marg);
  dfree(j->d_tile_cond);
  dfree(j->d_argb);
  dfree(j->d_fb);
  dfree(j->d_tone_part);
  dfree(j->d_tone_cnt);
  dfree(j->d_tone_tot);
  if (j->grid_ev) cudaEventDestroy(j->grid_ev);
  j->grid_ev = nullptr;
  if (j->rfork) cudaEventDestroy(j->rfork);
  j->rfork = nullptr;
  for (auto& rd : j->reads) {
    if (rd.ev) cudaEventDestroy(rd.ev);
    rd.ev = nullptr;
  }
  j->rdone = nullptr;
  if (j->rstream) cudaStreamDestroy(j->rstream);
  j->rstream = nullptr;
  for (auto& e : j->kev)
    if (e) cudaEventDestroy(e);
  j->kev.clear();
}

int check_cfg(const mt_render_config* c) {
  if (!c) return fail(MT_ERR_INVALID, "NULL config");
  if (c->width <= 0 || c->height <= 0 || (long long)c->width * c->height > (1ll << 30))
    return fail(MT_ERR_INVALID, "resolution %dx%d", c->width, c->height);
  if (c->max_depth < 1 || c->max_depth > kMaxDepth) return fail(MT_ERR_INVALID, "max_depth %d (1..%d)", c->max_depth, kMaxDepth);
  if (c->mode != 0 && c->mode != 1) return fail(MT_ERR_INVALID, "mode %d", c->mode);
  if (c->spp < 1 || c->spp > 4096) return fail(MT_ERR_INVALID, "spp %d", c->spp);
  if (c->inflight < 0 || c->inflight > 8) return fail(MT_ERR_INVALID, "inflight %d (0..8)", c->inflight);
  if (c->grid_updates < 0) return fail(MT_ERR_INVALID, "grid_updates %d", c->grid_updates);
  return MT_OK;
}

int alloc_slot(JobSlot& s, size_t N, int spp, int max_depth, size_t status_stride) {
  int r = MT_OK;
  for (int k = 0; k < 2 && !r; ++k) {
    r = dalloc(&s.fb.q_o[k], N);
    if (!r) r = dalloc(&s.fb.q_d[k], N);
  }
  if (!r) r = dalloc(&s.fb.hit_t, N);
  if (!r) r = dalloc(&s.fb.hit_prim, N);
  if (!r) r = dalloc(&s.fb.thr, N);
  if (!r) r = dalloc(&s.fb.ps, N);
  if (!r) r = dalloc(&s.fb.flag, N);
  if (!r) r = dalloc(&s.fb.s_o, N);
  if (!r) r = dalloc(&s.fb.s_d, N);
  if (!r) r = dalloc(&s.fb.s_c, N);
  if (!r) r = dalloc(&s.fb.film, N);
  if (!r) r = dalloc(&s.fb.film_c, N);
  if (!r) r = dalloc(&s.fb.live, N);
  if (!r) r = dalloc(&s.d_ctrl, (size_t)spp);
  if (!r) r = dalloc(&s.d_status, status_stride * (size_t)max_depth * spp);
  if (!r) r = dalloc(&s.d_pp, (size_t)spp);
  if (!r && cudaMallocHost((void**)&s.h_pp, sizeof(PassParams) * spp) != cudaSuccess)
    r = fail(MT_ERR_NOMEM, "pinned pass parameters");
  if (!r && cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  if (!r && cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  for (cudaEvent_t* e : {&s.fork, &s.ev0, &s.ev1, &s.done})
    if (!r && cudaEventCreate(e) != cudaSuccess) r = fail(MT_ERR_CUDA, "event create");
  for (cudaEvent_t* e : {&s.sfork, &s.sjoin})
    if (!r && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) r = fail(MT_ERR_CUDA, "event create");
  if (!r) std::memset(s.h_pp, 0, sizeof(PassParams) * spp);
  return r;
}

// Sets up the job's light grid from the scene (CAdaptiveEnvironment.setHDRLuminance,
// src/cl/algorithms/CAdaptiveEnvironment.java:69-84): initial func from the
// environment map, accumulation cleared, per-cell SATs built. Runs on the
// context stream with the job's frames finished.
int setup_grid(mt_job* j) {
  mt_scene* sc = j->scene;
  mt_context* ctx = j->ctx;
  const bool want = j->cfg.mode == 1 && sc->grid_on && sc->env_present;
  const bool same = want && j->grid_on && j->nu == sc->grid_nu && j->nv == sc->grid_nv && j->rx == sc->grid_rx &&
                    j->ry == sc->grid_ry && j->grid_fp64 == (sc->grid_on == 2);
  if (!same) {
    dfree(j->d_grid_func);
    dfree(j->d_grid_sat);
    dfree(j->d_grid_accum);
    dfree(j->d_grid_sat64);
    dfree(j->d_cell_marg);
    dfree(j->d_cell_cond);
    dfree(j->d_tile_marg);
    dfree(j->d_tile_cond);
    j->grid_on = 0;
  }
  j->grid_frames = 0;
  j->grid_tables = cdf_tables_enabled();
  if (!want) return MT_OK;
  if (sc->env_w % sc->grid_rx || sc->env_h % sc->grid_ry)
    return fail(MT_ERR_INVALID, "light-grid tiles (%d x %d) must divide the %d x %d environment map", sc->grid_rx,
                sc->grid_ry, sc->env_w, sc->env_h);
  const size_t n = (size_t)sc->grid_nu * sc->grid_nv;
  int r = MT_OK;
  if (!same) {
    j->nu = sc->grid_nu;
    j->nv = sc->grid_nv;
    j->rx = sc->grid_rx;
    j->ry = sc->grid_ry;
    j->grid_fp64 = sc->grid_on == 2;
    r = dalloc(&j->d_grid_func, n);
    if (!r) r = dalloc(&j->d_grid_sat, n);
    if (!r) r = dalloc(&j->d_grid_accum, n);
    if (!r && j->grid_fp64) r = dalloc(&j->d_grid_sat64, n);
    size_t cm = 0, tm = 0;
    const size_t cc = cell_table_floats(j->nu, j->nv, j->rx, j->ry, &cm);
    const size_t tc = tile_table_floats(sc->env_w, sc->env_h, j->rx, j->ry, &tm);
    if (!r) r = dalloc(&j->d_cell_marg, cm);
    if (!r) r = dalloc(&j->d_cell_cond, cc);
    if (!r) r = dalloc(&j->d_tile_marg, tm);
    if (!r) r = dalloc(&j->d_tile_cond, tc);
    if (r) return r;
  }
  CU(cudaMemsetAsync(j->d_grid_accum, 0, n * 4, ctx->stream));
  if (launch_grid_init(ctx->stream, sc->d_env_sat64, sc->d_env_sat, sc->env_w, sc->env_h, j->nu, j->nv, j->rx, j->ry,
                       j->d_grid_func) ||
      launch_grid_sat(ctx->stream, j->d_grid_func, j->d_grid_sat, j->d_grid_sat64, j->nu, j->nv, j->rx, j->ry,
                      j->grid_fp64) ||
      launch_cell_tables(ctx->stream, j->d_grid_sat, j->nu, j->nv, j->rx, j->ry, j->d_cell_marg, j->d_cell_cond) ||
      launch_tile_tables(ctx->stream, sc->d_env_sat, sc->env_w, sc->env_h, j->rx, j->ry, j->d_tile_marg,
                         j->d_tile_cond))
    return fail(MT_ERR_CUDA, "light-grid set-up launch: %s", cudaGetErrorString(cudaGetLastError()));
  j->grid_on = 1;
  return MT_OK;
}

}  // namespace

extern "C" int mt_job_create(mt_context* ctx, mt_scene* scene, const mt_render_config* cfg, mt_job** out) {
  if (!ctx || !scene || !out) return fail(MT_ERR_INVALID, "NULL argument");
  int r = check_cfg(cfg);
  if (r) return r;
  if (!scene->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH (mt_bvh_build / mt_bvh_import)");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  auto* j = new mt_job();
  j->ctx = ctx;
  j->scene = scene;
  j->cfg = *cfg;
  j->nslots = (cfg->profile || cfg->inflight < 1) ? 1 : cfg->inflight;
  const size_t N = (size_t)cfg->width * cfg->height;
  j->status_stride = (N + kShadeThreads - 1) / kShadeThreads;
  j->slots.resize(j->nslots);
  for (JobSlot& s : j->slots)
    if (!r) r = alloc_slot(s, N, cfg->spp, cfg->max_depth, j->status_stride);
  if (!r) r = dalloc(&j->d_totals, 4);
  if (!r && j->nslots > 1) r = dalloc(&j->d_film, N);
  if (!r && j->nslots > 1) r = dalloc(&j->d_film_c, N);
  if (!r && cudaStreamCreateWithFlags(&j->rstream, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  if (!r && cudaEventCreateWithFlags(&j->rfork, cudaEventDisableTiming) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "event create");
  if (!r && cudaEventCreateWithFlags(&j->grid_ev, cudaEventDisableTiming) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "event create");
  if (!r) {
    j->scene_version = scene->version;
    r = setup_grid(j);
  }
  for (auto& rd : j->reads)
    if (!r && cudaEventCreateWithFlags(&rd.ev, cudaEventDisableTiming) != cudaSuccess)
      r = fail(MT_ERR_CUDA, "event create");
  if (!r) j->rdone = j->reads[0].ev;
  if (!r && cfg->profile) {
    j->kev.resize((size_t)cfg->spp * (2 + 3 * cfg->max_depth));
    for (auto& e : j->kev)
      if (!r && cudaEventCreate(&e) != cudaSuccess) r = fail(MT_ERR_CUDA, "event create");
  }
  if (r) {
    std::string keep = mt_last_error();
    free_job(j);
    delete j;
    fail(r, "%s", keep.c_str());
    return r;
  }
  j->h_ctrl.resize(cfg->spp);
  for (JobSlot& s : j->slots) {
    cudaMemsetAsync(s.fb.film, 0, N * 16, ctx->stream);
    cudaMemsetAsync(s.fb.film_c, 0, N * 16, ctx->stream);
  }
  if (j->nslots > 1) {
    cudaMemsetAsync(j->d_film, 0, N * 16, ctx->stream);
    cudaMemsetAsync(j->d_film_c, 0, N * 16, ctx->stream);
  }
  cudaMemsetAsync(j->d_totals, 0, 32, ctx->stream);
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->jobs.push_back(j);
  *out = j;
  return MT_OK;
}

extern "C" int mt_job_destroy(mt_job* j) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  {
    mt_context* ctx = j->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    join_jobs(ctx);
    cudaStreamSynchronize(ctx->stream);
    if (j->rstream) cudaStreamSynchronize(j->rstream);
    ctx->jobs.erase(std::remove(ctx->jobs.begin(), ctx->jobs.end(), j), ctx->jobs.end());
    free_job(j);
  }
  delete j;
  return MT_OK;
}

extern "C" int mt_job_set_camera(mt_job* j, const void* camera) {
  if (!j || !camera) return fail(MT_ERR_INVALID, "NULL argument");
  std::memcpy(j->camera, camera, 64);
  j->has_camera = 1;
  return MT_OK;
}

namespace {
// Enqueue one frame's passes on the slot's stream.
int enqueue_frame(mt_job* j, JobSlot& s) {
  mt_context* ctx = j->ctx;
  const mt_render_config& c = j->cfg;
  DevScene S = j->scene->view();
  DevEnv E = j->scene->env_view();
  if (j->grid_on) {
    E.grid_on = 1;
    E.grid_func = j->d_grid_func;
    E.grid_sat = j->d_grid_sat;
    E.grid_accum = j->d_grid_accum;
    E.nu = j->nu;
    E.nv = j->nv;
    E.rx = j->rx;
    E.ry = j->ry;
    if (j->grid_tables) {
      E.cell_marg = j->d_cell_marg;
      E.cell_cond = j->d_cell_cond;
      E.tile_marg = j->d_tile_marg;
      E.tile_cond = j->d_tile_cond;
    }
  }
  const size_t per_pass_events = 2 + 3 * (size_t)c.max_depth;
  if (j->nslots > 1) {
    const size_t N = (size_t)c.width * c.height;
    CU(cudaMemsetAsync(s.fb.film, 0, N * 16, s.stream));
    CU(cudaMemsetAsync(s.fb.film_c, 0, N * 16, s.stream));
  }
  for (int p = 0; p < c.spp; ++p) {
    CU(cudaMemcpyAsync(s.d_pp + p, s.h_pp + p, sizeof(PassParams), cudaMemcpyHostToDevice, s.stream));
    CU(cudaMemsetAsync(s.d_ctrl + p, 0, sizeof(Ctrl), s.stream));
    CU(cudaMemsetAsync(s.d_status + j->status_stride * (size_t)c.max_depth * p, 0,
                       j->status_stride * (size_t)c.max_depth * 8, s.stream));
    cudaEvent_t* ev = j->kev.empty() ? nullptr : j->kev.data() + per_pass_events * p;
    if (launch_pass(s.stream, S, E, s.d_pp + p, c.mode, c.max_depth, c.film_kahan, c.width, c.height, s.d_ctrl + p,
                    s.fb, s.d_status + j->status_stride * (size_t)c.max_depth * p, j->status_stride, ctx->num_sms,
                    ev, j->d_totals, j->nslots > 1, s.side, s.sfork, s.sjoin, j->shade_split))
      return fail(MT_ERR_CUDA, "pass launch: %s", cudaGetErrorString(cudaGetLastError()));
  }
  return MT_OK;
}
}  // namespace

extern "C" int mt_render_frame(mt_job* j, const int32_t* seeds, float frame_count) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  if (!j->has_camera) return fail(MT_ERR_INVALID, "camera not set (mt_job_set_camera)");
  const mt_render_config& c = j->cfg;
  if (c.mode == 0 && !seeds) return fail(MT_ERR_INVALID, "mode 0 needs the allocateState seed pairs");
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  if (j->scene_version != j->scene->version) {
    // The scene's arrays or grid configuration changed (the change waited for
    // every frame): recapture the graphs and set the light grid up again.
    for (JobSlot& t : j->slots)
      for (cudaGraphExec_t& g : t.graphs)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
    int r = setup_grid(j);
    if (r) return r;
    j->scene_version = j->scene->version;
  }
  if (j->tune_version != tuning_version()) {
    // new launch shapes: capture the frames' graphs again, once their frames ran
    for (JobSlot& t : j->slots)
      for (cudaGraphExec_t& g : t.graphs)
        if (g) {
          CU(cudaStreamSynchronize(t.stream));
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
    j->tune_version = tuning_version();
  }
  JobSlot& s = j->slots[j->next];
  // The slot's previous frame must have consumed its pinned parameters; frames
  // on the other slots keep running meanwhile.
  CU(cudaEventSynchronize(s.done));
  const int split_setting = shade_split_setting();
  if (split_setting >= 0) {
    j->shade_split = split_setting;
  } else if (c.mode == 1 && c.max_depth >= 2) {
    // One launch or two for the shading of the next frames: a finished frame's
    // share of bounce-1 paths that went on decides (shade_split_for): this slot's
    // last frame, or, while nothing is decided yet, the job's latest frame once it
    // has finished. Both forms render the same film, and each slot holds a graph
    // of each (both captured at its first frame), so a change costs nothing.
    JobSlot* src = s.ran ? &s : nullptr;
    if (!src && j->shade_split < 0 && j->last >= 0 && j->slots[j->last].ran) {
      const cudaError_t q = cudaEventQuery(j->slots[j->last].done);
      if (q == cudaSuccess) src = &j->slots[j->last];
      else if (q != cudaErrorNotReady) return fail(MT_ERR_CUDA, "frame event: %s", cudaGetErrorString(q));
    }
    if (src) {
      int counts[3] = {0, 0, 0};
      CU(cudaMemcpyAsync(counts, src->d_ctrl, sizeof(counts), cudaMemcpyDeviceToHost, src->stream));
      CU(cudaStreamSynchronize(src->stream));
      j->shade_split = shade_split_for(counts[1], counts[2], j->shade_split < 0 ? 1 : j->shade_split);
    }
  }
  // CDeviceGI.loop updates the grid after each of its first frames
  // (src/cl/device/CDeviceGI.java:263-264): those frames accumulate.
  const int accumulate = j->grid_on && j->grid_frames < c.grid_updates;
  const int per_pass = 2 * (1 + 2 * c.max_depth);
  for (int p = 0; p < c.spp; ++p) {
    PassParams& pp = s.h_pp[p];
    camera_constants(j->camera, c.width, c.height, pp);
    pp.frame_count = frame_count + (float)p;
    pp.width = c.width;
    pp.height = c.height;
    pp.max_depth = c.max_depth;
    pp.mode = c.mode;
    pp.rr_depth = c.rr_depth;
    pp.kahan = c.film_kahan;
    pp.grid_accum = accumulate;
    if (c.mode == 0) std::memcpy(pp.seeds, seeds + (size_t)per_pass * p, sizeof(int32_t) * per_pass);
  }
  // order after work already on the context stream (film clears, uploads)
  CU(cudaEventRecord(s.fork, ctx->stream));
  CU(cudaStreamWaitEvent(s.stream, s.fork, 0));
  if (j->nslots == 1) CU(cudaStreamWaitEvent(s.stream, j->rdone, 0));
  if (j->grid_on) CU(cudaStreamWaitEvent(s.stream, j->grid_ev, 0));  // the last grid update
  CU(cudaEventRecord(s.ev0, s.stream));
  if (c.use_graph && !c.profile) {
    const int form = j->shade_split == 0 ? 0 : 1;
    const bool both = split_setting < 0 && c.mode == 1;  // the job may switch forms later
    for (int f = 0; f < 2; ++f) {
      if (s.graphs[f] || (f != form && !both)) continue;
      const int keep = j->shade_split;
      j->shade_split = f;
      cudaGraph_t g;
      CU(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
      int r = enqueue_frame(j, s);
      cudaError_t e = cudaStreamEndCapture(s.stream, &g);
      j->shade_split = keep;
      if (r) return r;
      if (e != cudaSuccess) return fail(MT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&s.graphs[f], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(MT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    CU(cudaGraphLaunch(s.graphs[form], s.stream));
  } else {
    int r = enqueue_frame(j, s);
    if (r) return r;
  }
  s.ran = true;
  {
    // per pass: raygen, per bounce closest hits + shading (one launch or two) +
    // shadow rays, the ray totals; then the film merge
    const int two = c.mode == 1 && (j->shade_split < 0 ? shade_split_setting() != 0 : j->shade_split != 0);
    j->launches += (int64_t)c.spp * (2 + (int64_t)c.max_depth * (3 + two)) + (j->nslots > 1 ? 1 : 0);
  }
  CU(cudaEventRecord(s.ev1, s.stream));
  if (accumulate) {
    // CAdaptiveEnvironment.update (CAdaptiveEnvironment.java:128-137): func = accum,
    // per-cell SATs rebuilt; later frames wait for it.
    const size_t n = (size_t)j->nu * j->nv;
    CU(cudaMemcpyAsync(j->d_grid_func, j->d_grid_accum, n * 4, cudaMemcpyDeviceToDevice, s.stream));
    if (launch_grid_sat(s.stream, j->d_grid_func, j->d_grid_sat, j->d_grid_sat64, j->nu, j->nv, j->rx, j->ry,
                        j->grid_fp64) ||
        launch_cell_tables(s.stream, j->d_grid_sat, j->nu, j->nv, j->rx, j->ry, j->d_cell_marg, j->d_cell_cond))
      return fail(MT_ERR_CUDA, "light-grid update launch: %s", cudaGetErrorString(cudaGetLastError()));
    CU(cudaEventRecord(j->grid_ev, s.stream));
    ++j->grid_frames;
  }
  if (j->nslots > 1) {
    // Add the frame into the job's film after the previous frame's add (frame
    // order) and after any film read still copying it out.
    if (j->last >= 0) CU(cudaStreamWaitEvent(s.stream, j->slots[j->last].done, 0));
    CU(cudaStreamWaitEvent(s.stream, j->rdone, 0));
    const size_t N = (size_t)c.width * c.height;
    k_film_merge<<<(unsigned)((N + 255) / 256), 256, 0, s.stream>>>(s.fb.film, s.fb.film_c, c.film_kahan, N,
                                                                    j->d_film, j->d_film_c);
    CU(cudaGetLastError());
  }
  CU(cudaEventRecord(s.done, s.stream));
  j->last = j->next;
  j->next = (j->next + 1) % j->nslots;
  j->frames += c.spp;
  return MT_OK;
}

extern "C" int mt_job_last_ms(mt_job* j, float* ms) {
  if (!j || !ms) return fail(MT_ERR_INVALID, "NULL argument");
  if (j->last < 0) return fail(MT_ERR_INVALID, "no frame rendered yet");
  JobSlot& s = j->slots[j->last];
  CU(cudaEventSynchronize(s.ev1));
  CU(cudaEventElapsedTime(ms, s.ev0, s.ev1));
  return MT_OK;
}

extern "C" int mt_job_total_rays(mt_job* j, int64_t* rays3) {
  if (!j || !rays3) return fail(MT_ERR_INVALID, "NULL argument");
  std::lock_guard<std::recursive_mutex> lk(j->ctx->mu);
  CU(cudaSetDevice(j->ctx->device));
  join_jobs(j->ctx);
  unsigned long long t[4];
  CU(cudaMemcpyAsync(t, j->d_totals, 32, cudaMemcpyDeviceToHost, j->ctx->stream));
  CU(cudaStreamSynchronize(j->ctx->stream));
  for (int k = 0; k < 3; ++k) rays3[k] = (int64_t)t[k];
  if (t[3]) return fail(MT_ERR_DEVICE, "device error %llu latched", t[3]);
  return MT_OK;
}

extern "C" int mt_job_launches(mt_job* j, int64_t* n) {
  if (!j || !n) return fail(MT_ERR_INVALID, "NULL argument");
  *n = j->launches;
  return MT_OK;
}

extern "C" int mt_job_kernel_ms(mt_job* j, float* ms) {
  if (!j || !ms) return fail(MT_ERR_INVALID, "NULL argument");
  if (j->kev.empty()) return fail(MT_ERR_INVALID, "job was not created with profile = 1");
  if (j->last < 0) return fail(MT_ERR_INVALID, "no frame rendered yet");
  CU(cudaEventSynchronize(j->slots[j->last].ev1));
  const mt_render_config& c = j->cfg;
  const size_t per = 2 + 3 * (size_t)c.max_depth;
  for (int p = 0; p < c.spp; ++p)
    for (size_t k = 0; k + 1 < per; ++k)
      CU(cudaEventElapsedTime(ms + (size_t)p * (per - 1) + k, j->kev[p * per + k], j->kev[p * per + k + 1]));
  return MT_OK;
}

extern "C" int mt_job_stats(mt_job* j, int64_t* rays3, int32_t* counts) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  std::lock_guard<std::recursive_mutex> lk(j->ctx->mu);
  CU(cudaSetDevice(j->ctx->device));
  join_jobs(j->ctx);
  CU(cudaStreamSynchronize(j->ctx->stream));
  const mt_render_config& c = j->cfg;
  const JobSlot& s = j->slots[j->last < 0 ? 0 : j->last];
  CU(cudaMemcpy(j->h_ctrl.data(), s.d_ctrl, sizeof(Ctrl) * c.spp, cudaMemcpyDeviceToHost));
  int64_t prim = 0, ext = 0, sh = 0;
  int err = 0;
  for (int p = 0; p < c.spp; ++p) {
    const Ctrl& k = j->h_ctrl[p];
    prim += (int64_t)c.width * c.height;
    for (int b = 2; b <= c.max_depth; ++b) ext += k.count[b];
    sh += (int64_t)k.rays[2];
    if (k.error) err = k.error;
  }
  if (rays3) {
    rays3[0] = prim;
    rays3[1] = ext;
    rays3[2] = sh;
  }
  if (counts) {
    const Ctrl& k = j->h_ctrl[c.spp - 1];
    for (int b = 1; b <= c.max_depth; ++b) counts[b - 1] = k.count[b + 1];
  }
  if (err) return fail(MT_ERR_DEVICE, "device error %d latched during the frame", err);
  return MT_OK;
}

namespace {
// averageAccum (src/cl/kernel/Image.cl:84-122): accum.xyz / frameCount, w = 1
void resolve_film(float* rgba, size_t n, double frames) {
  if (frames <= 0) return;
  const float fc = (float)frames;
  for (size_t i = 0; i < n; ++i) {
    rgba[4 * i + 0] = rgba[4 * i + 0] / fc;
    rgba[4 * i + 1] = rgba[4 * i + 1] / fc;
    rgba[4 * i + 2] = rgba[4 * i + 2] / fc;
    rgba[4 * i + 3] = 1.f;
  }
}

// Completes the oldest pending read: waits for its copy and resolves it.
int finish_oldest_read(mt_job* j) {
  mt_job::Read& rd = j->reads[j->r_head];
  j->r_head = (j->r_head + 1) % mt_job::kMaxReads;
  --j->r_count;
  CU(cudaEventSynchronize(rd.ev));
  if (rd.resolve) resolve_film(rd.host, (size_t)j->cfg.width * j->cfg.height, rd.frames);
  rd.host = nullptr;
  return MT_OK;
}

int finish_reads(mt_job* j) {
  while (j->r_count > 0) {
    int r = finish_oldest_read(j);
    if (r) return r;
  }
  return MT_OK;
}

// Enqueues on the job's read stream a copy of the film as of every frame
// submitted so far; returns the read's entry.
int enqueue_read(mt_job* j, float* rgba, int resolve, mt_job::Read** out) {
  if (j->r_count == mt_job::kMaxReads) {
    int r = finish_oldest_read(j);
    if (r) return r;
  }
  mt_context* ctx = j->ctx;
  mt_job::Read& rd = j->reads[(j->r_head + j->r_count) % mt_job::kMaxReads];
  CU(cudaEventRecord(j->rfork, ctx->stream));
  CU(cudaStreamWaitEvent(j->rstream, j->rfork, 0));
  if (j->last >= 0) CU(cudaStreamWaitEvent(j->rstream, j->slots[j->last].done, 0));
  const size_t N = (size_t)j->cfg.width * j->cfg.height;
  CU(cudaMemcpyAsync(rgba, j->film(), N * 16, cudaMemcpyDeviceToHost, j->rstream));
  CU(cudaEventRecord(rd.ev, j->rstream));
  j->rdone = rd.ev;
  rd.host = rgba;
  rd.resolve = resolve;
  rd.frames = j->frames;
  ++j->r_count;
  *out = &rd;
  return MT_OK;
}
}  // namespace

extern "C" int mt_film_read(mt_job* j, float* rgba, int resolve) {
  if (!j || !rgba) return fail(MT_ERR_INVALID, "NULL argument");
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  mt_job::Read* rd = nullptr;
  int r = enqueue_read(j, rgba, resolve, &rd);
  return r ? r : finish_reads(j);
}

extern "C" int mt_film_read_async(mt_job* j, float* rgba, int resolve) {
  if (!j || !rgba) return fail(MT_ERR_INVALID, "NULL argument");
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  mt_job::Read* rd = nullptr;
  return enqueue_read(j, rgba, resolve, &rd);
}

extern "C" int mt_film_wait(mt_job* j) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  std::lock_guard<std::recursive_mutex> lk(j->ctx->mu);
  CU(cudaSetDevice(j->ctx->device));
  return finish_reads(j);
}

extern "C" int mt_film_clear(mt_job* j) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  int r = finish_reads(j);
  if (r) return r;
  join_jobs(ctx);
  const size_t N = (size_t)j->cfg.width * j->cfg.height;
  for (JobSlot& s : j->slots) {
    CU(cudaMemsetAsync(s.fb.film, 0, N * 16, ctx->stream));
    CU(cudaMemsetAsync(s.fb.film_c, 0, N * 16, ctx->stream));
  }
  if (j->nslots > 1) {
    CU(cudaMemsetAsync(j->d_film, 0, N * 16, ctx->stream));
    CU(cudaMemsetAsync(j->d_film_c, 0, N * 16, ctx->stream));
  }
  CU(cudaMemsetAsync(j->d_totals, 0, 32, ctx->stream));
  image_reset(j);
  j->frames = 0;
  return MT_OK;
}

extern "C" int mt_job_grid_read(mt_job* j, float* func, float* sat, float* accum) {
  if (!j) return fail(MT_ERR_INVALID, "NULL job");
  if (!j->grid_on) return fail(MT_ERR_INVALID, "the job has no light grid (mode 1, scene grid on, environment set)");
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  join_jobs(ctx);
  const size_t n = (size_t)j->nu * j->nv;
  if (func) CU(cudaMemcpyAsync(func, j->d_grid_func, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (sat) CU(cudaMemcpyAsync(sat, j->d_grid_sat, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (accum) CU(cudaMemcpyAsync(accum, j->d_grid_accum, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return MT_OK;
}
