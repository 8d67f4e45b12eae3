// Merged batches: frames of uneven size (cameras, resolutions, spp) rendered
// through one set of wavefront queues. Pass p of the batch holds every frame
// with more than p passes; its paths are the frames' pixels back to back, so
// each bounce is one launch per kernel for the whole batch instead of one per
// frame. A path keys its samples on its frame's pixel and frame number, as a
// frame rendered alone does (benchmark semantics, full-map environment
// sampling, as served requests): every frame's film equals that frame rendered
// alone, bit for bit. The reference renders one frame at a time; this is the
// batched configuration of the benchmark (jobs of uneven resolution sharing
// global work queues).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "mt_internal.h"

namespace {

void free_bufs(FrameBufs& fb) {
  for (auto* p : {&fb.q_o[0], &fb.q_o[1], &fb.q_d[0], &fb.q_d[1], &fb.thr, &fb.ps, &fb.s_o, &fb.s_d, &fb.s_c,
                  &fb.film, &fb.film_c})
    dfree(*p);
  dfree(fb.hit_t);
  dfree(fb.hit_prim);
  dfree(fb.flag);
  dfree(fb.live);
}

int alloc_bufs(FrameBufs& fb, size_t n) {
  int r = MT_OK;
  for (auto* p : {&fb.q_o[0], &fb.q_o[1], &fb.q_d[0], &fb.q_d[1], &fb.thr, &fb.ps, &fb.s_o, &fb.s_d, &fb.s_c,
                  &fb.film, &fb.film_c})
    if (!r) r = dalloc(p, n);
  if (!r) r = dalloc(&fb.hit_t, n);
  if (!r) r = dalloc(&fb.hit_prim, n);
  if (!r) r = dalloc(&fb.flag, n);
  if (!r) r = dalloc(&fb.live, n);
  return r;
}

}  // namespace

extern "C" int mt_batch_render(mt_context* ctx, mt_scene* s, const mt_batch_frame* frames, int nframes, int max_depth,
                               int rr_depth, int film_kahan, float* films_out, int64_t* rays_out) {
  if (!ctx || !s || !frames || !films_out || nframes <= 0) return fail(MT_ERR_INVALID, "bad argument");
  if (s->ctx != ctx) return fail(MT_ERR_INVALID, "scene belongs to another context");
  if (!s->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH");
  if (max_depth < 1 || max_depth > kMaxDepth) return fail(MT_ERR_INVALID, "max_depth %d (1..%d)", max_depth, kMaxDepth);
  size_t total = 0;
  int max_spp = 0;
  for (int k = 0; k < nframes; ++k) {
    const mt_batch_frame& f = frames[k];
    if (f.width <= 0 || f.height <= 0 || f.spp <= 0 || f.spp > 4096)
      return fail(MT_ERR_INVALID, "frame %d: %d x %d, %d spp", k, f.width, f.height, f.spp);
    total += (size_t)f.width * f.height;
    max_spp = std::max(max_spp, f.spp);
  }
  if (total > (size_t)INT32_MAX / 2) return fail(MT_ERR_INVALID, "batch of %zu pixels", total);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;

  // per pass: the frames still rendering, their first path, film offset and parameters
  std::vector<int> h_start((size_t)max_spp * (nframes + 1)), h_film((size_t)max_spp * nframes);
  std::vector<PassParams> h_pp((size_t)max_spp * nframes);
  std::vector<int> nact(max_spp), tot(max_spp);
  std::vector<size_t> film_off(nframes);
  for (int k = 0, off = 0; k < nframes; ++k) {
    film_off[k] = (size_t)off;
    off += frames[k].width * frames[k].height;
  }
  for (int p = 0; p < max_spp; ++p) {
    int n = 0, g = 0;
    for (int k = 0; k < nframes; ++k) {
      const mt_batch_frame& f = frames[k];
      if (f.spp <= p) continue;
      PassParams& pp = h_pp[(size_t)p * nframes + n];
      std::memset(&pp, 0, sizeof(pp));
      camera_constants(f.camera, f.width, f.height, pp);
      pp.frame_count = f.frame_count + (float)p;
      pp.width = f.width;
      pp.height = f.height;
      pp.max_depth = max_depth;
      pp.mode = 1;
      pp.rr_depth = rr_depth;
      pp.kahan = film_kahan;
      pp.grid_accum = 0;
      h_start[(size_t)p * (nframes + 1) + n] = g;
      h_film[(size_t)p * nframes + n] = (int)film_off[k];
      g += f.width * f.height;
      ++n;
    }
    h_start[(size_t)p * (nframes + 1) + n] = g;
    nact[p] = n;
    tot[p] = g;
  }

  FrameBufs fb{};
  Ctrl* d_ctrl = nullptr;
  int *d_start = nullptr, *d_film = nullptr;
  PassParams* d_pp = nullptr;
  unsigned long long* d_totals = nullptr;
  int r = alloc_bufs(fb, total);
  if (!r) r = dalloc(&d_ctrl, (size_t)max_spp);
  if (!r) r = dalloc(&d_start, h_start.size());
  if (!r) r = dalloc(&d_film, h_film.size());
  if (!r) r = dalloc(&d_pp, h_pp.size());
  if (!r) r = dalloc(&d_totals, 4);
  auto done = [&](int code) {
    cudaStreamSynchronize(st);
    free_bufs(fb);
    dfree(d_ctrl);
    dfree(d_start);
    dfree(d_film);
    dfree(d_pp);
    dfree(d_totals);
    return code;
  };
  if (r) return done(r);
  cudaError_t e = cudaMemsetAsync(fb.film, 0, total * 16, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(fb.film_c, 0, total * 16, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl) * (size_t)max_spp, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_totals, 0, 32, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_start, h_start.data(), h_start.size() * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_film, h_film.data(), h_film.size() * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_pp, h_pp.data(), h_pp.size() * sizeof(PassParams), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return done(fail(MT_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e)));
  const DevScene S = s->view();
  const DevEnv E = s->env_view();  // full-map environment sampling
  // every pass of the batch (per pass: raygen, per bounce closest hits, shading
  // and shadow rays, ray totals) captured into one CUDA graph and launched once
  e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return done(fail(MT_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e)));
  int lr = 0;
  for (int p = 0; p < max_spp && !lr; ++p)
    lr = launch_batch_pass(st, S, E, d_start + (size_t)p * (nframes + 1), d_film + (size_t)p * nframes,
                           d_pp + (size_t)p * nframes, nact[p], tot[p], max_depth, film_kahan, d_ctrl + p, fb,
                           ctx->num_sms, d_totals);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(st, &graph);
  if (lr || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return done(fail(MT_ERR_CUDA, "batch pass capture: %s", cudaGetErrorString(lr ? cudaGetLastError() : e)));
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (exec) cudaGraphExecDestroy(exec);  // released once the launch completes
  if (e != cudaSuccess) return done(fail(MT_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e)));
  unsigned long long h_tot[4] = {0, 0, 0, 0};
  e = cudaMemcpyAsync(films_out, fb.film, total * 16, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_tot, d_totals, 32, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(fail(MT_ERR_CUDA, "batch: %s", cudaGetErrorString(e)));
  if (h_tot[3]) return done(fail(MT_ERR_DEVICE, "batch: device error %llu", h_tot[3]));
  if (rays_out)
    for (int i = 0; i < 3; ++i) rays_out[i] = (int64_t)h_tot[i];
  return done(MT_OK);
}
