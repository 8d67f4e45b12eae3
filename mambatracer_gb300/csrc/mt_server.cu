// Served and batched rendering: a native scheduler that runs many render
// requests of different scenes, resolutions and sample counts concurrently on
// one GPU.
//
// The reference renders one job at a time on one in-order queue
// (CDeviceGI.loop, src/cl/device/CDeviceGI.java:214-271). Here a request is a
// whole job (spp passes of benchmark-semantics frames) and runs on a lane: a
// stream with path state, queues, film and pass parameters preallocated for the
// largest frame the server takes, so no device memory is allocated or freed
// while requests run (cudaFree would synchronise the device). Up to `lanes`
// requests run at once; their kernels overlap on the GPU (persistent traversal
// grids are sized by the frame, so a small request leaves SMs to the others).
// Admission is first come, first served within a budget of path-state and film
// bytes (196 B per pixel). A completed request's film is copied to pinned
// staging and from there to the caller's buffer by the scheduler thread; a
// host callback on the lane's stream wakes the scheduler, which measures the
// request's latency from submission. Scenes are reference-counted while
// requests use them.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>

#include "mt_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kCancelled = 3, kFailed = 4 };

struct Request {
  int64_t id = 0;
  mt_scene* scene = nullptr;
  unsigned char camera[64];
  int width = 0, height = 0, spp = 0;
  float frame_count = 1.f;
  float* film_out = nullptr;
  int state = kQueued;
  bool cancel = false;
  size_t bytes = 0;
  Clock::time_point t_submit, t_start, t_done;
  std::string error;
};

struct Lane {
  cudaStream_t stream = nullptr;
  FrameBufs fb{};
  Ctrl* d_ctrl = nullptr;
  unsigned long long* d_status = nullptr;
  PassParams* h_pp = nullptr;
  PassParams* d_pp = nullptr;
  float4* h_stage = nullptr;  // pinned film staging
  Request* req = nullptr;
  bool finished = false;  // set by the host callback
  struct mt_server* server = nullptr;
};

constexpr size_t kPathBytesPerPixel = 196;

}  // namespace

struct mt_server {
  mt_context* ctx = nullptr;
  mt_server_config cfg{};
  size_t status_stride = 0;
  std::vector<Lane> lanes;
  unsigned long long* d_totals = nullptr;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-ups: submissions, completions, stop
  std::condition_variable done_cv;  // request completions, for waiters
  std::deque<Request*> pending;
  std::map<int64_t, Request*> all;
  int64_t next_id = 1;
  size_t used_bytes = 0;
  bool stop = false;
  int running = 0;
  std::vector<double> latencies_ms;
  size_t max_queue = 0;
  Clock::time_point t_first_submit, t_last_done;
  bool any_submit = false;
};

namespace {

void CUDART_CB lane_done(void* p) {
  Lane* L = static_cast<Lane*>(p);
  mt_server* s = L->server;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    L->finished = true;
  }
  s->cv.notify_all();
}

void free_lane(Lane& L) {
  for (int k = 0; k < 2; ++k) {
    dfree(L.fb.q_o[k]);
    dfree(L.fb.q_d[k]);
  }
  dfree(L.fb.hit_t);
  dfree(L.fb.hit_prim);
  dfree(L.fb.thr);
  dfree(L.fb.ps);
  dfree(L.fb.flag);
  dfree(L.fb.s_o);
  dfree(L.fb.s_d);
  dfree(L.fb.s_c);
  dfree(L.fb.film);
  dfree(L.fb.film_c);
  dfree(L.d_ctrl);
  dfree(L.d_status);
  dfree(L.d_pp);
  if (L.h_pp) cudaFreeHost(L.h_pp);
  if (L.h_stage) cudaFreeHost(L.h_stage);
  L.h_pp = nullptr;
  L.h_stage = nullptr;
  if (L.stream) cudaStreamDestroy(L.stream);
  L.stream = nullptr;
}

int alloc_lane(Lane& L, size_t N, int spp, int depth, size_t stride) {
  int r = MT_OK;
  for (int k = 0; k < 2 && !r; ++k) {
    r = dalloc(&L.fb.q_o[k], N);
    if (!r) r = dalloc(&L.fb.q_d[k], N);
  }
  if (!r) r = dalloc(&L.fb.hit_t, N);
  if (!r) r = dalloc(&L.fb.hit_prim, N);
  if (!r) r = dalloc(&L.fb.thr, N);
  if (!r) r = dalloc(&L.fb.ps, N);
  if (!r) r = dalloc(&L.fb.flag, N);
  if (!r) r = dalloc(&L.fb.s_o, N);
  if (!r) r = dalloc(&L.fb.s_d, N);
  if (!r) r = dalloc(&L.fb.s_c, N);
  if (!r) r = dalloc(&L.fb.film, N);
  if (!r) r = dalloc(&L.fb.film_c, N);
  if (!r) r = dalloc(&L.d_ctrl, (size_t)spp);
  if (!r) r = dalloc(&L.d_status, stride * (size_t)depth * spp);
  if (!r) r = dalloc(&L.d_pp, (size_t)spp);
  if (!r && cudaMallocHost((void**)&L.h_pp, sizeof(PassParams) * spp) != cudaSuccess)
    r = fail(MT_ERR_NOMEM, "pinned pass parameters");
  if (!r && cudaMallocHost((void**)&L.h_stage, sizeof(float4) * N) != cudaSuccess)
    r = fail(MT_ERR_NOMEM, "pinned film staging");
  if (!r && cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  if (!r) std::memset(L.h_pp, 0, sizeof(PassParams) * spp);
  return r;
}

// Enqueues request R on lane L (scheduler thread, context lock held).
int start_request(mt_server* s, Lane& L, Request* R) {
  const mt_server_config& c = s->cfg;
  const size_t N = (size_t)R->width * R->height;
  for (int p = 0; p < R->spp; ++p) {
    PassParams& pp = L.h_pp[p];
    camera_constants(R->camera, R->width, R->height, pp);
    pp.frame_count = R->frame_count + (float)p;
    pp.width = R->width;
    pp.height = R->height;
    pp.max_depth = c.max_depth;
    pp.mode = 1;
    pp.rr_depth = c.rr_depth;
    pp.kahan = c.film_kahan;
    pp.grid_accum = 0;
  }
  const size_t stride = (N + kShadeThreads - 1) / kShadeThreads;
  CU(cudaMemcpyAsync(L.d_pp, L.h_pp, sizeof(PassParams) * R->spp, cudaMemcpyHostToDevice, L.stream));
  CU(cudaMemsetAsync(L.d_ctrl, 0, sizeof(Ctrl) * R->spp, L.stream));
  CU(cudaMemsetAsync(L.d_status, 0, stride * (size_t)c.max_depth * R->spp * 8, L.stream));
  CU(cudaMemsetAsync(L.fb.film, 0, N * 16, L.stream));
  CU(cudaMemsetAsync(L.fb.film_c, 0, N * 16, L.stream));
  DevScene S = R->scene->view();
  DevEnv E = R->scene->env_view();
  for (int p = 0; p < R->spp; ++p)
    if (launch_pass(L.stream, S, E, L.d_pp + p, 1, c.max_depth, c.film_kahan, R->width, R->height, L.d_ctrl + p,
                    L.fb, L.d_status + stride * (size_t)c.max_depth * p, stride, s->ctx->num_sms, nullptr,
                    s->d_totals, s->lanes.size() > 1))
      return fail(MT_ERR_CUDA, "pass launch: %s", cudaGetErrorString(cudaGetLastError()));
  CU(cudaMemcpyAsync(L.h_stage, L.fb.film, N * 16, cudaMemcpyDeviceToHost, L.stream));
  CU(cudaLaunchHostFunc(L.stream, lane_done, &L));
  return MT_OK;
}

void release_scene(Request* R) {
  if (R->scene) R->scene->refs.fetch_sub(1);
  R->scene = nullptr;
}

void worker_main(mt_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    // completions
    for (Lane& L : s->lanes) {
      if (!L.req || !L.finished) continue;
      Request* R = L.req;
      lk.unlock();
      if (R->film_out && !R->cancel)
        std::memcpy(R->film_out, L.h_stage, (size_t)R->width * R->height * 16);
      lk.lock();
      R->t_done = Clock::now();
      R->state = R->cancel ? kCancelled : kDone;
      if (R->state == kDone)
        s->latencies_ms.push_back(std::chrono::duration<double, std::milli>(R->t_done - R->t_submit).count());
      s->t_last_done = R->t_done;
      s->used_bytes -= R->bytes;
      --s->running;
      release_scene(R);
      L.req = nullptr;
      L.finished = false;
      s->done_cv.notify_all();
    }
    // admissions: first come, first served within the lanes and the byte budget
    while (!s->pending.empty()) {
      Request* R = s->pending.front();
      if (R->cancel) {
        s->pending.pop_front();
        R->state = kCancelled;
        release_scene(R);
        s->done_cv.notify_all();
        continue;
      }
      Lane* free_lane_p = nullptr;
      for (Lane& L : s->lanes)
        if (!L.req) {
          free_lane_p = &L;
          break;
        }
      if (!free_lane_p || (s->running > 0 && s->used_bytes + R->bytes > s->cfg.budget_bytes)) break;
      s->pending.pop_front();
      R->state = kRunning;
      R->t_start = Clock::now();
      s->used_bytes += R->bytes;
      ++s->running;
      free_lane_p->req = R;
      free_lane_p->finished = false;
      lk.unlock();
      int r;
      {
        std::lock_guard<std::recursive_mutex> ck(s->ctx->mu);
        cudaSetDevice(s->ctx->device);
        r = start_request(s, *free_lane_p, R);
      }
      lk.lock();
      if (r) {
        // nothing of this request is left on the lane's stream that could call back
        cudaStreamSynchronize(free_lane_p->stream);
        R->state = kFailed;
        R->error = mt_last_error();
        s->used_bytes -= R->bytes;
        --s->running;
        release_scene(R);
        free_lane_p->req = nullptr;
        s->done_cv.notify_all();
      }
    }
    if (s->stop && s->running == 0) break;
    s->cv.wait(lk, [&] {
      if (s->stop && s->running == 0) return true;
      for (Lane& L : s->lanes)
        if (L.req && L.finished) return true;
      if (s->pending.empty()) return false;
      if (s->pending.front()->cancel) return true;
      for (Lane& L : s->lanes)
        if (!L.req) return s->running == 0 || s->used_bytes + s->pending.front()->bytes <= s->cfg.budget_bytes;
      return false;
    });
  }
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  // nearest rank
  size_t k = (size_t)std::ceil(q * (double)v.size());
  if (k < 1) k = 1;
  if (k > v.size()) k = v.size();
  return v[k - 1];
}

}  // namespace

extern "C" int mt_server_create(mt_context* ctx, const mt_server_config* cfg, mt_server** out) {
  if (!ctx || !cfg || !out) return fail(MT_ERR_INVALID, "NULL argument");
  const mt_server_config& c = *cfg;
  if (c.lanes < 1 || c.lanes > 64) return fail(MT_ERR_INVALID, "lanes %d (1..64)", c.lanes);
  if (c.max_width <= 0 || c.max_height <= 0 || (long long)c.max_width * c.max_height > (1ll << 26))
    return fail(MT_ERR_INVALID, "largest frame %d x %d", c.max_width, c.max_height);
  if (c.max_spp < 1 || c.max_spp > 4096) return fail(MT_ERR_INVALID, "max_spp %d", c.max_spp);
  if (c.max_depth < 1 || c.max_depth > kMaxDepth) return fail(MT_ERR_INVALID, "max_depth %d", c.max_depth);
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  auto* s = new mt_server();
  s->ctx = ctx;
  s->cfg = c;
  if (s->cfg.budget_bytes == 0) s->cfg.budget_bytes = ~(uint64_t)0;
  const size_t N = (size_t)c.max_width * c.max_height;
  s->status_stride = (N + kShadeThreads - 1) / kShadeThreads;
  s->lanes.resize(c.lanes);
  int r = dalloc(&s->d_totals, 4);
  for (Lane& L : s->lanes) {
    L.server = s;
    if (!r) r = alloc_lane(L, N, c.max_spp, c.max_depth, s->status_stride);
  }
  if (!r && cudaMemset(s->d_totals, 0, 32) != cudaSuccess) r = fail(MT_ERR_CUDA, "memset");
  if (r) {
    std::string keep = mt_last_error();
    for (Lane& L : s->lanes) free_lane(L);
    dfree(s->d_totals);
    delete s;
    return fail(r, "%s", keep.c_str());
  }
  s->worker = std::thread(worker_main, s);
  ctx->servers.push_back(s);
  *out = s;
  return MT_OK;
}

extern "C" int mt_server_destroy(mt_server* s) {
  if (!s) return fail(MT_ERR_INVALID, "NULL server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (Request* R : s->pending) R->cancel = true;
    s->stop = true;
  }
  s->cv.notify_all();
  s->worker.join();
  {
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    cudaSetDevice(s->ctx->device);
    for (Lane& L : s->lanes) {
      if (L.stream) cudaStreamSynchronize(L.stream);
      free_lane(L);
    }
    dfree(s->d_totals);
    auto& v = s->ctx->servers;
    v.erase(std::remove(v.begin(), v.end(), s), v.end());
  }
  for (auto& kv : s->all) {
    release_scene(kv.second);
    delete kv.second;
  }
  delete s;
  return MT_OK;
}

extern "C" int mt_job_submit(mt_server* s, mt_scene* scene, const void* camera, int width, int height, int spp,
                             float frame_count, float* film_out, int64_t* id_out) {
  if (!s || !scene || !camera || !id_out) return fail(MT_ERR_INVALID, "NULL argument");
  if (width <= 0 || height <= 0 || (long long)width * height > (long long)s->cfg.max_width * s->cfg.max_height)
    return fail(MT_ERR_INVALID, "frame %d x %d exceeds the server's largest (%d x %d pixels)", width, height,
                s->cfg.max_width, s->cfg.max_height);
  if (spp < 1 || spp > s->cfg.max_spp) return fail(MT_ERR_INVALID, "spp %d (1..%d)", spp, s->cfg.max_spp);
  if (!scene->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH");
  if (scene->ctx != s->ctx) return fail(MT_ERR_INVALID, "scene belongs to another context");
  auto* R = new Request();
  R->scene = scene;
  std::memcpy(R->camera, camera, 64);
  R->width = width;
  R->height = height;
  R->spp = spp;
  R->frame_count = frame_count;
  R->film_out = film_out;
  R->bytes = (size_t)width * height * kPathBytesPerPixel;
  scene->refs.fetch_add(1);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      release_scene(R);
      delete R;
      return fail(MT_ERR_INVALID, "server is shutting down");
    }
    R->id = s->next_id++;
    R->t_submit = Clock::now();
    if (!s->any_submit) {
      s->t_first_submit = R->t_submit;
      s->any_submit = true;
    }
    s->all[R->id] = R;
    s->pending.push_back(R);
    s->max_queue = std::max(s->max_queue, s->pending.size());
    *id_out = R->id;
  }
  s->cv.notify_all();
  return MT_OK;
}

extern "C" int mt_job_poll(mt_server* s, int64_t id, int* state, double* latency_ms) {
  if (!s || !state) return fail(MT_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail(MT_ERR_INVALID, "no request %lld", (long long)id);
  const Request* R = it->second;
  *state = R->state;
  if (latency_ms)
    *latency_ms = (R->state == kDone || R->state == kCancelled)
                      ? std::chrono::duration<double, std::milli>(R->t_done - R->t_submit).count()
                      : -1.0;
  if (R->state == kFailed) return fail(MT_ERR_CUDA, "request %lld failed: %s", (long long)id, R->error.c_str());
  return MT_OK;
}

extern "C" int mt_job_cancel(mt_server* s, int64_t id) {
  if (!s) return fail(MT_ERR_INVALID, "NULL server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return fail(MT_ERR_INVALID, "no request %lld", (long long)id);
    it->second->cancel = true;
  }
  s->cv.notify_all();
  return MT_OK;
}

extern "C" int mt_job_wait(mt_server* s, int64_t id, double timeout_ms) {
  if (!s) return fail(MT_ERR_INVALID, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail(MT_ERR_INVALID, "no request %lld", (long long)id);
  Request* R = it->second;
  auto ready = [&] { return R->state >= kDone; };
  if (timeout_ms < 0)
    s->done_cv.wait(lk, ready);
  else if (!s->done_cv.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
    return fail(MT_ERR_TIMEOUT, "request %lld still %s", (long long)id, R->state == kQueued ? "queued" : "running");
  if (R->state == kFailed) return fail(MT_ERR_CUDA, "request %lld failed: %s", (long long)id, R->error.c_str());
  return MT_OK;
}

extern "C" int mt_server_drain(mt_server* s) {
  if (!s) return fail(MT_ERR_INVALID, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->done_cv.wait(lk, [&] { return s->pending.empty() && s->running == 0; });
  return MT_OK;
}

extern "C" int mt_server_stats(mt_server* s, mt_served_stats* out) {
  if (!s || !out) return fail(MT_ERR_INVALID, "NULL argument");
  std::memset(out, 0, sizeof(*out));
  unsigned long long t[4] = {0, 0, 0, 0};
  {
    std::lock_guard<std::recursive_mutex> ck(s->ctx->mu);
    cudaSetDevice(s->ctx->device);
    CU(cudaMemcpy(t, s->d_totals, 32, cudaMemcpyDeviceToHost));  // device-ordered after the lanes' passes
  }
  std::lock_guard<std::mutex> lk(s->mu);
  out->completed = (int64_t)s->latencies_ms.size();
  int64_t cancelled = 0, failed = 0, queued = 0, running = 0;
  for (auto& kv : s->all) {
    cancelled += kv.second->state == kCancelled;
    failed += kv.second->state == kFailed;
    queued += kv.second->state == kQueued;
    running += kv.second->state == kRunning;
  }
  out->cancelled = cancelled;
  out->failed = failed;
  out->queued = queued;
  out->running = running;
  for (int k = 0; k < 3; ++k) out->rays[k] = (int64_t)t[k];
  out->p50_ms = percentile(s->latencies_ms, 0.50);
  out->p95_ms = percentile(s->latencies_ms, 0.95);
  out->p99_ms = percentile(s->latencies_ms, 0.99);
  out->max_ms = s->latencies_ms.empty() ? 0.0 : *std::max_element(s->latencies_ms.begin(), s->latencies_ms.end());
  out->span_ms = s->any_submit && out->completed
                     ? std::chrono::duration<double, std::milli>(s->t_last_done - s->t_first_submit).count()
                     : 0.0;
  out->max_queue = (int64_t)s->max_queue;
  if (t[3]) return fail(MT_ERR_DEVICE, "device error %llu latched", t[3]);
  return MT_OK;
}

void servers_sync(mt_context* ctx) {
  for (mt_server* s : ctx->servers)
    for (Lane& L : s->lanes)
      if (L.stream) cudaStreamSynchronize(L.stream);
}
