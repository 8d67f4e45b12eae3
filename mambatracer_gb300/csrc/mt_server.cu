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
// bytes (200 B per pixel). A completed request's film is copied to pinned
// staging and from there to the caller's buffer by the scheduler thread; a
// host callback on the lane's stream wakes the scheduler, which measures the
// request's latency from submission. Scenes are reference-counted while
// requests use them.
//
// Merged mode (config `merged` = m >= 1): the running requests share wavefront
// queues instead of a lane each. The slots are split over m merge streams
// (slot k on stream k mod m); each stream works in rounds, a round being, per
// scene, one merged pass (launch_batch_pass) holding the next pass of every
// running request of the stream's slots, so each bounce is one launch per
// kernel for all of them, and the streams overlap one another's last bounces.
// Requests join at their stream's next round and leave when their last pass is
// issued (continuous batching at pass granularity); a cancelled running request
// stops at the next round. Slot k's film is the arena's k-th frame-sized
// region, a stream's path state its slots' share of the arena. Per-round frame
// tables live in a ring of kRounds entries per stream; a host callback at the
// end of each round frees its entry, which also keeps the scheduler at most
// kRounds rounds ahead of the GPU on each stream. A merged pass keys every
// path's samples on its own frame's pixel and frame number, so each film equals
// the request rendered alone, bit for bit.
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
  cudaStream_t side = nullptr;  // shadow rays beside the next bounce's extension rays
  cudaEvent_t sfork = nullptr, sjoin = nullptr;
  FrameBufs fb{};
  Ctrl* d_ctrl = nullptr;
  unsigned long long* d_status = nullptr;
  PassParams* h_pp = nullptr;
  PassParams* d_pp = nullptr;
  float4* h_stage = nullptr;  // pinned film staging
  Request* req = nullptr;
  bool finished = false;  // set by the host callback
  struct mt_server* server = nullptr;
  int pass = 0;         // merged mode: passes of `req` issued so far
  bool issued = false;  // merged mode: the request's completion is on the stream
  int group = -1;       // merged mode: its merge stream
};

// One merged-mode round's frame tables: per scene group the first path of each
// frame and the total (n + 1 ints), the frames' film offsets (n ints), their
// pass parameters, and a control block.
struct Round {
  int* h_tab = nullptr;  // pinned
  PassParams* h_pp = nullptr;
  int* d_tab = nullptr;
  PassParams* d_pp = nullptr;
  Ctrl* d_ctrl = nullptr;
  cudaEvent_t done = nullptr;
  bool used = false;
};

constexpr size_t kPathBytesPerPixel = 200;
constexpr int kRounds = 3;
constexpr size_t kGraphsPerStream = 16;  // scenes whose merged-pass graph a merge stream keeps

// One merge stream: its slots, its share of the queues, its round ring.
struct MergeGroup {
  struct mt_server* server = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<int> slots;
  FrameBufs fb{};  // path state of its slots' paths; the films of the whole arena
  Round rounds[kRounds];
  int next_round = 0;
  int inflight = 0;  // rounds whose end callback has not run (server lock)
  // per scene: the executable graph of its merged pass, updated every round
  std::vector<std::pair<const mt_scene*, cudaGraphExec_t>> graphs;
};

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
  // merged mode
  FrameBufs mfb{};  // queues for lanes x slot_px paths; slot k's film at k x slot_px
  size_t slot_px = 0;
  std::vector<MergeGroup> groups;  // sized once at creation (callbacks hold their addresses)
  std::string broken;  // set when a round failed: later requests fail with it
};

namespace {

void CUDART_CB round_done(void* p) {
  MergeGroup* G = static_cast<MergeGroup*>(p);
  mt_server* s = G->server;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    --G->inflight;
  }
  s->cv.notify_all();
}

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
  dfree(L.fb.live);
  dfree(L.d_ctrl);
  dfree(L.d_status);
  dfree(L.d_pp);
  if (L.h_pp) cudaFreeHost(L.h_pp);
  if (L.h_stage) cudaFreeHost(L.h_stage);
  L.h_pp = nullptr;
  L.h_stage = nullptr;
  if (L.stream) cudaStreamDestroy(L.stream);
  L.stream = nullptr;
  if (L.side) cudaStreamDestroy(L.side);
  L.side = nullptr;
  for (cudaEvent_t* e : {&L.sfork, &L.sjoin}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
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
  if (!r) r = dalloc(&L.fb.live, N);
  if (!r) r = dalloc(&L.d_ctrl, (size_t)spp);
  if (!r) r = dalloc(&L.d_status, stride * (size_t)depth * spp);
  if (!r) r = dalloc(&L.d_pp, (size_t)spp);
  if (!r && cudaMallocHost((void**)&L.h_pp, sizeof(PassParams) * spp) != cudaSuccess)
    r = fail(MT_ERR_NOMEM, "pinned pass parameters");
  if (!r && cudaMallocHost((void**)&L.h_stage, sizeof(float4) * N) != cudaSuccess)
    r = fail(MT_ERR_NOMEM, "pinned film staging");
  if (!r && cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  if (!r && cudaStreamCreateWithFlags(&L.side, cudaStreamNonBlocking) != cudaSuccess)
    r = fail(MT_ERR_CUDA, "stream create");
  for (cudaEvent_t* e : {&L.sfork, &L.sjoin})
    if (!r && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) r = fail(MT_ERR_CUDA, "event create");
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
                    s->d_totals, s->lanes.size() > 1, L.side, L.sfork, L.sjoin))
      return fail(MT_ERR_CUDA, "pass launch: %s", cudaGetErrorString(cudaGetLastError()));
  CU(cudaMemcpyAsync(L.h_stage, L.fb.film, N * 16, cudaMemcpyDeviceToHost, L.stream));
  CU(cudaLaunchHostFunc(L.stream, lane_done, &L));
  return MT_OK;
}

void release_scene(Request* R) {
  if (R->scene) R->scene->refs.fetch_sub(1);
  R->scene = nullptr;
}

void free_merged(mt_server* s) {
  for (auto* p : {&s->mfb.q_o[0], &s->mfb.q_o[1], &s->mfb.q_d[0], &s->mfb.q_d[1], &s->mfb.thr, &s->mfb.ps,
                  &s->mfb.s_o, &s->mfb.s_d, &s->mfb.s_c, &s->mfb.film, &s->mfb.film_c})
    dfree(*p);
  dfree(s->mfb.hit_t);
  dfree(s->mfb.hit_prim);
  dfree(s->mfb.flag);
  dfree(s->mfb.live);
  for (MergeGroup& G : s->groups) {
    for (Round& Rd : G.rounds) {
      if (Rd.h_tab) cudaFreeHost(Rd.h_tab);
      if (Rd.h_pp) cudaFreeHost(Rd.h_pp);
      Rd.h_tab = nullptr;
      Rd.h_pp = nullptr;
      dfree(Rd.d_tab);
      dfree(Rd.d_pp);
      dfree(Rd.d_ctrl);
      if (Rd.done) cudaEventDestroy(Rd.done);
      Rd.done = nullptr;
    }
    for (auto& g : G.graphs)
      if (g.second) cudaGraphExecDestroy(g.second);
    G.graphs.clear();
    if (G.stream) cudaStreamDestroy(G.stream);
    G.stream = nullptr;
  }
}

// Merged mode: the queues for lanes x N paths, the slots' films and pinned
// staging, and per merge stream its slots, its share of the queues, its round
// ring and its stream.
int alloc_merged(mt_server* s, size_t N, int m) {
  const size_t P = N * s->lanes.size();
  const int lanes = (int)s->lanes.size();
  s->groups.resize((size_t)m);
  for (int k = 0; k < lanes; ++k) {
    s->lanes[k].group = k % m;
    s->groups[k % m].slots.push_back(k);
  }
  int r = MT_OK;
  for (auto* p : {&s->mfb.q_o[0], &s->mfb.q_o[1], &s->mfb.q_d[0], &s->mfb.q_d[1], &s->mfb.thr, &s->mfb.ps,
                  &s->mfb.s_o, &s->mfb.s_d, &s->mfb.s_c, &s->mfb.film, &s->mfb.film_c})
    if (!r) r = dalloc(p, P);
  if (!r) r = dalloc(&s->mfb.hit_t, P);
  if (!r) r = dalloc(&s->mfb.hit_prim, P);
  if (!r) r = dalloc(&s->mfb.flag, P);
  if (!r) r = dalloc(&s->mfb.live, P);
  for (Lane& L : s->lanes)
    if (!r && cudaMallocHost((void**)&L.h_stage, sizeof(float4) * N) != cudaSuccess)
      r = fail(MT_ERR_NOMEM, "pinned film staging");
  size_t base = 0;  // first path of the group's share
  for (MergeGroup& G : s->groups) {
    G.server = s;
    const int n = (int)G.slots.size();
    for (Round& Rd : G.rounds) {
      if (!r && cudaMallocHost((void**)&Rd.h_tab, sizeof(int) * 3 * n) != cudaSuccess)
        r = fail(MT_ERR_NOMEM, "pinned round tables");
      if (!r && cudaMallocHost((void**)&Rd.h_pp, sizeof(PassParams) * n) != cudaSuccess)
        r = fail(MT_ERR_NOMEM, "pinned round tables");
      if (!r) r = dalloc(&Rd.d_tab, (size_t)3 * n);
      if (!r) r = dalloc(&Rd.d_pp, (size_t)n);
      if (!r) r = dalloc(&Rd.d_ctrl, (size_t)n);
      if (!r && cudaEventCreateWithFlags(&Rd.done, cudaEventDisableTiming) != cudaSuccess)
        r = fail(MT_ERR_CUDA, "event create");
    }
    if (!r && cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking) != cudaSuccess)
      r = fail(MT_ERR_CUDA, "stream create");
    if (r) break;
    G.fb = s->mfb;  // films stay whole: slot k's film is at k x N
    for (int q = 0; q < 2; ++q) {
      G.fb.q_o[q] += base;
      G.fb.q_d[q] += base;
    }
    G.fb.hit_t += base;
    G.fb.hit_prim += base;
    G.fb.thr += base;
    G.fb.ps += base;
    G.fb.flag += base;
    G.fb.s_o += base;
    G.fb.s_d += base;
    G.fb.s_c += base;
    G.fb.live += base;
    base += (size_t)n * N;
  }
  s->slot_px = N;
  return r;
}

// Merged mode: enqueues one round of merge stream G over the slots in `work`
// (scheduler thread, context lock held, server lock not held). cancel[i]: slot
// work[i]'s request was cancelled; it gets no more passes and completes
// without a film.
int issue_round(mt_server* s, MergeGroup& G, const std::vector<int>& work, const std::vector<char>& cancel) {
  const mt_server_config& c = s->cfg;
  const size_t N = s->slot_px;
  cudaStream_t st = G.stream;
  Round& Rd = G.rounds[G.next_round];
  G.next_round = (G.next_round + 1) % kRounds;
  if (Rd.used) CU(cudaEventSynchronize(Rd.done));  // its tables were read, its passes ran
  Rd.used = true;
  std::vector<int> go;
  for (size_t i = 0; i < work.size(); ++i) {
    Lane& L = s->lanes[work[i]];
    if (cancel[i]) {
      CU(cudaLaunchHostFunc(st, lane_done, &L));
      L.issued = true;
      continue;
    }
    if (L.pass == 0) {
      CU(cudaMemsetAsync(s->mfb.film + N * work[i], 0, (size_t)L.req->width * L.req->height * 16, st));
      CU(cudaMemsetAsync(s->mfb.film_c + N * work[i], 0, (size_t)L.req->width * L.req->height * 16, st));
    }
    go.push_back(work[i]);
  }
  // scene groups in slot order; per group: starts (n + 1), film offsets (n), pass parameters (n)
  struct Group {
    mt_scene* scene;
    int tab, pp, n, total;
  };
  std::vector<Group> groups;
  std::vector<char> taken(go.size(), 0);
  int ti = 0, pi = 0;
  for (size_t a = 0; a < go.size(); ++a) {
    if (taken[a]) continue;
    Group Gr{s->lanes[go[a]].req->scene, ti, pi, 0, 0};
    std::vector<int> members;
    for (size_t b = a; b < go.size(); ++b)
      if (!taken[b] && s->lanes[go[b]].req->scene == Gr.scene) {
        taken[b] = 1;
        members.push_back(go[b]);
      }
    Gr.n = (int)members.size();
    int* start = Rd.h_tab + ti;
    int* film = start + Gr.n + 1;
    for (int m = 0; m < Gr.n; ++m) {
      const Lane& L = s->lanes[members[m]];
      const Request* R = L.req;
      PassParams& pp = Rd.h_pp[pi + m];
      std::memset(&pp, 0, sizeof(pp));
      camera_constants(R->camera, R->width, R->height, pp);
      pp.frame_count = R->frame_count + (float)L.pass;
      pp.width = R->width;
      pp.height = R->height;
      pp.max_depth = c.max_depth;
      pp.mode = 1;
      pp.rr_depth = c.rr_depth;
      pp.kahan = c.film_kahan;
      pp.grid_accum = 0;
      start[m] = Gr.total;
      film[m] = (int)(N * members[m]);
      Gr.total += R->width * R->height;
    }
    start[Gr.n] = Gr.total;
    ti += 2 * Gr.n + 1;
    pi += Gr.n;
    groups.push_back(Gr);
  }
  if (!groups.empty()) {
    CU(cudaMemcpyAsync(Rd.d_tab, Rd.h_tab, sizeof(int) * ti, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(Rd.d_pp, Rd.h_pp, sizeof(PassParams) * pi, cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(Rd.d_ctrl, 0, sizeof(Ctrl) * groups.size(), st));
  }
  for (size_t g = 0; g < groups.size(); ++g) {
    // The scene group's merged pass (raygen, per bounce closest hits, shading and
    // shadow rays, ray totals) as one CUDA graph: captured every round, since
    // its path total sizes the grids and its tables move through the ring, and
    // applied to the stream's executable graph of that scene by an update (the
    // same kernels every round), instantiated again only when an update fails.
    const Group& Gr = groups[g];
    const DevScene S = Gr.scene->view();
    const DevEnv E = Gr.scene->env_view();  // full-map environment sampling
    CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int lr = launch_batch_pass(st, S, E, Rd.d_tab + Gr.tab, Rd.d_tab + Gr.tab + Gr.n + 1, Rd.d_pp + Gr.pp,
                                     Gr.n, Gr.total, c.max_depth, c.film_kahan, Rd.d_ctrl + g, G.fb,
                                     s->ctx->num_sms, s->d_totals, s->groups.size() > 1);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (lr || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(MT_ERR_CUDA, "merged pass capture: %s", cudaGetErrorString(lr ? cudaGetLastError() : e));
    }
    cudaGraphExec_t* ex = nullptr;
    for (auto& kv : G.graphs)
      if (kv.first == Gr.scene) ex = &kv.second;
    if (!ex) {
      if (G.graphs.size() >= kGraphsPerStream) {
        // the oldest scene's graph goes (a graph still running is freed when it ends)
        if (G.graphs.front().second) cudaGraphExecDestroy(G.graphs.front().second);
        G.graphs.erase(G.graphs.begin());
      }
      G.graphs.emplace_back(Gr.scene, nullptr);
      ex = &G.graphs.back().second;
    }
    if (*ex) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(*ex, graph, &info) != cudaSuccess) {
        cudaGetLastError();  // an update that does not apply is not an error: instantiate again
        cudaGraphExecDestroy(*ex);
        *ex = nullptr;
      }
    }
    if (!*ex) e = cudaGraphInstantiate(ex, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      *ex = nullptr;
      return fail(MT_ERR_CUDA, "merged pass graph: %s", cudaGetErrorString(e));
    }
    CU(cudaGraphLaunch(*ex, st));
  }
  for (int k : go) {
    Lane& L = s->lanes[k];
    if (++L.pass < L.req->spp) continue;
    CU(cudaMemcpyAsync(L.h_stage, s->mfb.film + N * k, (size_t)L.req->width * L.req->height * 16,
                       cudaMemcpyDeviceToHost, st));
    CU(cudaLaunchHostFunc(st, lane_done, &L));
    L.issued = true;
  }
  CU(cudaEventRecord(Rd.done, st));
  CU(cudaLaunchHostFunc(st, round_done, &G));
  return MT_OK;
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
      L.pass = 0;
      L.issued = false;
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
      if (!s->groups.empty()) {
        // merged: a free slot of the merge stream with the fewest running pixels
        size_t best = ~(size_t)0;
        for (const MergeGroup& G : s->groups) {
          size_t px = 0;
          Lane* slot = nullptr;
          for (int k : G.slots) {
            Lane& L = s->lanes[k];
            if (L.req)
              px += (size_t)L.req->width * L.req->height;
            else if (!slot)
              slot = &L;
          }
          if (slot && px < best) {
            best = px;
            free_lane_p = slot;
          }
        }
      } else {
        for (Lane& L : s->lanes)
          if (!L.req) {
            free_lane_p = &L;
            break;
          }
      }
      if (!free_lane_p || (s->running > 0 && s->used_bytes + R->bytes > s->cfg.budget_bytes)) break;
      s->pending.pop_front();
      if (!s->broken.empty()) {
        R->state = kFailed;
        R->error = s->broken;
        release_scene(R);
        s->done_cv.notify_all();
        continue;
      }
      R->state = kRunning;
      R->t_start = Clock::now();
      s->used_bytes += R->bytes;
      ++s->running;
      free_lane_p->req = R;
      free_lane_p->finished = false;
      free_lane_p->pass = 0;
      free_lane_p->issued = false;
      if (s->cfg.merged) continue;  // its passes join its merge stream's next round
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
        cudaStreamSynchronize(free_lane_p->side);
        R->state = kFailed;
        R->error = mt_last_error();
        s->used_bytes -= R->bytes;
        --s->running;
        release_scene(R);
        free_lane_p->req = nullptr;
        s->done_cv.notify_all();
      }
    }
    // merged mode: on each merge stream with a free round entry, the next round
    // over its running requests with passes to go
    bool issued_round = false;
    for (MergeGroup& G : s->groups) {
      if (G.inflight >= kRounds || !s->broken.empty()) continue;
      std::vector<int> work;
      std::vector<char> cancel;
      for (int k : G.slots)
        if (s->lanes[k].req && !s->lanes[k].issued) {
          work.push_back(k);
          cancel.push_back(s->lanes[k].req->cancel ? 1 : 0);
        }
      if (work.empty()) continue;
      ++G.inflight;
      issued_round = true;
      lk.unlock();
      int r;
      {
        std::lock_guard<std::recursive_mutex> ck(s->ctx->mu);
        cudaSetDevice(s->ctx->device);
        r = issue_round(s, G, work, cancel);
        if (r)
          for (MergeGroup& H : s->groups) cudaStreamSynchronize(H.stream);
      }
      lk.lock();
      if (r) {
        // every running request fails, and so does every later one
        s->broken = mt_last_error();
        for (Lane& L : s->lanes) {
          if (!L.req) continue;
          L.req->state = kFailed;
          L.req->error = s->broken;
          L.req->t_done = Clock::now();
          s->used_bytes -= L.req->bytes;
          --s->running;
          release_scene(L.req);
          L.req = nullptr;
          L.finished = false;
          L.issued = false;
          L.pass = 0;
        }
        s->done_cv.notify_all();
        break;
      }
    }
    if (issued_round) continue;
    if (s->stop && s->running == 0) break;
    s->cv.wait(lk, [&] {
      if (s->stop && s->running == 0) return true;
      for (Lane& L : s->lanes)
        if (L.req && L.finished) return true;
      if (s->broken.empty())
        for (const MergeGroup& G : s->groups)
          if (G.inflight < kRounds)
            for (int k : G.slots)
              if (s->lanes[k].req && !s->lanes[k].issued) return true;
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
  if (c.lanes < 1 || c.lanes > 256) return fail(MT_ERR_INVALID, "lanes %d (1..256)", c.lanes);
  if (c.max_width <= 0 || c.max_height <= 0 || (long long)c.max_width * c.max_height > (1ll << 26))
    return fail(MT_ERR_INVALID, "largest frame %d x %d", c.max_width, c.max_height);
  if (c.max_spp < 1 || c.max_spp > 4096) return fail(MT_ERR_INVALID, "max_spp %d", c.max_spp);
  if (c.max_depth < 1 || c.max_depth > kMaxDepth) return fail(MT_ERR_INVALID, "max_depth %d", c.max_depth);
  if (c.merged < 0 || c.merged > c.lanes) return fail(MT_ERR_INVALID, "merged %d (0..lanes)", c.merged);
  if (c.merged && (long long)c.lanes * c.max_width * c.max_height > (1ll << 30))
    return fail(MT_ERR_INVALID, "merged: lanes x largest frame above 2^30 paths");
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
    if (!r && !c.merged) r = alloc_lane(L, N, c.max_spp, c.max_depth, s->status_stride);
  }
  if (!r && c.merged) r = alloc_merged(s, N, c.merged);
  if (!r && cudaMemset(s->d_totals, 0, 32) != cudaSuccess) r = fail(MT_ERR_CUDA, "memset");
  if (r) {
    std::string keep = mt_last_error();
    for (Lane& L : s->lanes) free_lane(L);
    free_merged(s);
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
    for (MergeGroup& G : s->groups)
      if (G.stream) cudaStreamSynchronize(G.stream);
    for (Lane& L : s->lanes) {
      for (cudaStream_t q : {L.stream, L.side})
        if (q) cudaStreamSynchronize(q);
      free_lane(L);
    }
    free_merged(s);
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
  for (mt_server* s : ctx->servers) {
    for (MergeGroup& G : s->groups)
      if (G.stream) cudaStreamSynchronize(G.stream);
    for (Lane& L : s->lanes)
      for (cudaStream_t q : {L.stream, L.side})
        if (q) cudaStreamSynchronize(q);
  }
}
