// Host-visible declarations of the device launchers.
#pragma once
#include <cuda_runtime.h>

#include "mt_common.h"

namespace mt {

// Per-job frame buffers (structure of arrays).
struct FrameBufs {
  float4* q_o[2];   // ray queue: origin.xyz, bits(pixel)  (ping-pong by bounce parity)
  float4* q_d[2];   // ray queue: direction.xyz, 0
  float* hit_t;     // closest-hit distance per queue slot
  int* hit_prim;    // closest-hit face id per queue slot (-1 = miss)
  float4* thr;      // path throughput per pixel (4 lanes as the reference)
  float4* ps;       // path: hitpoint.xyz, lastPdfW
  int* flag;        // path: lastSpecular
  float4* s_o;      // shadow queue: origin.xyz, bits(pixel or -1)
  float4* s_d;      // shadow queue: direction.xyz, tMax
  float4* s_c;      // shadow queue: contribution.xyz
  float4* film;     // accumulated radiance per pixel
  float4* film_c;   // Kahan compensation per pixel
  int* live;        // queue slots of the paths that go on after the hit phase (two-launch shading)
};

// Launch shapes of the hot kernels, process-wide (one GPU per process):
// closest_minb / shadow_minb: the traversal build, by the resident blocks per
// SM its registers are bounded for (8, 12, 16); closest_grid / shadow_grid:
// blocks per SM of a traversal launch that shares the GPU with other frames (0:
// half of what fits); shade_minb: the benchmark-semantics shading build (3, 4,
// 5); refill_steps: traversal steps between refills of finished lanes (4..1024);
// shadow_stream: a frame's shadow rays of bounce b run on a second stream beside
// its extension rays of bounce b + 1 (1) or after them on one stream (0).
// Every choice gives the same results; only the speed differs.
struct Tuning {
  int closest_minb, shadow_minb, closest_grid, shadow_grid, shade_minb, refill_steps, shadow_stream;
};
Tuning get_tuning();
bool set_tuning(const Tuning& t);  // false when a field is out of range
unsigned tuning_version();         // bumped by every set_tuning (jobs recapture their graphs)

// events: optional array of 2 + 3 * max_depth events recorded around each launch.
// totals: optional running ray counts [primary, extension, shadow, error] of the job.
// shared: other frames or requests run beside this pass on the GPU (frames in
// flight, served lanes): each persistent traversal launch then takes half the
// blocks an SM can hold, leaving room for their kernels.
// side, fork, join: a second stream and two events of the caller's; with the
// tuning's shadow_stream on, the shadow rays run there.
// A merged batch pass (benchmark semantics, full-map environment sampling):
// frames 0 .. nframes-1 share the queues; path g belongs to the frame k with
// d_start[k] <= g < d_start[k+1] (pixel g - d_start[k]), its film slots start at
// d_film[k], its parameters are d_pp[k]. total = d_start[nframes].
int launch_batch_pass(cudaStream_t st, const DevScene& S, const DevEnv& E, const int* d_start, const int* d_film,
                      const PassParams* d_pp, int nframes, int total, int max_depth, int kahan, Ctrl* ctrl,
                      FrameBufs fb, int num_sms, unsigned long long* totals, bool shared = false);
int launch_pass(cudaStream_t st, const DevScene& S, const DevEnv& E, const PassParams* d_pp, int mode,
                int max_depth, int kahan, int width, int height, Ctrl* ctrl, FrameBufs fb,
                unsigned long long* status, size_t status_stride, int num_sms, cudaEvent_t* events,
                unsigned long long* totals, bool shared = false, cudaStream_t side = nullptr,
                cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr, int shade_split = -1);
// The process's benchmark-semantics shading setting (MT_SHADE_SPLIT): -1 render
// jobs choose per frame (shade_split_for) and other passes run two launches; 0
// always one launch; 1 always two.
int shade_split_setting();
// Whether shading in two launches pays for a frame whose bounce-1 queue of
// `queued` paths left `went_on` going on (two launches pay when many paths end at
// their first hit: their lanes would idle through the light and BSDF samples);
// current: the choice so far, kept near the crossover.
int shade_split_for(int queued, int went_on, int current);

// Closest or any hit of reference-layout rays with the traversal work per ray
// (interior-node visits, triangle tests), one ray per thread.
int launch_count(cudaStream_t st, const DevScene& S, const float4* rays, int n, int any, float* t_out, int* prim_out,
                 int* counts, int* err);
int launch_query(cudaStream_t st, const DevScene& S, const float4* rays, int n, int any, float* t_out,
                 int* prim_out, int* work, int* err, int num_sms);

// Environment: luminance (FP32, RGBSpace.cl:28-32) and the inclusive SAT built
// in FP64, with an FP32 copy for sampling.
int launch_env_build(cudaStream_t st, const float4* rgb, int w, int h, float* lum, double* sat64, float* sat32);

// Light-grid per-cell SAT (row passes of rx, column passes of ry), FP32 in the
// reference's Kogge-Stone order or FP64.
int launch_grid_sat(cudaStream_t st, const float* func, float* sat32, double* sat64, int nu, int nv, int rx, int ry,
                    int fp64);
// Initial light-grid func: each cell's tiles get the map's luminance summed over
// the tile (from sat64 when not NULL, else sat32).
int launch_grid_init(cudaStream_t st, const double* sat64, const float* sat32, int w, int h, int nu, int nv, int rx,
                     int ry, float* func);
// CDF tables of the grid-guided environment sampling (dv::RegionTab): for the
// rx x ry tiles of the map (from its FP32 SAT) and for the grid's cells (from
// the per-cell SATs). *_floats return the cond table's size and the marg table's
// through *marg_floats.
size_t tile_table_floats(int w, int h, int rx, int ry, size_t* marg_floats);
size_t map_table_floats(int w, int h, size_t* marg_floats);
int launch_map_tables(cudaStream_t st, const float* sat, int w, int h, float* marg, float* cond);
size_t cell_table_floats(int nu, int nv, int rx, int ry, size_t* marg_floats);
int launch_tile_tables(cudaStream_t st, const float* sat, int w, int h, int rx, int ry, float* marg, float* cond);
int launch_cell_tables(cudaStream_t st, const float* grid_sat, int nu, int nv, int rx, int ry, float* marg,
                       float* cond);

}  // namespace mt
