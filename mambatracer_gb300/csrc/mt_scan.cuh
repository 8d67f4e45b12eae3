// Single-pass stable compaction: warp ballot/popc ranks, a block scan of the
// warp totals, and decoupled look-back over tile aggregates (Merrill &
// Garland, "Single-pass Parallel Prefix Scan with Decoupled Look-back").
// Two flags are counted at once, packed as a + (b << 31) in 64 bits.
// Every wait is bounded; when a bound runs out the error is latched and the
// kernel carries on with a partial prefix (wrong output, no hang).
#pragma once
#include <cuda_runtime.h>

#include "mt_common.h"

namespace mt {
namespace scan {

constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPfx = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr unsigned long long kLowMask = (1ull << 31) - 1;
constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Decoupled look-back over tile aggregates (single-pass stable compaction).
// Returns the exclusive prefix of `tile`. Every wait is bounded: after
// kSpinLimit polls the error is latched and the partial prefix is used.
__device__ __forceinline__ unsigned long long lookback(unsigned long long* status, int tile, unsigned long long agg, int* err) {
  if (tile == 0) {
    st_release(&status[0], kFlagPfx | agg);
    return 0;
  }
  st_release(&status[tile], kFlagAgg | agg);
  unsigned long long excl = 0;
  int t = tile - 1;
  while (t >= 0) {
    unsigned long long s = 0;
    int it = 0;
    for (; it < kSpinLimit; ++it) {
      s = ld_acquire(&status[t]);
      if (s >> 62) break;
      __nanosleep(32);
    }
    if (it == kSpinLimit) {
      atomicExch(err, kDevErrLookback);
      break;
    }
    excl += s & kValMask;
    if ((s >> 62) == 2) break;
    --t;
  }
  st_release(&status[tile], kFlagPfx | (excl + agg));
  return excl;
}

// Block-wide exclusive scan of packed 64-bit counts (THREADS threads).
template <int THREADS>
__device__ __forceinline__ unsigned long long block_scan(unsigned long long v, unsigned long long* total,
                                                         unsigned long long* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < THREADS / 32 ? sh[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < THREADS / 32) sh[lane] = w;
  }
  __syncthreads();
  unsigned long long warp_excl = warp == 0 ? 0ull : sh[warp - 1];
  *total = sh[THREADS / 32 - 1];
  __syncthreads();
  return warp_excl + x - v;
}

// Exclusive block-wide ranks of two flags a, b (THREADS threads, all of them
// calling): returns the packed exclusive prefix a + (b << 31) of this thread,
// *total the packed block total. Warp level by ballot/popc.
template <int THREADS>
__device__ __forceinline__ unsigned long long block_rank2(bool a, bool b, unsigned long long* total,
                                                          unsigned long long* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned ba = __ballot_sync(0xffffffffu, a), bb = __ballot_sync(0xffffffffu, b);
  const unsigned lt = (1u << lane) - 1u;
  unsigned long long mine = (unsigned long long)__popc(ba & lt) | ((unsigned long long)__popc(bb & lt) << 31);
  if (lane == 0) sh[warp] = (unsigned long long)__popc(ba) | ((unsigned long long)__popc(bb) << 31);
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < THREADS / 32 ? sh[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < THREADS / 32) sh[lane] = w;
  }
  __syncthreads();
  unsigned long long warp_excl = warp == 0 ? 0ull : sh[warp - 1];
  *total = sh[THREADS / 32 - 1];
  __syncthreads();
  return warp_excl + mine;
}

}  // namespace scan
}  // namespace mt
