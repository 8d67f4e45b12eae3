// Stable compaction of hit records: CompactAtomic (src/cl/kernel/Compact.cl:21-40)
// as a single-pass prefix-sum compaction.
//
// The reference keeps every Intersection whose hit flag is set and its pixel
// id, at slot atomic_inc(count): on a GPU the slot order is whatever order the
// atomics land in; a serial run gives input order. This kernel gives input
// order always (warp ballot/popc ranks, block scan, decoupled look-back), so
// its output equals a serial CompactAtomic bit for bit. Slots start at the
// value *count holds on entry, as atomic_inc's would, and *count ends at
// entry value + kept.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mambatracer.h"
#include "mt_compact.h"
#include "mt_scan.cuh"

namespace mt {

using namespace scan;

// Intersection (src/cl/kernel/Util.cl:141-151): 96 B = 6 float4, hit at byte 80.
__global__ void __launch_bounds__(kCompactThreads)
    k_compact_isects(const float4* __restrict__ in, const int* __restrict__ pix_in, int n, float4* __restrict__ out,
                     int* __restrict__ pix_out, int* __restrict__ count, unsigned long long* __restrict__ status,
                     int* __restrict__ tile_counter, const int* __restrict__ base, int* __restrict__ err) {
  __shared__ unsigned long long sh[kCompactThreads / 32 + 1];
  __shared__ int s_tile;
  __shared__ unsigned long long s_excl;
  const int ntiles = (n + kCompactThreads - 1) / kCompactThreads;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  __syncthreads();
  const int tile = s_tile;
  if (tile >= ntiles) return;
  const int i = tile * kCompactThreads + threadIdx.x;
  bool keep = false;
  if (i < n) keep = __ldg(reinterpret_cast<const int*>(in + 6 * (size_t)i) + 20) != 0;
  unsigned long long tot;
  const unsigned long long excl = block_rank2<kCompactThreads>(keep, false, &tot, sh);
  if (threadIdx.x == 0) s_excl = lookback(status, tile, tot, err);
  __syncthreads();
  const int b0 = *base;
  if (keep) {
    const size_t slot = (size_t)b0 + (size_t)(s_excl + excl);
    const float4* src = in + 6 * (size_t)i;
    float4* dst = out + 6 * slot;
#pragma unroll
    for (int k = 0; k < 6; ++k) dst[k] = __ldg(src + k);
    pix_out[slot] = __ldg(pix_in + i);
  }
  if (tile == ntiles - 1 && threadIdx.x == 0) *count = b0 + (int)(s_excl + tot);
}

cudaError_t launch_compact_isects(cudaStream_t st, const void* isects_in, const int32_t* pixels_in, int n,
                                  void* isects_out, int32_t* pixels_out, int32_t* count_io, CompactScratch s) {
  const int ntiles = (n + kCompactThreads - 1) / kCompactThreads;
  cudaError_t e = cudaMemsetAsync(s.status, 0, sizeof(unsigned long long) * (size_t)(ntiles > 0 ? ntiles : 1), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(s.words, 0, 4 * sizeof(int), st);
  if (e != cudaSuccess) return e;
  // words: [0] tile counter, [1] entry value of *count, [2] device error
  e = cudaMemcpyAsync(s.words + 1, count_io, sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (ntiles > 0) {
    k_compact_isects<<<ntiles, kCompactThreads, 0, st>>>(
        static_cast<const float4*>(isects_in), pixels_in, n, static_cast<float4*>(isects_out), pixels_out, count_io,
        s.status, s.words, s.words + 1, s.words + 2);
    e = cudaGetLastError();
  }
  return e;
}

// ------------------------------------------------------- no-allocation variant
// For callers that cannot call cudaMalloc: a host whose device memory all
// belongs to another allocator (a JVM-side pool, or a framework's caching
// allocator that would first have to give memory back), or a plugin that may
// not allocate on its caller's behalf. The compaction's scratch (one status
// word per 256-record tile plus four counters) is this file-scope array, sized
// for kNoAllocMaxRecords records; every GPU that loads the library holds it
// (128 KiB) until the process exits.
constexpr int kNoAllocMaxRecords = 1 << 22;
constexpr int kNoAllocTiles = kNoAllocMaxRecords / kCompactThreads;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocTiles + 2];

}  // namespace mt

#include <mutex>
#include <string>

namespace mt {
__attribute__((visibility("hidden"))) void set_last_error(const char* msg);  // read by mt_last_error()
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
// The scratch array's device address as looked up in one CUDA context: an
// address from cudaGetSymbolAddress holds only in the context current at the
// lookup. Contexts are told apart by cuCtxGetId, which never reuses an id in a
// process, so a new primary context (after cudaDeviceReset) or another context
// a host made current on the device gets a fresh lookup.
struct ScratchAddr {
  unsigned long long ctx_id = 0;  // 0: no lookup yet
  unsigned long long* ptr = nullptr;
};
ScratchAddr g_noalloc_addr[kMaxDevices];
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

int noalloc_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
  std::string m = msg;
  if (e != cudaSuccess) {
    m += ": ";
    m += cudaGetErrorString(e);
  }
  mt::set_last_error(m.c_str());
  return code;
}

// Id of the context current on this thread. The driver function is fetched
// through the runtime, so the library needs no link to libcuda.
int current_ctx_id(unsigned long long* id) {
  static CtxGetIdFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetIdFn>(p);
  });
  if (!fn) return noalloc_fail(MT_ERR_CUDA, "cuCtxGetId is not available from the driver");
  if (fn(nullptr, id) != CUDA_SUCCESS || *id == 0) return noalloc_fail(MT_ERR_CUDA, "no current CUDA context");
  return MT_OK;
}
}  // namespace

extern "C" int mt_compact_isects_noalloc(void* stream, const void* isects_in, const int32_t* pixels_in, int n,
                                         void* isects_out, int32_t* pixels_out, int32_t* count_io) {
  if (n < 0 || (n > 0 && (!isects_in || !pixels_in || !isects_out || !pixels_out)) || !count_io)
    return noalloc_fail(MT_ERR_INVALID, "bad argument");
  if (n > mt::kNoAllocMaxRecords)
    return noalloc_fail(MT_ERR_INVALID, "n exceeds the 4194304 records the static scratch holds");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(MT_ERR_CUDA, "cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(MT_ERR_INVALID, "device index out of range");
  // Make sure a context is current (the device's primary context unless the
  // host made another one current), then identify it.
  e = cudaStreamQuery(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess && e != cudaErrorNotReady) return noalloc_fail(MT_ERR_CUDA, "stream", e);
  unsigned long long ctx_id = 0;
  if (int r = current_ctx_id(&ctx_id)) return r;
  unsigned long long* scratch;
  {
    // Set-up, once per device and context: the scratch array's device address
    // in the current context.
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    ScratchAddr& a = g_noalloc_addr[dev];
    if (a.ctx_id != ctx_id) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, mt::g_noalloc_scratch);
      if (e != cudaSuccess || !p) return noalloc_fail(MT_ERR_CUDA, "cudaGetSymbolAddress", e);
      a.ptr = static_cast<unsigned long long*>(p);
      a.ctx_id = ctx_id;
    }
    scratch = a.ptr;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  mt::CompactScratch s{scratch, reinterpret_cast<int*>(scratch + mt::kNoAllocTiles)};
  e = mt::launch_compact_isects(st, isects_in, pixels_in, n, isects_out, pixels_out, count_io, s);
  if (e != cudaSuccess) return noalloc_fail(MT_ERR_CUDA, "compaction launch", e);
  int err = 0;
  e = cudaMemcpyAsync(&err, s.words + 2, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return noalloc_fail(MT_ERR_CUDA, "compaction", e);
  if (err) return noalloc_fail(MT_ERR_DEVICE, "compaction: a bounded wait ran out");
  return MT_OK;
}
