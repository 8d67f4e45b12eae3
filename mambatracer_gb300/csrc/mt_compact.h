// Stable hit-record compaction (CompactAtomic) launcher.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace mt {

constexpr int kCompactThreads = 256;

// Device scratch of one compaction: one status word per 256-element tile and
// four ints (tile counter, entry value of *count, error, spare).
struct CompactScratch {
  unsigned long long* status;
  int* words;
};

// Returns the error of the first call that failed (cudaSuccess: all enqueued).
cudaError_t launch_compact_isects(cudaStream_t st, const void* isects_in, const int32_t* pixels_in, int n,
                                  void* isects_out, int32_t* pixels_out, int32_t* count_io, CompactScratch s);

}  // namespace mt
