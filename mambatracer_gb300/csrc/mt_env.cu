// Environment-map luminance and SAT, light-grid per-cell SATs.
//
// The reference builds the full-map SAT in FP32 on the CPU through an external
// class (src/cl/algorithms/CEnvironment.java:46-60) and samples straight off it
// (src/cl/kernel/SAT.cl:158-334); the light grid's per-cell SATs are FP32
// Kogge-Stone row and column passes (src/cl/kernel/LightGrid.cl:347-400). Here
// the full-map SAT (whose last column is the marginal CDF's numerator) is built
// on the GPU in FP64: one CTA per row scans the row, then one thread per column
// adds the rows up, both coalesced. The FP32 copy is rounded once from FP64.
#include <cuda_runtime.h>

#include "mt_device.cuh"
#include "mt_kernels.h"

namespace mt {

namespace {

constexpr int kRowThreads = 256;

__global__ void k_env_lum(const float4* __restrict__ rgb, int n, float* __restrict__ lum) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 c = __ldg(rgb + i);
  lum[i] = dv::luminance(c.x, c.y, c.z);
}

// One CTA per row: inclusive FP64 prefix of the row, chunk by chunk.
__global__ void __launch_bounds__(kRowThreads) k_sat_rows(const float* __restrict__ lum, int w, double* __restrict__ sat) {
  __shared__ double warp_tot[kRowThreads / 32];
  __shared__ double carry;
  const int y = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (int x0 = 0; x0 < w; x0 += kRowThreads) {
    int x = x0 + threadIdx.x;
    double v = x < w ? (double)lum[(size_t)y * w + x] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      double u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    double before = carry;
    for (int k = 0; k < warp; ++k) before += warp_tot[k];
    if (x < w) sat[(size_t)y * w + x] = before + v;
    __syncthreads();
    if (threadIdx.x == kRowThreads - 1) carry = before + v;
    __syncthreads();
  }
}

// One thread per column: add the row prefixes down the column.
__global__ void k_sat_cols(double* __restrict__ sat, int w, int h, float* __restrict__ sat32) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= w) return;
  double acc = 0.0;
  for (int y = 0; y < h; ++y) {
    size_t i = (size_t)y * w + x;
    acc += sat[i];
    sat[i] = acc;
    sat32[i] = (float)acc;
  }
}

// Kogge-Stone over groups of G consecutive lanes, reference addition order
// (aux[i] = aux[i - off] + aux[i] with every read before any write).
template <int G, typename T>
__device__ __forceinline__ T kogge(T x, int l) {
#pragma unroll
  for (int off = 1; off < G; off <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, off, G);
    if (l >= off) x = y + x;
  }
  return x;
}

// prefixSumRowSubgrid: groups of rx consecutive elements (rx = 16: two groups per warp).
template <typename T, int RX>
__global__ void k_grid_rows(const float* __restrict__ func, T* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  T v = i < n ? (T)func[i] : (T)0;
  v = kogge<RX, T>(v, threadIdx.x & (RX - 1));
  if (i < n) out[i] = v;
}
// prefixSumColSubgrid: group g covers column (ry*g)/nv, rows (ry*g)%nv .. +ry-1.
template <typename T, int RY>
__global__ void k_grid_cols(T* __restrict__ sat, int nu, int nv, size_t groups) {
  size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / RY;
  int l = threadIdx.x & (RY - 1);
  bool ok = g < groups;
  size_t i = (size_t)RY * (ok ? g : 0);
  int xi = (int)(i / nv), yi = (int)(i % nv) + l;
  size_t idx = (size_t)xi + (size_t)yi * nu;
  T v = ok ? sat[idx] : (T)0;
  v = kogge<RY, T>(v, l);
  if (ok) sat[idx] = v;
}
__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

template <typename T>
int grid_sat_t(cudaStream_t st, const float* func, T* out, int nu, int nv, int rx, int ry) {
  size_t n = (size_t)nu * nv;
  int blocks = (int)((n + 255) / 256);
  if (rx == 16) k_grid_rows<T, 16><<<blocks, 256, 0, st>>>(func, out, n);
  else if (rx == 32) k_grid_rows<T, 32><<<blocks, 256, 0, st>>>(func, out, n);
  else if (rx == 8) k_grid_rows<T, 8><<<blocks, 256, 0, st>>>(func, out, n);
  else return -1;
  size_t groups = n / ry;
  int cb = (int)((groups * ry + 255) / 256);
  if (ry == 32) k_grid_cols<T, 32><<<cb, 256, 0, st>>>(out, nu, nv, groups);
  else if (ry == 16) k_grid_cols<T, 16><<<cb, 256, 0, st>>>(out, nu, nv, groups);
  else if (ry == 8) k_grid_cols<T, 8><<<cb, 256, 0, st>>>(out, nu, nv, groups);
  else return -1;
  return 0;
}

// Initial grid func: every cell's tile (tx, ty) gets the environment luminance
// summed over the tile's region of the map (the noise-free version of the
// reference's per-tile luminance histogram, CAdaptiveEnvironment.java:77),
// from the FP64 SAT when there is one, else the FP32 SAT.
__global__ void k_grid_init_func(const double* __restrict__ sat64, const float* __restrict__ sat32, int w, int h,
                                 int nu, int nv, int rx, int ry, float* __restrict__ func) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)nu * nv) return;
  const int tx = (int)(i % nu) % rx, ty = (int)(i / nu) % ry;
  const int x0 = (int)((float)w * ((float)tx / (float)rx)), y0 = (int)((float)h * ((float)ty / (float)ry));
  const int x1 = (int)((float)w * ((float)(tx + 1) / (float)rx)) - 1;
  const int y1 = (int)((float)h * ((float)(ty + 1) / (float)ry)) - 1;
  auto at64 = [&](int x, int y) { return (x < 0 || y < 0) ? 0.0 : sat64[(size_t)y * w + x]; };
  auto at32 = [&](int x, int y) { return (x < 0 || y < 0) ? 0.f : sat32[(size_t)y * w + x]; };
  float v;
  if (sat64)
    v = (float)(at64(x1, y1) - at64(x0 - 1, y1) - at64(x1, y0 - 1) + at64(x0 - 1, y0 - 1));
  else
    v = at32(x0 - 1, y0 - 1) + at32(x1, y1) - at32(x1, y0 - 1) - at32(x0 - 1, y1);  // SAT.cl:149-156 order
  func[i] = v;
}

}  // namespace

int launch_grid_init(cudaStream_t st, const double* sat64, const float* sat32, int w, int h, int nu, int nv, int rx,
                     int ry, float* func) {
  size_t n = (size_t)nu * nv;
  k_grid_init_func<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sat64, sat32, w, h, nu, nv, rx, ry, func);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_env_build(cudaStream_t st, const float4* rgb, int w, int h, float* lum, double* sat64, float* sat32) {
  int n = w * h;
  k_env_lum<<<(n + 255) / 256, 256, 0, st>>>(rgb, n, lum);
  k_sat_rows<<<h, kRowThreads, 0, st>>>(lum, w, sat64);
  k_sat_cols<<<(w + 127) / 128, 128, 0, st>>>(sat64, w, h, sat32);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_grid_sat(cudaStream_t st, const float* func, float* sat32, double* sat64, int nu, int nv, int rx, int ry,
                    int fp64) {
  if ((size_t)nu * nv % rx || (size_t)nu * nv % ry || nu % rx || nv % ry) return -1;
  int r;
  if (fp64) {
    r = grid_sat_t<double>(st, func, sat64, nu, nv, rx, ry);
    size_t n = (size_t)nu * nv;
    if (r == 0) k_d2f<<<(int)((n + 255) / 256), 256, 0, st>>>(sat64, sat32, n);
  } else {
    r = grid_sat_t<float>(st, func, sat32, nu, nv, rx, ry);
  }
  if (r != 0) return r;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace mt
