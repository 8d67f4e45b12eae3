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

// CDF tables (dv::RegionTab) of n regions of size sx x sy, one thread per value:
// region k's values are marg for rows minY-1 .. minY+sy, then cond for rows
// minY-1 .. minY+sy-1 and columns minX-1 .. minX+sx, computed by the functions
// the sampler uses, so a table value equals the value it replaces.
template <class RegionOf>
__global__ void k_region_tables(int n, int sx, int sy, RegionOf region_of, float* marg, float* cond) {
  const size_t per = (size_t)(sy + 2) + (size_t)(sy + 1) * (sx + 2);
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * (size_t)n) return;
  const int k = (int)(i / per);
  const size_t e = i % per;
  const float* sat;
  const dv::Region r = region_of(k, &sat);
  const float last = dv::sat_range(r, r.minX, r.minY, dv::last_x(r), dv::last_y(r), sat);
  if (e < (size_t)(sy + 2)) {
    marg[(size_t)k * (sy + 2) + e] = dv::marg_value(r, r.minY - 1 + (int)e, sat, last);
  } else {
    const size_t e2 = e - (sy + 2);
    const int row = (int)(e2 / (sx + 2)), col = (int)(e2 % (sx + 2));
    const int y = r.minY - 1 + row, x = r.minX - 1 + col;
    const float fi = dv::sat_range(r, r.minX, y, dv::last_x(r), y, sat);
    cond[(size_t)k * (sy + 1) * (sx + 2) + e2] = dv::cond_value(r, x, y, sat, fi);
  }
}
// the rx x ry tiles of the w x h map (tile ty * rx + tx), on the map's FP32 SAT
struct TileRegions {
  DevEnv E;
  const float* sat;
  __device__ dv::Region operator()(int k, const float** s) const {
    *s = sat;
    return dv::env_tile_region(E, k % E.rx, k / E.rx);
  }
};
// the cells of the grid, each its own rx x ry SAT at its first tile
struct CellRegions {
  DevEnv E;
  const float* sat;
  __device__ dv::Region operator()(int k, const float** s) const {
    *s = sat + dv::grid_cell_base(E, k);
    return dv::Region{E.nu, E.nv, 0, 0, E.rx, E.ry};
  }
};

}  // namespace

size_t map_table_floats(int w, int h, size_t* marg_floats) {
  *marg_floats = (size_t)h + 2;
  return (size_t)(h + 1) * (w + 2);
}

int launch_map_tables(cudaStream_t st, const float* sat, int w, int h, float* marg, float* cond) {
  DevEnv E{};
  E.w = w;
  E.h = h;
  E.rx = 1;
  E.ry = 1;
  const size_t total = (size_t)(h + 2) + (size_t)(h + 1) * (w + 2);
  k_region_tables<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(1, w, h, TileRegions{E, sat}, marg, cond);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t tile_table_floats(int w, int h, int rx, int ry, size_t* marg_floats) {
  const int tw = w / rx, th = h / ry;
  *marg_floats = (size_t)rx * ry * (th + 2);
  return (size_t)rx * ry * (th + 1) * (tw + 2);
}
size_t cell_table_floats(int nu, int nv, int rx, int ry, size_t* marg_floats) {
  const size_t cells = (size_t)(nu / rx) * (nv / ry);
  *marg_floats = cells * (ry + 2);
  return cells * (ry + 1) * (rx + 2);
}

int launch_tile_tables(cudaStream_t st, const float* sat, int w, int h, int rx, int ry, float* marg, float* cond) {
  if (w % rx || h % ry) return -1;
  DevEnv E{};
  E.w = w;
  E.h = h;
  E.rx = rx;
  E.ry = ry;
  const int tw = w / rx, th = h / ry, n = rx * ry;
  const size_t total = (size_t)n * ((th + 2) + (size_t)(th + 1) * (tw + 2));
  k_region_tables<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, tw, th, TileRegions{E, sat}, marg, cond);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_cell_tables(cudaStream_t st, const float* grid_sat, int nu, int nv, int rx, int ry, float* marg,
                       float* cond) {
  if (nu % rx || nv % ry) return -1;
  DevEnv E{};
  E.nu = nu;
  E.nv = nv;
  E.rx = rx;
  E.ry = ry;
  const int n = (nu / rx) * (nv / ry);
  const size_t total = (size_t)n * ((ry + 2) + (size_t)(ry + 1) * (rx + 2));
  k_region_tables<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, rx, ry, CellRegions{E, grid_sat}, marg, cond);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

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
