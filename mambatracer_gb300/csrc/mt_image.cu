// The displayed image: CImage.processImage (src/cl/image/CImage.java:124-136,
// src/cl/kernel/Image.cl:29-118, src/cl/kernel/RGBSpace.cl:9-106).
//
// averageAccum divides the film by the frame count and takes log(0.01 + Lw)
// of every pixel with luminance Lw > 0; the log-average of those is the key of
// the Reinhard operator that updateFrameImage applies to the exposure-scaled
// luminance through xyY, followed by gamma and 8-bit ARGB packing. Pixels with
// Lw <= 0 keep their previous ARGB value (opaque black after initialisation,
// InitIntDataRGB). The log total is summed in FP64 in a fixed order (block
// partials, then one block over the partials) and recomputed on every call;
// the reference's float prefix scan for it reads aux[-1] in lane 0 and
// truncates through an int, and runs on its first two frames only.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "mt_internal.h"

namespace {

constexpr int kToneThreads = 256;
constexpr int kOpaqueBlack = (int)0xFF000000u;  // getIntARGB((0, 0, 0, 1))

__device__ __forceinline__ float lum3(float x, float y, float z) { return (0.2989f * x + 0.5866f * y) + 0.1145f * z; }

__global__ void k_argb_fill(int* argb, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) argb[i] = kOpaqueBlack;
}

// averageAccum (Image.cl:29-67) and per-block sums of its log luminance.
__global__ void __launch_bounds__(kToneThreads)
    k_tone_average(const float4* __restrict__ film, float frame_count, int n, float4* __restrict__ fb,
                   double* __restrict__ part_sum, int* __restrict__ part_cnt) {
  __shared__ double ssum[kToneThreads / 32];
  __shared__ int scnt[kToneThreads / 32];
  const int i = blockIdx.x * kToneThreads + threadIdx.x;
  double v = 0.0;
  int c = 0;
  if (i < n) {
    const float4 a = film[i];
    const float4 f = make_float4(a.x / frame_count, a.y / frame_count, a.z / frame_count, 1.f);
    fb[i] = f;
    const float Lw = lum3(f.x, f.y, f.z);
    if (Lw > 0.f) {
      v = (double)logf(0.01f + Lw);
      c = 1;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_down_sync(0xffffffffu, v, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    ssum[warp] = v;
    scnt[warp] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    int k = 0;
    for (int w = 0; w < kToneThreads / 32; ++w) {
      s += ssum[w];
      k += scnt[w];
    }
    part_sum[blockIdx.x] = s;
    part_cnt[blockIdx.x] = k;
  }
}

// One block: the partials summed in a fixed order; out = {total (FP32), count}.
__global__ void __launch_bounds__(1024) k_tone_total(const double* __restrict__ part_sum,
                                                     const int* __restrict__ part_cnt, int nparts,
                                                     float* __restrict__ out) {
  __shared__ double ssum[1024];
  __shared__ int scnt[1024];
  double v = 0.0;
  int c = 0;
  for (int k = threadIdx.x; k < nparts; k += 1024) {
    v += part_sum[k];
    c += part_cnt[k];
  }
  ssum[threadIdx.x] = v;
  scnt[threadIdx.x] = c;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      ssum[threadIdx.x] += ssum[threadIdx.x + s];
      scnt[threadIdx.x] += scnt[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = (float)ssum[0];
    out[1] = __int_as_float(scnt[0]);
  }
}

__device__ __forceinline__ int argb_of(float r, float g, float b, float a) {  // getIntARGB, Util.cl:469-480
  auto q = [](float v) { return (int)(fminf(fmaxf(v, 0.f), 1.f) * 255.0f); };
  return (q(a) << 24) | (q(r) << 16) | (q(g) << 8) | q(b);
}

// updateFrameImage (Image.cl:70-118) with RGBSpace.cl's conversions.
__global__ void k_tone_map(float4* __restrict__ fb, int n, const float* __restrict__ totals, float exposure,
                           float gamma, int* __restrict__ argb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float logavg = totals[0] / (float)__float_as_int(totals[1]);
  logavg = expf(logavg);
  float4 c = fb[i];
  const float L = lum3(c.x, c.y, c.z);
  if (!(L > 0.f)) return;
  const float scaled = exposure * L / logavg;
  float Y = scaled / (1.f + scaled);                                // toneSimpleReinhard
  if (isinf(Y) || isnan(Y) || Y < 0.000001f) Y = 0.f;              // check, Util.cl:381-387
  const float X_ = 0.5893f * c.x + 0.1789f * c.y + 0.1831f * c.z;  // convertRGBtoXYZ
  const float Y_ = 0.2904f * c.x + 0.6051f * c.y + 0.1045f * c.z;
  const float Z_ = 0.0000f * c.x + 0.0684f * c.y + 1.0202f * c.z;
  float x = 0.f, y = 0.f;  // xyz(): unset (zero) when X + Y + Z < 1e-6
  const float XYZ = X_ + Y_ + Z_;
  if (!(XYZ < 1e-6f)) {
    const float s = 1.f / XYZ;
    x = X_ * s;
    y = Y_ * s;
  }
  const float X = y < 1e-6f ? 0.f : Y * (x / y);  // xyYtoXYZ
  const float Z = y < 1e-6f ? 0.f : (Y * (1 - x - y)) / y;
  c.x = 1.967f * X - 0.548f * Y - 0.297f * Z;  // convertXYZtoRGB
  c.y = -0.955f * X + 1.938f * Y - 0.027f * Z;
  c.z = 0.064f * X - 0.130f * Y + 0.982f * Z;
  c.w = 1.f;
  const float ig = 1.f / gamma;
  c.x = powf(c.x, ig);
  c.y = powf(c.y, ig);
  c.z = powf(c.z, ig);
  fb[i] = c;
  argb[i] = argb_of(c.x, c.y, c.z, c.w);
}

int ensure_image(mt_job* j) {
  if (j->d_argb) return MT_OK;
  const size_t N = (size_t)j->cfg.width * j->cfg.height;
  const int nparts = (int)((N + kToneThreads - 1) / kToneThreads);
  int r = dalloc(&j->d_argb, N);
  if (!r) r = dalloc(&j->d_fb, N);
  if (!r) r = dalloc(&j->d_tone_part, (size_t)nparts);
  if (!r) r = dalloc(&j->d_tone_cnt, (size_t)nparts);
  if (!r) r = dalloc(&j->d_tone_tot, 2);
  if (r) return r;
  k_argb_fill<<<(unsigned)((N + 255) / 256), 256, 0, j->ctx->stream>>>(j->d_argb, N);
  CU(cudaGetLastError());
  return MT_OK;
}

}  // namespace

void image_reset(mt_job* j) {
  if (!j->d_argb) return;
  const size_t N = (size_t)j->cfg.width * j->cfg.height;
  k_argb_fill<<<(unsigned)((N + 255) / 256), 256, 0, j->ctx->stream>>>(j->d_argb, N);
}

extern "C" int mt_image_argb(mt_job* j, int32_t* argb, float exposure, float gamma, float* log_average) {
  if (!j || !argb) return fail(MT_ERR_INVALID, "NULL argument");
  if (!(gamma > 0.f)) return fail(MT_ERR_INVALID, "gamma %g", (double)gamma);
  mt_context* ctx = j->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  int r = ensure_image(j);
  if (r) return r;
  join_jobs(ctx);
  const int n = j->cfg.width * j->cfg.height;
  const int nparts = (n + kToneThreads - 1) / kToneThreads;
  if (j->frames > 0) {
    k_tone_average<<<nparts, kToneThreads, 0, ctx->stream>>>(j->film(), (float)j->frames, n, j->d_fb,
                                                              j->d_tone_part, j->d_tone_cnt);
    k_tone_total<<<1, 1024, 0, ctx->stream>>>(j->d_tone_part, j->d_tone_cnt, nparts, j->d_tone_tot);
    k_tone_map<<<(n + 255) / 256, 256, 0, ctx->stream>>>(j->d_fb, n, j->d_tone_tot, exposure, gamma, j->d_argb);
    CU(cudaGetLastError());
  }
  float tot[2] = {0.f, 0.f};
  CU(cudaMemcpyAsync(argb, j->d_argb, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (log_average && j->frames > 0) CU(cudaMemcpyAsync(tot, j->d_tone_tot, 8, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (log_average) {
    int cnt;
    std::memcpy(&cnt, &tot[1], 4);
    *log_average = (j->frames > 0 && cnt > 0) ? std::exp(tot[0] / (float)cnt) : 0.f;
  }
  return MT_OK;
}
