// The preview device's frame in one launch: CDeviceRT.loop
// (src/cl/device/CDeviceRT.java:176-197) runs InitCameraRayData,
// IntersectPrimitives, SetupBSDFRaytrace, backgroundShade, fastShade and
// updateGroupbufferShadeImage (src/cl/kernel/Raytrace.cl) one launch each; here
// a persistent traversal kernel generates each pixel's unjittered camera ray,
// finds its closest hit on the scene's traversal layout and writes the quick
// colour (emission, or diffuse colour x the cosine to the camera) or the gamma-2.2
// environment texel, and the material group, directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "mt_device.cuh"
#include "mt_internal.h"
#include "mt_traverse.cuh"

namespace mt {
namespace {

using namespace dv;

__device__ __forceinline__ int pack_argb(float r, float g, float b, float a) {  // getIntARGB, Util.cl:469-480
  auto q = [](float v) { return (int)(fminf(fmaxf(v, 0.f), 1.f) * 255.0f); };
  return (q(a) << 24) | (q(r) << 16) | (q(g) << 8) | q(b);
}

struct CameraRays {  // InitCameraRayData (Raytrace.cl:1-31)
  PassParams pp;
  __device__ __forceinline__ tr::RayT operator()(int id) const {
    const int W = pp.width;
    const float px = (float)(id % W), py = (float)(id / W);
    V d = normalize4(mk(pp.cam_a * (2.f * px / pp.dim_w - 1.f), -2.f * py / pp.dim_h + 1.f, -pp.cam_d, 0.f));
    const float* m = pp.cam_m;
    V z = zero4();
    V m0 = mk(m[0], m[1], m[2], m[3]), m1 = mk(m[4], m[5], m[6], m[7]), m2 = mk(m[8], m[9], m[10], m[11]),
      m3 = mk(m[12], m[13], m[14], m[15]);
    V o = mk(dot3(m0, z) + m0.w, dot3(m1, z) + m1.w, dot3(m2, z) + m2.w, dot3(m3, z) + m3.w);
    if (!(o.w == 1.f)) o = mk(o.x / o.w, o.y / o.w, o.z / o.w, 0.f);
    V dw = mk(dot4(m0, d), dot4(m1, d), dot4(m2, d), 0.f);
    return tr::make_ray(make_float4(o.x, o.y, o.z, 0.f), make_float4(dw.x, dw.y, dw.z, 0.f), 0.001f, CUDART_INF_F);
  }
};

struct PreviewOut {  // setupBsdf's cosine, fastShade, backgroundShade, group
  DevScene S;
  DevEnv E;
  int* argb;
  int* group;
  __device__ __forceinline__ void operator()(int id, const tr::RayT& r, int hit) const {
    const V d = mk(r.dx, r.dy, r.dz, 0.f);
    if (hit >= 0) {
      Hit H;
      hit_record(S, mk(r.ox, r.oy, r.oz, 0.f), d, r.tmax, hit, H);
      const Frame f = get_frame(H.n);
      const float coeff = local_coord(f, neg(d)).z;
      const Material& P = S.materials[H.mat];
      const float4 ec = P.emission_color;
      float4 dc = P.diffuse_color;
      // textureInitPassRT, CTextureApplyPass.process, updateToTextureColorRT
      // (Raytrace.cl:52-145): the quick colour takes the diffuse texel at the hit's uv
      if (S.tex_on && P.isDiffuseTexture && !is_emitter(P)) {
        const int4 t = __ldg(S.tex_ref + 4 * (size_t)H.mat);
        dc = argb_float4(t.y > 0 ? tex_fetch(S.texels, t, H.u, H.v) : 0);
      }
      const V c = is_emitter(P) ? mk(ec.x, ec.y, ec.z, ec.w) : muls(mk(dc.x, dc.y, dc.z, dc.w), coeff);
      argb[id] = pack_argb(c.x, c.y, c.z, 1.f);
      if (group) group[id] = H.mat;
    } else {
      if (E.present) {
        int x, y;
        sph_xy(E.w, E.h, d, &x, &y);
        const float4 e = E.rgb[sph_index(E.w, E.h, x, y)];
        const float ig = 1.f / 2.2f;
        argb[id] = pack_argb(powf(e.x, ig), powf(e.y, ig), powf(e.z, ig), e.w);
      } else {
        argb[id] = pack_argb(0.f, 0.f, 0.f, 1.f);
      }
      if (group) group[id] = -1;
    }
  }
};

__global__ void __launch_bounds__(kTraceThreads, 8)
    k_preview(DevScene S, DevEnv E, PassParams pp, int n, int* argb, int* group, int* work, int* err) {
  bool overflow = false;
  tr::trace_persistent<false, 32>(S, n, work, CameraRays{pp}, PreviewOut{S, E, argb, group}, &overflow);
  if (overflow) atomicExch(err, kDevErrStack);
}

}  // namespace
}  // namespace mt

extern "C" int mt_preview_frame(mt_scene* s, const void* camera, int width, int height, int32_t* argb,
                                int32_t* group) {
  if (!s || !camera || !argb) return fail(MT_ERR_INVALID, "NULL argument");
  if (width <= 0 || height <= 0 || (long long)width * height > (1ll << 28))
    return fail(MT_ERR_INVALID, "frame %d x %d", width, height);
  if (!s->has_bvh) return fail(MT_ERR_INVALID, "scene has no BVH");
  mt_context* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  join_jobs(ctx);
  const int n = width * height;
  PassParams pp{};
  camera_constants(camera, width, height, pp);
  pp.width = width;
  pp.height = height;
  int *d_argb = nullptr, *d_group = nullptr;
  CU(cudaMallocAsync((void**)&d_argb, (size_t)n * 4, ctx->stream));
  if (group) CU(cudaMallocAsync((void**)&d_group, (size_t)n * 4, ctx->stream));
  CU(cudaMemsetAsync(ctx->d_scratch, 0, 8, ctx->stream));
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, mt::k_preview, kTraceThreads, 0);
  const int grid = std::max(1, std::min(ctx->num_sms * std::max(bps, 1), (n + kTraceThreads - 1) / kTraceThreads));
  mt::k_preview<<<grid, kTraceThreads, 0, ctx->stream>>>(s->view(), s->env_view(), pp, n, d_argb, d_group,
                                                         ctx->d_scratch, ctx->d_scratch + 1);
  cudaError_t e = cudaGetLastError();
  int err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(argb, d_argb, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && group)
    e = cudaMemcpyAsync(group, d_group, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, ctx->d_scratch + 1, 4, cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(d_argb, ctx->stream);
  if (d_group) cudaFreeAsync(d_group, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(MT_ERR_CUDA, "preview: %s", cudaGetErrorString(e));
  if (err) return fail(MT_ERR_DEPTH, "BVH deeper than the traversal stack");
  return MT_OK;
}
