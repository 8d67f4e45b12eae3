// Wavefront frame kernels: raygen, closest-hit traversal, fused shading with
// stable queue compaction, shadow traversal with film resolve.
//
// One pass of CDeviceGI.loop (src/cl/device/CDeviceGI.java:214-271) is
//   k_raygen                       InitCameraRayDataJitter + InitPathData +
//                                  InitIntersection + InitIntDataToIndex
//   per bounce b:
//     k_trace_closest              IntersectPrimitives (traversal part)
//     k_shade                      IntersectPrimitives (hit record) + SetupBSDFPath +
//                                  LightHitPass + CCompact.execute + DirectLight (light
//                                  sample and BSDF evaluation) + SampleBSDFRayDirection
//     k_trace_shadow               DirectLight's testOcclusion + addAccum
// with every queue on the device, so a pass needs no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "mt_device.cuh"
#include "mt_kernels.h"
#include "mt_scan.cuh"
#include "mt_traverse.cuh"

namespace mt {

using namespace dv;

namespace {

using namespace scan;

__device__ __forceinline__ void film_add(float4* __restrict__ acc, float4* __restrict__ comp, int pixel, V v, int kahan) {
  if (!abs_valid4(v)) return;  // addAccum, src/cl/kernel/Render.cl:1-7
  V a = acc[pixel];
  if (!kahan) {
    acc[pixel] = add(a, v);
    return;
  }
  V c = comp[pixel];
  V y = sub(v, c);
  V t = add(a, y);
  comp[pixel] = sub(sub(t, a), y);
  acc[pixel] = t;
}

}  // namespace

// ----------------------------------------------------------------- raygen
// InitCameraRayDataJitter (src/cl/kernel/Initialize.cl:129-172) with the
// per-frame camera constants precomputed on the host, plus the path and queue
// resets of InitPathData / InitIntersection / InitIntDataToIndex.
// The camera ray of pixel id (InitCameraRayDataJitter): origin, world direction.
__device__ __forceinline__ void camera_ray(const PassParams* __restrict__ pp, int id, V* o_out, V* d_out) {
  int32_t sx, sy;
  if (pp->mode == 0) {
    sx = pp->seeds[0];
    sy = pp->seeds[1];
  } else {
    stage_seed(0, 0, &sx, &sy);
  }
  Seed s = gen_seed(sx, sy, pp->frame_count, pp->mode == 0 ? id : pixel_gid(id));
  float r0 = rnd(s), r1 = rnd(s);
  const int W = pp->width;
  float px = (float)(id % W), py = (float)(id / W);
  float j1 = pp->inv_w * (2.f * r0 - 1.f);
  float j2 = pp->inv_h * (2.f * r1 - 1.f);
  V d = normalize4(mk(pp->cam_a * (2.f * px / pp->dim_w - 1.f + j1), -2.f * py / pp->dim_h + 1.f + j2, -pp->cam_d, 0.f));
  const float* m = pp->cam_m;
  V z = zero4();
  V m0 = mk(m[0], m[1], m[2], m[3]), m1 = mk(m[4], m[5], m[6], m[7]), m2 = mk(m[8], m[9], m[10], m[11]),
    m3 = mk(m[12], m[13], m[14], m[15]);
  V o = mk(dot3(m0, z) + m0.w, dot3(m1, z) + m1.w, dot3(m2, z) + m2.w, dot3(m3, z) + m3.w);
  if (!(o.w == 1.f)) o = mk(o.x / o.w, o.y / o.w, o.z / o.w, 0.f);
  V dw = mk(dot4(m0, d), dot4(m1, d), dot4(m2, d), 0.f);
  *o_out = o;
  *d_out = dw;
}
// Queue slot and path state g of a new path (InitPathData).
__device__ __forceinline__ void start_path(FrameBufs& fb, int g, V o, V dw) {
  fb.q_o[0][g] = mk(o.x, o.y, o.z, __int_as_float(g));
  fb.q_d[0][g] = mk(dw.x, dw.y, dw.z, 0.f);
  fb.thr[g] = mk(1.f, 1.f, 1.f, 1.f);
  fb.ps[g] = mk(0.f, 0.f, 0.f, 1.f);  // hitpoint.xyz, lastPdfW
  fb.flag[g] = 1;                     // lastSpecular
}
__global__ void k_raygen(const PassParams* __restrict__ pp, Ctrl* ctrl, FrameBufs fb) {
  const int N = pp->width * pp->height;
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id == 0) ctrl->count[1] = N;
  if (id >= N) return;
  V o, dw;
  camera_ray(pp, id, &o, &dw);
  start_path(fb, id, o, dw);
}

// ----------------------------------------------------------- traversal
namespace {
struct QueueRays {
  const float4* qo;
  const float4* qd;
  __device__ __forceinline__ tr::RayT operator()(int i) const {
    return tr::make_ray(__ldg(qo + i), __ldg(qd + i), 0.001f, CUDART_INF_F);  // initGlobalRay, Util.cl:577-587
  }
};
struct HitOut {
  float* t;
  int* prim;
  __device__ __forceinline__ void operator()(int i, const tr::RayT& r, int hit) const {
    t[i] = r.tmax;
    prim[i] = hit;
  }
};
struct ShadowRays {
  const float4* so;
  const float4* sd;
  __device__ __forceinline__ tr::RayT operator()(int i) const {
    float4 o = __ldg(so + i), d = __ldg(sd + i);
    // initGlobalRayT (Util.cl:590-600); a slot without a shadow ray (pixel < 0)
    // gets an empty interval and ends at the first node
    return tr::make_ray(o, d, 0.0001f, __float_as_int(o.w) >= 0 ? d.w : -CUDART_INF_F);
  }
};
struct ShadowResolve {
  const float4* so;
  const float4* sc;
  float4* film;
  float4* film_c;
  int kahan;
  unsigned* traced;
  __device__ __forceinline__ void operator()(int i, const tr::RayT&, int hit) const {
    int pixel = __float_as_int(__ldg(so + i).w);
    if (pixel < 0) return;
    ++*traced;
    if (hit < 0) {  // unoccluded: addAccum(&accum[pixel], contrib), Render.cl:456-461
      float4 c = __ldg(sc + i);
      film_add(film, film_c, pixel, mk(c.x, c.y, c.z, 1.f), kahan);
    }
  }
};
// traversal steps between two refill points of a warp (the default of
// Tuning::refill_steps): measured 576, 588, 608, 614, 608, 595 Mrays/s at 8,
// 16, 32, 64, 128, 256 on the 1M soup
constexpr int kSteps = 64;
}  // namespace

// MINB: resident blocks per SM the register allocation is bounded for (the
// traversal is latency-bound: more resident warps hide more load latency, at
// the price of registers).
// PREC: the BVH format (0 FP32 child boxes, 1 FP16 outward-rounded, 2 the wide
// BVH with 8-bit boxes, 3 4-wide FP16 nodes).
template <int MINB, int PREC>
__global__ void __launch_bounds__(kTraceThreads, MINB) k_trace_closest(DevScene S, Ctrl* ctrl, int b, FrameBufs fb,
                                                                       int steps) {
  const int count = ctrl->count[b];
  bool overflow = false;
  tr::trace_persistent<false, kSteps, QueueRays, HitOut, PREC>(
      S, count, &ctrl->work[2 * b], QueueRays{fb.q_o[(b + 1) & 1], fb.q_d[(b + 1) & 1]}, HitOut{fb.hit_t, fb.hit_prim},
      &overflow, steps);
  if (overflow) atomicExch(&ctrl->error, kDevErrStack);
}

template <int MINB, int PREC>
__global__ void __launch_bounds__(kTraceThreads, MINB) k_trace_shadow(DevScene S, Ctrl* ctrl, int b, int mode,
                                                                      FrameBufs fb, int kahan, int steps) {
  // mode 0: shadow slots are the compacted survivor slots (flagged by pixel >= 0)
  const int count = mode == 0 ? ctrl->count[b + 1] : ctrl->shadow[b];
  bool overflow = false;
  unsigned traced = 0;
  tr::trace_persistent<true, kSteps, ShadowRays, ShadowResolve, PREC>(
      S, count, &ctrl->work[2 * b + 1], ShadowRays{fb.s_o, fb.s_d},
      ShadowResolve{fb.s_o, fb.s_c, fb.film, fb.film_c, kahan, &traced}, &overflow, steps);
  unsigned long long tot = traced;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
  if ((threadIdx.x & 31) == 0 && tot) atomicAdd(&ctrl->rays[2], tot);
  if (overflow) atomicExch(&ctrl->error, kDevErrStack);
}

// ----------------------------------------------------------------- shade
// The per-path work, in two phases around the reference's compaction:
//   shade_hit       IntersectPrimitives' hit record, SetupBSDFPath and
//                   LightHitPass (emitter or environment contribution);
//   shade_continue  the texture pass, DirectLight (light sample, BSDF
//                   evaluation, shadow ray) and SampleBSDFRayDirection, then
//                   Russian roulette in benchmark semantics.
struct PathState {
  bool alive;
  int pixel;                // queue slot's path index (path state)
  int fidx;                 // film index of its pixel
  int local;                // its pixel within its frame (the samples' key)
  const PassParams* pp;     // its frame's parameters
  V thr, ps;
  int spec;
  Hit H;
  Bsdf B;
};
struct ShadeOut {
  bool has_shadow;
  V sho, shd, shc, ndir;
};
// LEAN: an instance for scenes without mesh lights (hence without emitters) lit
// by an environment map through the light grid, the benchmark scenes' case; it
// leaves out the code of the other cases, which keeps the shading kernel's
// instruction footprint small.
template <int LEAN> __device__ __forceinline__ bool mesh_lights(const DevScene& S) { return !LEAN && S.nlights > 0; }
template <int LEAN> __device__ __forceinline__ bool env_present(const DevEnv& E) { return LEAN || E.present; }
template <int LEAN> __device__ __forceinline__ bool grid_on(const DevEnv& E) { return LEAN || E.grid_on; }

// Which frame a path belongs to: one frame (its parameters, film index = path
// index), or a batch of frames sharing the queues (BatchFrames).
struct OneFrame {
  const PassParams* pp;
  __device__ __forceinline__ void operator()(int g, PathState& P) const {
    P.pp = pp;
    P.fidx = g;
    P.local = g;
  }
};
// Frames of a merged batch pass: frame k holds the paths start[k] .. start[k+1]-1
// (pixel g - start[k] of that frame), its film at film[k] .. and its parameters
// at pp[k].
struct BatchFrames {
  const int* start;  // n + 1
  const int* film;   // n
  const PassParams* pp;
  int n;
  __device__ __forceinline__ void operator()(int g, PathState& P) const {
    int lo = 0, hi = n - 1;  // the last frame with start <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(start + mid) <= g) lo = mid;
      else hi = mid - 1;
    }
    P.pp = pp + lo;
    P.local = g - __ldg(start + lo);
    P.fidx = __ldg(film + lo) + P.local;
  }
};

template <int MODE, int LEAN = 0, class Res = OneFrame>
__device__ __forceinline__ void shade_hit(const DevScene& S, const DevEnv& E, Res res, int b, const FrameBufs& fb,
                                          int j, int count, PathState& P) {
  P.alive = false;
  P.pixel = 0;
  P.thr = zero4();
  P.ps = zero4();
  P.spec = 0;
  P.B.mat = -1;
  if (j >= count) return;
  float4 qo = __ldg(fb.q_o[(b + 1) & 1] + j);
  float4 qd = __ldg(fb.q_d[(b + 1) & 1] + j);
  const int pixel = __float_as_int(qo.w);
  P.pixel = pixel;
  res(pixel, P);
  const PassParams* __restrict__ pp = P.pp;
  const int kahan = pp->kahan;
  V o = mk(qo.x, qo.y, qo.z, 0.f), d = mk(qd.x, qd.y, qd.z, 0.f);
  const float t = fb.hit_t[j];
  const int prim = fb.hit_prim[j];
  P.thr = fb.thr[pixel];
  P.ps = fb.ps[pixel];
  P.spec = fb.flag[pixel];
  if (prim >= 0) {
    hit_record(S, o, d, t, prim, P.H);
    P.B = setup_bsdf(S, d, P.H.n, P.H.mat);
    if (P.B.mat >= 0) {
      const Material& M = S.materials[P.B.mat];
      if (!LEAN && is_emitter(M)) {  // LightHitPass emitter branch, Render.cl:76-104
        float pick = 1.f / (float)S.nlights;
        if (MODE == 1 && E.present && S.nlights > 0) pick = pick * 0.5f;
        AreaLight L = get_area_light(S, M, prim);
        float pdfA = 0.f;
        V c = radiance_area(L, d, &pdfA);
        if (zero3(c)) {
          P.alive = true;  // Render.cl:88-89 returns with isect->hit still set
        } else {
          float w = 1.f;
          if (!P.spec) {
            float pdfW = pdf_a_to_w(pdfA, t, P.B.fix.z);
            w = mis2(P.ps.w, pdfW * pick);
          }
          film_add(fb.film, fb.film_c, P.fidx, muls(mul(P.thr, c), w), kahan);
        }
      } else {
        P.alive = true;
      }
    }
  } else if (env_present<LEAN>(E)) {  // LightHitPass environment branch, Render.cl:106-123
    float pdfW = 0.f;
    V c;
    if (MODE == 1 && grid_on<LEAN>(E))
      c = radiance_env_grid(E, pp->cam_pos, P.ps, d, &pdfW, pp->grid_accum && !P.spec);
    else
      c = radiance_env(E, d, &pdfW);
    if (!zero3(c)) {
      if (MODE == 1 && mesh_lights<LEAN>(S)) pdfW = pdfW * 0.5f;
      float w = 1.f;
      if (!P.spec) w = mis2(P.ps.w, pdfW);
      film_add(fb.film, fb.film_c, P.fidx, muls(mul(P.thr, c), w), kahan);
    }
  }
}

// A path that shade_hit kept going (benchmark semantics), loaded again from its
// queue slot j: the hit record and BSDF set-up are recomputed from the same
// inputs by the same code, so they equal what shade_hit computed.
template <class Res>
__device__ __forceinline__ void shade_load(const DevScene& S, Res res, int b, const FrameBufs& fb, int j,
                                           PathState& P) {
  const float4 qo = __ldg(fb.q_o[(b + 1) & 1] + j);
  const float4 qd = __ldg(fb.q_d[(b + 1) & 1] + j);
  const int pixel = __float_as_int(qo.w);
  P.alive = true;
  P.pixel = pixel;
  res(pixel, P);
  const V o = mk(qo.x, qo.y, qo.z, 0.f), d = mk(qd.x, qd.y, qd.z, 0.f);
  P.thr = fb.thr[pixel];
  P.ps = fb.ps[pixel];
  P.spec = fb.flag[pixel];
  hit_record(S, o, d, __ldg(fb.hit_t + j), __ldg(fb.hit_prim + j), P.H);
  P.B = setup_bsdf(S, d, P.H.n, P.H.mat);
}

// gid: the work-item id the samples are keyed on (mode 0: the compacted slot,
// mode 1: the pixel's id). Writes the path state back; P.alive turns false when
// Russian roulette ends the path.
template <int MODE, bool TEX, int LEAN = 0>
__device__ __forceinline__ void shade_continue(const DevScene& S, const DevEnv& E, int b, const FrameBufs& fb,
                                               int gid, PathState& P, ShadeOut& R) {
  const PassParams* __restrict__ pp = P.pp;
  const float fc = pp->frame_count;
  R.has_shadow = false;
  R.ndir = zero4();
  Bsdf B = P.B;
  Material tm;  // the path's textured copy of its material
  if (TEX && has_textures(*B.pm)) {
    tm = *B.pm;
    apply_textures(S, B.mat, P.H.u, P.H.v, tm);
    B.pm = &tm;
  }
  int32_t lx, ly, bx, by;
  if (MODE == 0) {
    lx = pp->seeds[2 * (2 * b)];
    ly = pp->seeds[2 * (2 * b) + 1];
    bx = lx;
    by = ly;
  } else {
    stage_seed(b, 1, &lx, &ly);
    stage_seed(b, 2, &bx, &by);
  }
  Seed s = gen_seed(lx, ly, fc, gid);
  V dir = zero4();
  float dist = 0.f, pdfW = 0.f, pick = 1.f;
  V smp;
  smp.x = rnd(s);
  smp.y = rnd(s);
  smp.z = rnd(s);
  smp.w = rnd(s);
  V rad = zero4();
  bool smesh = false, senv = false;
  if (env_present<LEAN>(E) && mesh_lights<LEAN>(S)) {
    float r = rnd(s);
    pick = pick * 0.5f;
    if (r < 0.5f) smesh = true; else senv = true;
  } else if (env_present<LEAN>(E)) {
    senv = true;
  } else if (mesh_lights<LEAN>(S)) {
    smesh = true;
  }
  if (smesh) {
    int li = (int)(rnd(s) * (float)S.nlights);
    li = li < S.nlights ? li : S.nlights - 1;  // rounding of rnd * n for n > 2^22
    int tri = S.light_faces[MODE == 0 ? 0 : li];  // Render.cl:305 reads light 0
    pick = pick * (1.f / (float)S.nlights);
    const Material& Ml = S.materials[__ldg(reinterpret_cast<const int*>(S.faces + tri) + 9) & 0xFFFF];
    AreaLight L = get_area_light(S, Ml, tri);
    rad = illuminate_area(L, P.H.p, smp.x, smp.y, &dir, &dist, &pdfW);
  } else if (senv) {
    if (MODE == 1 && grid_on<LEAN>(E))
      rad = illuminate_env_grid(E, pp->cam_pos, P.H.p, smp, &dir, &dist, &pdfW);
    else
      rad = illuminate_env(E, smp, &dir, &dist, &pdfW);
  }
  if (!zero3(rad)) {
    float bpdf = 0.f, cosO = 0.f;
    V f = eval_bsdf(S, B, dir, &bpdf, &cosO);
    if (!zero3(f)) {
      float w = mis2(pdfW, bpdf);
      float sc = (w * cosO / (pick * pdfW));
      R.shc = mk(sc * (rad.x * f.x) * P.thr.x, sc * (rad.y * f.y) * P.thr.y, sc * (rad.z * f.z) * P.thr.z, 1.f);
      R.sho = mk(P.H.p.x, P.H.p.y, P.H.p.z, __int_as_float(P.fidx));
      R.shd = mk(dir.x, dir.y, dir.z, dist - 2.f * 1e-3f);
      R.has_shadow = true;
    }
  }
  // BSDF sample
  Seed s2 = gen_seed(bx, by, fc, gid);
  float s0 = rnd(s2), s1 = rnd(s2), sz = rnd(s2);
  float pdf = 0.f, cosO = 0.f;
  V f = sample_bsdf(S, B, s0, s1, sz, &R.ndir, &pdf, &cosO);
  float q = cosO / pdf;
  V thr = mul(P.thr, muls(f, q));
  V ps = mk(P.H.p.x, P.H.p.y, P.H.p.z, pdf);
  if (MODE == 1 && pp->rr_depth > 0 && b >= pp->rr_depth) {
    int32_t rx, ry;
    stage_seed(b, 3, &rx, &ry);
    Seed rs = gen_seed(rx, ry, fc, gid);
    float u = rnd(rs);
    float mx = maxf_(thr.x, maxf_(thr.y, thr.z));
    float cont = minf_(0.95f, mx);
    if (!(u < cont)) P.alive = false;
    else thr = divs(thr, cont);
  }
  fb.thr[P.pixel] = thr;
  fb.ps[P.pixel] = ps;
  fb.flag[P.pixel] = 0;
}

// Benchmark semantics: a warp appends its survivors to the next queue and its
// shadow rays to the shadow queue, one atomic per queue (ranks by ballot).
__device__ __forceinline__ void append_warp(Ctrl* ctrl, int b, const FrameBufs& fb, const PathState& P,
                                            const ShadeOut& R) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int nq = b & 1;  // queue written for bounce b + 1
  const unsigned am = __ballot_sync(0xffffffffu, P.alive), sm = __ballot_sync(0xffffffffu, R.has_shadow);
  int qa = 0, qs = 0;
  if (lane == 0) {
    if (am) qa = atomicAdd(&ctrl->count[b + 1], __popc(am));
    if (sm) qs = atomicAdd(&ctrl->shadow[b], __popc(sm));
  }
  qa = __shfl_sync(0xffffffffu, qa, 0);
  qs = __shfl_sync(0xffffffffu, qs, 0);
  if (P.alive) {
    const int slot = qa + __popc(am & lt);
    fb.q_o[nq][slot] = mk(P.H.p.x, P.H.p.y, P.H.p.z, __int_as_float(P.pixel));
    fb.q_d[nq][slot] = mk(R.ndir.x, R.ndir.y, R.ndir.z, 0.f);
  }
  if (R.has_shadow) {
    const int sslot = qs + __popc(sm & lt);
    fb.s_o[sslot] = R.sho;
    fb.s_d[sslot] = R.shd;
    fb.s_c[sslot] = R.shc;
  }
}

// Reference semantics (mode 0), one 256-path tile per block: survivors are
// compacted in order (block scan + decoupled look-back) between the two phases,
// and the light and BSDF samples of a survivor are keyed on its compacted slot
// as DirectLight and SampleBSDFRayDirection key them on get_global_id; the
// shadow ray of survivor j' sits at shadow slot j' (pixel -1: none).
// TEX: the scene has textures (a separate instance keeps the untextured one lean).
template <int MINB, bool TEX = false>
__global__ void __launch_bounds__(kShadeThreads, MINB) k_shade_ref(DevScene S, DevEnv E, const PassParams* __restrict__ pp,
                                                             Ctrl* ctrl, int b, FrameBufs fb,
                                                             unsigned long long* status) {
  __shared__ unsigned long long sh[kShadeThreads / 32 + 1];
  __shared__ int s_tile;
  __shared__ unsigned long long s_base;
  const int count = ctrl->count[b];
  const int ntiles = (count + kShadeThreads - 1) / kShadeThreads;
  if (threadIdx.x == 0) s_tile = atomicAdd(&ctrl->tiles[b], 1);
  __syncthreads();
  const int tile = s_tile;
  if (tile >= ntiles) return;
  const int j = tile * kShadeThreads + threadIdx.x;
  PathState P;
  shade_hit<0>(S, E, OneFrame{pp}, b, fb, j, count, P);
  unsigned long long tot = 0;
  unsigned long long excl = block_rank2<kShadeThreads>(P.alive, false, &tot, sh);
  if (threadIdx.x == 0) s_base = lookback(status, tile, tot, &ctrl->error);
  __syncthreads();
  const int slot = (int)(s_base + excl);
  if (tile == ntiles - 1 && threadIdx.x == 0) {
    ctrl->count[b + 1] = (int)(s_base + tot);
    ctrl->shadow[b] = (int)(s_base + tot);
  }
  if (!P.alive) return;
  ShadeOut R;
  shade_continue<0, TEX>(S, E, b, fb, slot, P, R);
  const int nq = b & 1;  // queue written for bounce b + 1
  fb.q_o[nq][slot] = mk(P.H.p.x, P.H.p.y, P.H.p.z, __int_as_float(P.pixel));
  fb.q_d[nq][slot] = mk(R.ndir.x, R.ndir.y, R.ndir.z, 0.f);
  if (R.has_shadow) {
    fb.s_o[slot] = R.sho;
    fb.s_d[slot] = R.shd;
    fb.s_c[slot] = R.shc;
  } else {
    fb.s_o[slot] = mk(0.f, 0.f, 0.f, __int_as_float(-1));
  }
}

// Benchmark semantics (mode 1): samples are keyed on the pixel, so the order of
// the queues carries no meaning and no block ever waits for another. Warps run
// persistently over 32-path chunks (a chunk counter per bounce); each warp
// appends its survivors and its shadow rays to the next queues with one atomic
// per queue per chunk (ballot ranks inside the warp). Russian roulette runs after
// the BSDF sample.
// Res: OneFrame (pp = the frame's parameters) or BatchFrames (a merged batch pass).
template <int MINB, bool TEX = false, int LEAN = 0, class Res = OneFrame>
__global__ void __launch_bounds__(kShadeThreads, MINB) k_shade(DevScene S, DevEnv E, Res res, Ctrl* ctrl, int b,
                                                         FrameBufs fb) {
  const int count = ctrl->count[b];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int nq = b & 1;  // queue written for bounce b + 1
  for (;;) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(&ctrl->tiles[b], 1);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk * 32 >= count) break;
    const int j = chunk * 32 + lane;
    PathState P;
    shade_hit<1, LEAN>(S, E, res, b, fb, j, count, P);
    ShadeOut R;
    R.has_shadow = false;
    if (P.alive) shade_continue<1, TEX, LEAN>(S, E, b, fb, pixel_gid(P.local), P, R);
    const unsigned am = __ballot_sync(0xffffffffu, P.alive), sm = __ballot_sync(0xffffffffu, R.has_shadow);
    int qa = 0, qs = 0;
    if (lane == 0) {
      if (am) qa = atomicAdd(&ctrl->count[b + 1], __popc(am));
      if (sm) qs = atomicAdd(&ctrl->shadow[b], __popc(sm));
    }
    qa = __shfl_sync(0xffffffffu, qa, 0);
    qs = __shfl_sync(0xffffffffu, qs, 0);
    if (P.alive) {
      const int slot = qa + __popc(am & lt);
      fb.q_o[nq][slot] = mk(P.H.p.x, P.H.p.y, P.H.p.z, __int_as_float(P.pixel));
      fb.q_d[nq][slot] = mk(R.ndir.x, R.ndir.y, R.ndir.z, 0.f);
    }
    if (R.has_shadow) {
      const int sslot = qs + __popc(sm & lt);
      fb.s_o[sslot] = R.sho;
      fb.s_d[sslot] = R.shd;
      fb.s_c[sslot] = R.shc;
    }
  }
}

// Benchmark semantics in two launches (the default; MT_SHADE_SPLIT=0 runs the
// single kernel above). k_shade_hit runs the hit record, the BSDF set-up and
// LightHitPass over the whole queue and lists the slots of the paths that go
// on; k_shade_cont runs the texture pass, DirectLight, SampleBSDFRayDirection
// and Russian roulette over that list alone. Each is half the code (less
// instruction fetch), and the second runs on full warps instead of warps whose
// terminated paths idle through the light and BSDF samples. Samples are keyed on
// the pixel, so the list's order carries no meaning.
template <int MINB, int LEAN = 0, class Res = OneFrame>
__global__ void __launch_bounds__(kShadeThreads, MINB) k_shade_hit(DevScene S, DevEnv E, Res res, Ctrl* ctrl, int b,
                                                             FrameBufs fb) {
  const int count = ctrl->count[b];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(&ctrl->tiles[b], 1);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk * 32 >= count) break;
    const int j = chunk * 32 + lane;
    PathState P;
    shade_hit<1, LEAN>(S, E, res, b, fb, j, count, P);
    const unsigned am = __ballot_sync(0xffffffffu, P.alive);
    int base = 0;
    if (lane == 0 && am) base = atomicAdd(&ctrl->live[b], __popc(am));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (P.alive) fb.live[base + __popc(am & lt)] = j;
  }
}

template <int MINB, bool TEX = false, int LEAN = 0, class Res = OneFrame>
__global__ void __launch_bounds__(kShadeThreads, MINB) k_shade_cont(DevScene S, DevEnv E, Res res, Ctrl* ctrl, int b,
                                                              FrameBufs fb) {
  const int count = ctrl->live[b];
  const int lane = threadIdx.x & 31;
  for (;;) {
    int chunk = 0;
    if (lane == 0) chunk = atomicAdd(&ctrl->tiles2[b], 1);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk * 32 >= count) break;
    const int k = chunk * 32 + lane;
    PathState P;
    P.alive = false;
    ShadeOut R;
    R.has_shadow = false;
    if (k < count) {
      shade_load(S, res, b, fb, __ldg(fb.live + k), P);
      shade_continue<1, TEX, LEAN>(S, E, b, fb, pixel_gid(P.local), P, R);
    }
    append_warp(ctrl, b, fb, P, R);
  }
}

// Adds a finished pass's ray counts into the job's running totals
// [primary, extension, shadow].
__global__ void k_accumulate(const Ctrl* ctrl, int max_depth, int n_pixels, unsigned long long* totals) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long ext = 0;
  for (int b = 2; b <= max_depth; ++b) ext += (unsigned long long)ctrl->count[b];
  // frames of in-flight slots finish concurrently: the totals are shared
  atomicAdd(totals + 0, (unsigned long long)n_pixels);
  atomicAdd(totals + 1, ext);
  atomicAdd(totals + 2, (unsigned long long)ctrl->rays[2]);
  if (ctrl->error) atomicExch(totals + 3, (unsigned long long)ctrl->error);
}

// ---------------------------------------------------------------- launchers
namespace {
// Register bounds of the traversal kernels (resident 128-thread blocks per SM):
// measured best on the 1M soup, 12 for closest hits (42 registers, a few bytes
// of spill) and 8 for shadow rays. MT_TRACE_MINB / MT_SHADOW_MINB (8, 12 or 16)
// select another build of either.
int env_minb(const char* name, int dflt) {
  const char* e = std::getenv(name);
  int x = e ? std::atoi(e) : dflt;
  return (x == 8 || x == 12 || x == 16) ? x : dflt;
}
// Persistent traversal grids of a shared pass, in blocks per SM (MT_TRACE_GRID /
// MT_SHADOW_GRID; 0: half of what fits). Frames in flight run their launches
// side by side, so a launch that leaves room on each SM lets another frame's
// kernels run there. Measured on the 1M soup with six frames in flight (blocks
// per SM for closest / shadow rays): 12/8 (all that fits) 613-616 Mrays/s,
// 8/8 637, 8/4 644, 6/4 633-651, 4/4 653, 3/3 651.
int grid_bps(const char* name, int dflt) {
  const char* e = std::getenv(name);
  int x = e ? std::atoi(e) : dflt;
  return x >= 0 && x <= 32 ? x : dflt;
}
// Resident 256-thread blocks per SM the benchmark-semantics shading kernel is
// bounded for (MT_SHADE_MINB: 3, 4 or 5).
int env_shade_minb() {
  const char* e = std::getenv("MT_SHADE_MINB");
  int x = e ? std::atoi(e) : kShadeMinBlocks;
  return (x == 3 || x == 4 || x == 5) ? x : kShadeMinBlocks;
}
// MT_SHADE_SPLIT: unset, render jobs choose one or two shading launches frame by
// frame (shade_split_for) and other passes take two; 0 always one; 1 always two.
int shade_split_mode() {
  static const int m = [] {
    const char* e = std::getenv("MT_SHADE_SPLIT");
    if (!e) return -1;
    return std::atoi(e) == 0 ? 0 : 1;
  }();
  return m;
}
bool shade_split() { return shade_split_mode() != 0; }

int env_steps() {
  const char* e = std::getenv("MT_REFILL_STEPS");
  int x = e ? std::atoi(e) : kSteps;
  return x >= 4 && x <= 1024 ? x : kSteps;
}
// The process's launch shapes: the defaults above, the MT_* knobs, then
// whatever set_tuning installs.
Tuning& tuning_ref() {
  static Tuning t = {env_minb("MT_TRACE_MINB", kTraceMinBlocksClosest), env_minb("MT_SHADOW_MINB", kTraceMinBlocksShadow),
                     grid_bps("MT_TRACE_GRID", 0), grid_bps("MT_SHADOW_GRID", 0), env_shade_minb(), env_steps(),
                     std::getenv("MT_SHADOW_STREAM") && std::atoi(std::getenv("MT_SHADOW_STREAM")) == 0 ? 0 : 1};
  return t;
}
std::atomic<unsigned> g_tuning_version{1};
int trace_grid_bps() { return tuning_ref().closest_grid; }
int shadow_grid_bps() { return tuning_ref().shadow_grid; }
int trace_minb() { return tuning_ref().closest_minb; }
int shadow_minb() { return tuning_ref().shadow_minb; }
int shade_minb() { return tuning_ref().shade_minb; }
// Resident blocks per SM of the benchmark-semantics shading kernel (its grid is
// one resident wave of persistent warps).
int shade_blocks_per_sm(int minb) {
  int n = 0;
  if (minb == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<4>, kShadeThreads, 0);
  else if (minb == 5) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<5>, kShadeThreads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<3>, kShadeThreads, 0);
  return n > 0 ? n : 1;
}
template <int MINB>
int trace_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace_closest<MINB, 0>, kTraceThreads, 0);
  return n > 0 ? n : 1;
}
// The wide-BVH kernels are built for 8 resident blocks per SM whatever the
// tuning's bound (at 12 or 16 their wide node tests spill registers), and
// refill after an eighth of the binary kernels' steps (a wide step tests eight
// child boxes; measured on the 1M soup at 1080p, refill every 4, 8, 12, 16, 32,
// 64 wide steps: bounce-1 closest hits 1.73, 1.76, 1.81, 1.86, 2.02, 2.21 ms).
constexpr int kWideMinBlocks = 8;
int wide_steps_of(int steps) { return std::max(2, steps / 8); }
int wide_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace_closest<kWideMinBlocks, 2>, kTraceThreads, 0);
  return n > 0 ? n : 1;
}
// 4-wide FP16 nodes (built for the tuning's bound like the binary kernels): a
// step visits a node of four child boxes (two binary levels) or tests a triangle.
int quad_steps_of(int steps) { return std::max(2, steps / 2); }
template <int MINB>
void launch_traces(cudaStream_t st, int grid, const DevScene& S, Ctrl* ctrl, int b, int mode, FrameBufs fb, int kahan,
                   bool closest) {
  const int steps = tuning_ref().refill_steps;
  if (S.bitstack && S.precision <= 1) {
    if (closest) {
      if (S.precision == 1) k_trace_closest<MINB, 5><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, steps);
      else k_trace_closest<MINB, 4><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, steps);
    } else {
      if (S.precision == 1) k_trace_shadow<MINB, 5><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan, steps);
      else k_trace_shadow<MINB, 4><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan, steps);
    }
    return;
  }
  if (closest) {
    const int f = S.precision;
    if (f == 3)
      k_trace_closest<MINB, 3><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, quad_steps_of(steps));
    else if (f == 2)
      k_trace_closest<kWideMinBlocks, 2><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, wide_steps_of(steps));
    else if (f == 1)
      k_trace_closest<MINB, 1><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, steps);
    else
      k_trace_closest<MINB, 0><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, fb, steps);
  } else {
    const int f = S.precision;
    if (f == 3)
      k_trace_shadow<MINB, 3><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan, quad_steps_of(steps));
    else if (f == 2)
      k_trace_shadow<kWideMinBlocks, 2><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan,
                                                                        wide_steps_of(steps));
    else if (f == 1)
      k_trace_shadow<MINB, 1><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan, steps);
    else
      k_trace_shadow<MINB, 0><<<grid, kTraceThreads, 0, st>>>(S, ctrl, b, mode, fb, kahan, steps);
  }
}
}  // namespace

Tuning get_tuning() { return tuning_ref(); }

int shade_split_setting() { return shade_split_mode(); }

// Measured with six frames in flight: the 1M soup (53 % of bounce-1 paths go
// on) 915 Mrays/s in two launches against 861 in one; the stadium (71 % go on)
// 2588 against 2743. A band around the crossover keeps the current choice.
int shade_split_for(int queued, int went_on, int current) {
  if (queued <= 0) return current;
  const double f = (double)went_on / queued;
  if (f < 0.58) return 1;
  if (f > 0.66) return 0;
  return current;
}

bool set_tuning(const Tuning& t) {
  auto minb_ok = [](int x) { return x == 8 || x == 12 || x == 16; };
  if (!minb_ok(t.closest_minb) || !minb_ok(t.shadow_minb) || t.closest_grid < 0 || t.closest_grid > 32 ||
      t.shadow_grid < 0 || t.shadow_grid > 32 || t.shade_minb < 3 || t.shade_minb > 5 || t.refill_steps < 4 ||
      t.refill_steps > 1024 || (t.shadow_stream != 0 && t.shadow_stream != 1))
    return false;
  tuning_ref() = t;
  g_tuning_version.fetch_add(1);
  return true;
}

unsigned tuning_version() { return g_tuning_version.load(); }

// One persistent traversal launch over a queue of at most N rays.
void launch_trace(cudaStream_t st, const DevScene& S, Ctrl* ctrl, int b, int mode, FrameBufs fb, int kahan, bool closest,
                  int N, int num_sms, bool shared) {
  static int bps[17] = {};
  static int wide_bps = 0;
  const int minb = closest ? trace_minb() : shadow_minb();
  if (bps[minb] == 0)
    bps[minb] = minb == 16 ? trace_blocks_per_sm<16>() : minb == 12 ? trace_blocks_per_sm<12>() : trace_blocks_per_sm<8>();
  if (wide_bps == 0) wide_bps = wide_blocks_per_sm();
  const int fit = S.precision == 2 ? wide_bps : bps[minb];
  const int want = closest ? trace_grid_bps() : shadow_grid_bps();
  const int per_sm = !shared ? fit : want > 0 ? std::min(want, fit) : std::max(1, fit / 2);
  const int grid = std::max(1, std::min(num_sms * per_sm, (N + kTraceThreads - 1) / kTraceThreads));
  if (minb == 16) launch_traces<16>(st, grid, S, ctrl, b, mode, fb, kahan, closest);
  else if (minb == 12) launch_traces<12>(st, grid, S, ctrl, b, mode, fb, kahan, closest);
  else launch_traces<8>(st, grid, S, ctrl, b, mode, fb, kahan, closest);
}

int launch_pass(cudaStream_t st, const DevScene& S, const DevEnv& E, const PassParams* d_pp, int mode, int max_depth,
                int kahan, int width, int height, Ctrl* ctrl, FrameBufs fb, unsigned long long* status,
                size_t status_stride, int num_sms, cudaEvent_t* ev, unsigned long long* totals, bool shared,
                cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, int shade_split_req) {
  const bool two_launches = shade_split_req < 0 ? shade_split() : shade_split_req != 0;
  const int N = width * height;
  static int shade_bps[6] = {};
  // shadow rays of bounce b beside the extension rays of bounce b + 1 (no
  // per-kernel events): both read only what shading b wrote (in reference
  // semantics both read its survivor count), and shading b + 1, which rewrites
  // the shadow queue and adds to the film after the shadow kernel's adds, waits
  // for them
  const bool split = side && fork && join && !ev && tuning_ref().shadow_stream;
  if (split) shared = true;
  auto trace = [&](bool closest, int b) { launch_trace(st, S, ctrl, b, mode, fb, kahan, closest, N, num_sms, shared); };
  // persistent traversal: one resident wave, or fewer blocks for a small frame
  // (a queue never exceeds the frame's pixels), leaving SMs to other streams
  const int tiles = (N + kShadeThreads - 1) / kShadeThreads;
  int e = 0;
  if (ev) cudaEventRecord(ev[e++], st);
  k_raygen<<<(N + 255) / 256, 256, 0, st>>>(d_pp, ctrl, fb);
  if (ev) cudaEventRecord(ev[e++], st);
  for (int b = 1; b <= max_depth; ++b) {
    trace(true, b);
    if (ev) cudaEventRecord(ev[e++], st);
    if (split && b > 1) cudaStreamWaitEvent(st, join, 0);
    unsigned long long* stb = status + (size_t)(b - 1) * status_stride;
    if (mode == 0) {
      if (S.tex_on)
        k_shade_ref<3, true><<<tiles, kShadeThreads, 0, st>>>(S, E, d_pp, ctrl, b, fb, stb);
      else
        k_shade_ref<3><<<tiles, kShadeThreads, 0, st>>>(S, E, d_pp, ctrl, b, fb, stb);
    } else if (two_launches) {
      const int sm = shade_minb();
      if (shade_bps[sm] == 0) shade_bps[sm] = shade_blocks_per_sm(sm);
      const int sgrid = std::max(1, std::min(num_sms * shade_bps[sm], tiles));
      const bool lean = S.nlights == 0 && E.present && E.grid_on && !S.tex_on;
      const OneFrame R1{d_pp};
      if (lean)
        k_shade_hit<4, 1><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      else
        k_shade_hit<4><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      if (S.tex_on)
        k_shade_cont<4, true><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      else if (lean && sm == 4)
        k_shade_cont<4, false, 1><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      else if (sm == 4)
        k_shade_cont<4><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      else if (sm == 5)
        k_shade_cont<5><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
      else
        k_shade_cont<3><<<sgrid, kShadeThreads, 0, st>>>(S, E, R1, ctrl, b, fb);
    } else {
      const int sm = shade_minb();
      if (shade_bps[sm] == 0) shade_bps[sm] = shade_blocks_per_sm(sm);
      const int sgrid = std::max(1, std::min(num_sms * shade_bps[sm], tiles));
      const bool lean = S.nlights == 0 && E.present && E.grid_on;
      if (S.tex_on)
        k_shade<4, true><<<sgrid, kShadeThreads, 0, st>>>(S, E, OneFrame{d_pp}, ctrl, b, fb);
      else if (lean && sm == 4)
        k_shade<4, false, 1><<<sgrid, kShadeThreads, 0, st>>>(S, E, OneFrame{d_pp}, ctrl, b, fb);
      else if (sm == 4)
        k_shade<4><<<sgrid, kShadeThreads, 0, st>>>(S, E, OneFrame{d_pp}, ctrl, b, fb);
      else if (sm == 5)
        k_shade<5><<<sgrid, kShadeThreads, 0, st>>>(S, E, OneFrame{d_pp}, ctrl, b, fb);
      else
        k_shade<3><<<sgrid, kShadeThreads, 0, st>>>(S, E, OneFrame{d_pp}, ctrl, b, fb);
    }
    if (ev) cudaEventRecord(ev[e++], st);
    if (split) {
      cudaEventRecord(fork, st);
      cudaStreamWaitEvent(side, fork, 0);
      launch_trace(side, S, ctrl, b, mode, fb, kahan, false, N, num_sms, shared);
      cudaEventRecord(join, side);
    } else {
      trace(false, b);
    }
    if (ev) cudaEventRecord(ev[e++], st);
  }
  if (split) cudaStreamWaitEvent(st, join, 0);
  if (totals) k_accumulate<<<1, 32, 0, st>>>(ctrl, max_depth, N, totals);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

namespace {
// Camera rays of a merged batch pass: path g is pixel g - start[k] of frame k.
__global__ void k_raygen_batch(BatchFrames B, int total, Ctrl* ctrl, FrameBufs fb) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g == 0) ctrl->count[1] = total;
  if (g >= total) return;
  PathState P;
  B(g, P);
  V o, dw;
  camera_ray(P.pp, P.local, &o, &dw);
  start_path(fb, g, o, dw);
}
}  // namespace

int launch_batch_pass(cudaStream_t st, const DevScene& S, const DevEnv& E, const int* d_start, const int* d_film,
                      const PassParams* d_pp, int nframes, int total, int max_depth, int kahan, Ctrl* ctrl,
                      FrameBufs fb, int num_sms, unsigned long long* totals, bool shared) {
  const BatchFrames B{d_start, d_film, d_pp, nframes};
  static int shade_bps = 0;
  if (shade_bps == 0) shade_bps = shade_blocks_per_sm(4);
  const int tiles = (total + kShadeThreads - 1) / kShadeThreads;
  const int sgrid = std::max(1, std::min(num_sms * shade_bps, tiles));
  k_raygen_batch<<<(total + 255) / 256, 256, 0, st>>>(B, total, ctrl, fb);
  for (int b = 1; b <= max_depth; ++b) {
    launch_trace(st, S, ctrl, b, 1, fb, kahan, true, total, num_sms, shared);
    if (shade_split()) {
      k_shade_hit<4, 0, BatchFrames><<<sgrid, kShadeThreads, 0, st>>>(S, E, B, ctrl, b, fb);
      if (S.tex_on)
        k_shade_cont<4, true, 0, BatchFrames><<<sgrid, kShadeThreads, 0, st>>>(S, E, B, ctrl, b, fb);
      else
        k_shade_cont<4, false, 0, BatchFrames><<<sgrid, kShadeThreads, 0, st>>>(S, E, B, ctrl, b, fb);
    } else if (S.tex_on)
      k_shade<4, true, 0, BatchFrames><<<sgrid, kShadeThreads, 0, st>>>(S, E, B, ctrl, b, fb);
    else
      k_shade<4, false, 0, BatchFrames><<<sgrid, kShadeThreads, 0, st>>>(S, E, B, ctrl, b, fb);
    launch_trace(st, S, ctrl, b, 1, fb, kahan, false, total, num_sms, shared);
  }
  if (totals) k_accumulate<<<1, 32, 0, st>>>(ctrl, max_depth, total, totals);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Ray queries on reference-layout rays (80 B): closest or any hit.
namespace {
struct RefRays {
  const float4* rays;
  __device__ __forceinline__ tr::RayT operator()(int i) const {
    const float4* R = rays + 5 * (size_t)i;  // Ray: o, d, inv_d, sign, (extra, tMin, tMax)
    float4 o = __ldg(R + 0), d = __ldg(R + 1), tail = __ldg(R + 4);
    return tr::make_ray(o, d, tail.z, tail.w);
  }
};
struct QueryOut {
  int any;
  float* t;
  int* prim;
  __device__ __forceinline__ void operator()(int i, const tr::RayT& r, int hit) const {
    if (any) {
      prim[i] = hit >= 0 ? 1 : 0;
    } else {
      t[i] = r.tmax;
      prim[i] = hit;
    }
  }
};
}  // namespace

template <int PREC>
__global__ void __launch_bounds__(kTraceThreads, 8) k_query(DevScene S, const float4* __restrict__ rays, int n, int any,
                                                            float* __restrict__ t_out, int* __restrict__ prim_out,
                                                            int* work, int* err) {
  bool overflow = false;
  const int steps = PREC == 2 ? kSteps / 8 : PREC == 3 ? kSteps / 2 : kSteps;  // 4, 5: stackless binary
  if (any)
    tr::trace_persistent<true, kSteps, RefRays, QueryOut, PREC>(S, n, work, RefRays{rays}, QueryOut{1, t_out, prim_out},
                                                                &overflow, steps);
  else
    tr::trace_persistent<false, kSteps, RefRays, QueryOut, PREC>(S, n, work, RefRays{rays},
                                                                 QueryOut{0, t_out, prim_out}, &overflow, steps);
  if (overflow) atomicExch(err, kDevErrStack);
}

// Traversal work per ray: the same traversal as k_query, one step at a time,
// counting interior-node visits and triangle tests (counts[2 i], counts[2 i + 1]).
// Binary records: the visits the reference's algorithm makes (a step is one or
// the other, classified before it runs); the wide BVH: its node visits (96-byte
// nodes); 4-wide FP16 nodes: their node visits (64-byte nodes).
template <int PREC, bool ANY>
__global__ void __launch_bounds__(kTraceThreads) k_count(DevScene S, const float4* __restrict__ rays, int n,
                                                         float* __restrict__ t_out, int* __restrict__ prim_out,
                                                         int* __restrict__ counts, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tr::RayT r = RefRays{rays}(i);
  bool overflow = false;
  int hit = -1, sp = 0, visits = 0, tests = 0;
  if constexpr (PREC == 2) {
    uint2 stack[kWideStack];
    tr::WideState w;
    tr::wide_init(r, w);
    int cnt[2] = {0, 0};
    while (!tr::wide_steps<ANY>(S, r, w, sp, hit, stack, 1, &overflow, cnt)) {
    }
    visits = cnt[0];
    tests = cnt[1];
  } else {
    typename tr::StackEntry<ANY>::type stack[PREC == 3 ? kQuadStack : kStackDepth], top;
    int ref = S.root_ref;
    const bool finite = tr::ray_is_finite(r);
    if constexpr (PREC >= 4) {
      unsigned long long bits = 0;
      int par = -1, sib = -1;
      for (;;) {
        const bool node = ref >= 0;
        const bool done = tr::bitstack_steps<ANY, PREC - 4>(S, r, ref, bits, par, sib, hit, finite, 1);
        visits += node;
        tests += !node;
        if (done) break;
      }
    } else if constexpr (PREC == 3) {
      int leaf = kQuadEmpty, cnt[2] = {0, 0};
      while (!tr::quad_steps<ANY>(S, r, ref, leaf, sp, hit, finite, stack, top, 1, &overflow, cnt)) {
      }
      visits = cnt[0];
      tests = cnt[1];
    } else {
      for (;;) {
        const bool node = ref >= 0;
        const bool done = tr::trav_steps<ANY, PREC>(S, r, ref, sp, hit, finite, stack, top, 1, &overflow);
        visits += node;
        tests += !node;
        if (done) break;
      }
    }
  }
  if (overflow) atomicExch(err, kDevErrStack);
  QueryOut{ANY ? 1 : 0, t_out, prim_out}(i, r, hit);
  counts[2 * i] = visits;
  counts[2 * i + 1] = tests;
}

int launch_count(cudaStream_t st, const DevScene& S, const float4* rays, int n, int any, float* t_out, int* prim_out,
                 int* counts, int* err) {
  const int g = (n + kTraceThreads - 1) / kTraceThreads;
  if (n <= 0) return 0;
#define MT_COUNT(P)                                                                              \
  if (any) k_count<P, true><<<g, kTraceThreads, 0, st>>>(S, rays, n, t_out, prim_out, counts, err); \
  else k_count<P, false><<<g, kTraceThreads, 0, st>>>(S, rays, n, t_out, prim_out, counts, err);
  const int f = S.bitstack && S.precision <= 1 ? 4 + S.precision : S.precision;
  if (f == 5) {
    MT_COUNT(5)
  } else if (f == 4) {
    MT_COUNT(4)
  } else if (f == 3) {
    MT_COUNT(3)
  } else if (f == 2) {
    MT_COUNT(2)
  } else if (f == 1) {
    MT_COUNT(1)
  } else {
    MT_COUNT(0)
  }
#undef MT_COUNT
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_query(cudaStream_t st, const DevScene& S, const float4* rays, int n, int any, float* t_out, int* prim_out,
                 int* work, int* err, int num_sms) {
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_query<0>, kTraceThreads, 0);
  if (bps < 1) bps = 1;
  const int f = S.precision;
  if (S.bitstack && f <= 1) {
    if (f == 1) k_query<5><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
    else k_query<4><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
  } else if (f == 3)
    k_query<3><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
  else if (f == 2)
    k_query<2><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
  else if (f == 1)
    k_query<1><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
  else
    k_query<0><<<num_sms * bps, kTraceThreads, 0, st>>>(S, rays, n, any, t_out, prim_out, work, err);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace mt
