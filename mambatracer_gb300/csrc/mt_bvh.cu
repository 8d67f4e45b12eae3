// The reference's BVH built on the GPU.
//
// CNormalBVH.build (src/cl/scene/CNormalBVH.java:45-148) splits a node's
// triangles at the centre of their centroid bound's longest axis (stable
// partition "centroid < split", the middle index when one side would be empty),
// one triangle per leaf, children allocated as adjacent pairs in the order the
// recursion subdivides. The host restatement (mt_bvh_build_host) runs it
// recursively; here it runs level by level over all nodes of a level at once:
//
//   reduce      bounds and centroid bounds of every node (exact min/max through
//               order-preserving integer atomics, one per warp where the warp's
//               triangles share a node)
//   decide      per node: its records, leaf or split axis and position
//   count       triangles left of the split per node
//   scan        a stable partition: exclusive scan of the left flags
//   scatter     triangles to their child's range (order kept on each side)
//   children    the next level's nodes
//
// A node subdivided when the allocation counter reads P gets children P and
// P + 1; its left subtree (k triangles) then allocates 2(k - 1) nodes, so its
// right child is subdivided at P + 2k and its left child at P + 2: every
// node's index follows from its parent's counter and its left sibling's size.
// The result equals the host build element for element (the test compares the
// reference-layout arrays). The traversal layout is written in the same pass:
// interior records in depth-first preorder (an interior node with record R and
// a left child of k triangles has its left child at R + 1 and its right child
// at R + k, since the left subtree holds k - 1 interior nodes), leaf slots = the
// triangles' final positions (the depth-first leaf order), each record holding
// its two children's boxes.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mt_internal.h"

namespace mt {
namespace {

constexpr int kT = 256;

// order-preserving float <-> int keys for atomicMin/atomicMax
__device__ __forceinline__ int fkey(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float fval(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }

struct Seg {
  int node, start, end, P, depth, prec, side;  // prec: parent's record (-1 for the root), side 0 left 1 right
  int rec;                                     // its own record when interior (preorder rank)
};
struct Acc {
  int mn[3], mx[3], cmn[3], cmx[3];
  int nl;
  int pad[3];
};
struct Dec {
  int dim, mid, interior, pad;
  float split;
};

__global__ void k_prims(const float4* __restrict__ pts, const Face* __restrict__ faces, int n, float4* lo, float4* hi,
                        float4* cen, int* obj, int* seg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const Face f = faces[t];
  const float4 p[3] = {pts[f.vx], pts[f.vy], pts[f.vz]};
  float l[3], h[3], c[3];
  for (int a = 0; a < 3; ++a) {
    float vlo = CUDART_INF_F, vhi = -CUDART_INF_F;
    for (int k = 0; k < 3; ++k) {
      const float v = a == 0 ? p[k].x : a == 1 ? p[k].y : p[k].z;
      if (v < vlo) vlo = v;
      if (v > vhi) vhi = v;
    }
    l[a] = vlo;
    h[a] = vhi;
    c[a] = 0.5f * (vlo + vhi);
  }
  lo[t] = make_float4(l[0], l[1], l[2], 0.f);
  hi[t] = make_float4(h[0], h[1], h[2], 0.f);
  cen[t] = make_float4(c[0], c[1], c[2], 0.f);
  obj[t] = t;
  seg[t] = 0;
}

__global__ void k_acc_init(Acc* acc, int nseg) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  Acc a;
  for (int k = 0; k < 3; ++k) {
    a.mn[k] = a.cmn[k] = fkey(CUDART_INF_F);
    a.mx[k] = a.cmx[k] = fkey(-CUDART_INF_F);
  }
  a.nl = 0;
  a.pad[0] = a.pad[1] = a.pad[2] = 0;
  acc[s] = a;
}

// the lanes of `active` that share s reduce first when the whole warp shares it
__device__ __forceinline__ int wmin(int v, bool uniform) {
  if (uniform)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int wmax(int v, bool uniform) {
  if (uniform)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void k_reduce(int n, const int* __restrict__ seg, const int* __restrict__ obj, const float4* __restrict__ lo,
                         const float4* __restrict__ hi, const float4* __restrict__ cen, Acc* acc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = p < n ? seg[p] : -1;
  const int s0 = __shfl_sync(0xffffffffu, s, 0);
  const bool uniform = __all_sync(0xffffffffu, s == s0) && s0 >= 0;
  int v[12];
  if (s >= 0) {
    const int t = obj[p];
    const float4 l = lo[t], h = hi[t], c = cen[t];
    v[0] = fkey(l.x); v[1] = fkey(l.y); v[2] = fkey(l.z);
    v[3] = fkey(h.x); v[4] = fkey(h.y); v[5] = fkey(h.z);
    v[6] = fkey(c.x); v[7] = fkey(c.y); v[8] = fkey(c.z);
    v[9] = v[6]; v[10] = v[7]; v[11] = v[8];
  } else {
    for (int k = 0; k < 12; ++k) v[k] = (k < 3 || (k >= 6 && k < 9)) ? INT_MAX : INT_MIN;
  }
  if (uniform) {
    for (int k = 0; k < 3; ++k) {
      v[k] = wmin(v[k], true);
      v[3 + k] = wmax(v[3 + k], true);
      v[6 + k] = wmin(v[6 + k], true);
      v[9 + k] = wmax(v[9 + k], true);
    }
    if ((threadIdx.x & 31) != 0) return;
  } else if (s < 0) {
    return;
  }
  const int ss = uniform ? s0 : s;
  Acc* a = acc + ss;
  for (int k = 0; k < 3; ++k) {
    atomicMin(&a->mn[k], v[k]);
    atomicMax(&a->mx[k], v[3 + k]);
    atomicMin(&a->cmn[k], v[6 + k]);
    atomicMax(&a->cmx[k], v[9 + k]);
  }
}

// Per node: reference-layout records, leaf or split, its box into its parent's
// traversal record once its own record index is known (k_link).
__global__ void k_decide(int nseg, const Seg* __restrict__ segs, const Acc* __restrict__ acc, const int* __restrict__ obj,
                         Dec* dec, int* ref_nodes, float* ref_bounds, int* max_depth, long long nn, int* err) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const Seg g = segs[s];
  if (g.node < 0 || g.node >= nn || (g.end - g.start >= 2 && g.P + 1 >= nn)) {  // numbering out of range
    atomicExch(err, 1);
    dec[s] = Dec{};
    return;
  }
  const Acc a = acc[s];
  int* nd = ref_nodes + 7 * (size_t)g.node;
  float* bd = ref_bounds + 8 * (size_t)g.node;
  nd[0] = g.node;  // bound
  for (int k = 0; k < 3; ++k) {
    bd[k] = fval(a.mn[k]);
    bd[4 + k] = fval(a.mx[k]);
  }
  bd[3] = bd[7] = 0.f;
  atomicMax(max_depth, g.depth);
  Dec d{};
  if (g.end - g.start < 2) {
    nd[6] = obj[g.start];  // child
    nd[5] = 1;             // isLeaf
    d.interior = 0;
    dec[s] = d;
    return;
  }
  const int li = g.P, ri = g.P + 1;
  int* ln = ref_nodes + 7 * (size_t)li;
  int* rn = ref_nodes + 7 * (size_t)ri;
  for (int k = 0; k < 7; ++k) ln[k] = rn[k] = 0;
  ln[4] = g.node;  // parent
  rn[4] = g.node;
  ln[1] = ri;      // sibling
  rn[1] = li;
  nd[2] = li;      // left
  nd[3] = ri;      // right
  const float cmn[3] = {fval(a.cmn[0]), fval(a.cmn[1]), fval(a.cmn[2])};
  const float cmx[3] = {fval(a.cmx[0]), fval(a.cmx[1]), fval(a.cmx[2])};
  const float ex = cmx[0] - cmn[0], ey = cmx[1] - cmn[1], ez = cmx[2] - cmn[2];
  d.dim = (ex > ey && ex > ez) ? 0 : (ey > ez ? 1 : 2);
  d.split = 0.5f * (cmn[d.dim] + cmx[d.dim]);
  d.interior = 1;
  dec[s] = d;
}

__global__ void k_count(int n, const int* __restrict__ seg, const int* __restrict__ obj, const float4* __restrict__ cen,
                        const Dec* __restrict__ dec, Acc* acc, int* flag) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = p < n ? seg[p] : -1;
  int f = 0;
  if (s >= 0) {
    const Dec d = dec[s];
    if (d.interior) {
      const float4 c = cen[obj[p]];
      const float v = d.dim == 0 ? c.x : d.dim == 1 ? c.y : c.z;
      f = v < d.split ? 1 : 0;
    }
  }
  if (p < n) flag[p] = f;
  const int s0 = __shfl_sync(0xffffffffu, s, 0);
  const bool uniform = __all_sync(0xffffffffu, s == s0) && s0 >= 0;
  if (uniform) {
    const int c = __popc(__ballot_sync(0xffffffffu, f));
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&acc[s0].nl, c);
  } else if (f) {
    atomicAdd(&acc[s].nl, 1);
  }
}

// exclusive scan of ints: per-block scans, a scan of the block sums, add back
__global__ void k_scan_blocks(const int* __restrict__ in, int n, int* out, int* bsum) {
  __shared__ int sh[kT];
  const int p = blockIdx.x * kT + threadIdx.x;
  const int v = p < n ? in[p] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kT; o <<= 1) {
    const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (p < n) out[p] = sh[threadIdx.x] - v;
  if (threadIdx.x == kT - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}
__global__ void k_scan_sums(int* bsum, int nb, int* total) {  // one block of kT threads
  __shared__ int sh[kT];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nb; b0 += kT) {
    const int b = b0 + threadIdx.x;
    const int v = b < nb ? bsum[b] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kT; o <<= 1) {
      const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (b < nb) bsum[b] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == kT - 1) carry += sh[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}
__global__ void k_scan_add(int* out, int n, const int* __restrict__ bsum) {
  const int p = blockIdx.x * kT + threadIdx.x;
  if (p < n) out[p] += bsum[blockIdx.x];
}

// Per node: its split position, the link from its parent's traversal record
// (interior nodes numbered in level order), and its children in the next level.
__global__ void k_link(int nseg, const Seg* __restrict__ segs, const Acc* __restrict__ acc, Dec* dec,
                       const int* __restrict__ kint, float4* __restrict__ recs, int nrec_cap, Seg* next,
                       int next_cap, int* err) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const Seg g = segs[s];
  Dec d = dec[s];
  const int size = g.end - g.start;
  const int rec = g.rec;
  if ((d.interior && (rec < 0 || rec >= nrec_cap || 2 * kint[s] + 1 >= next_cap)) || g.prec >= nrec_cap) {
    atomicExch(err, 1);
    d.interior = 0;
    dec[s] = d;
    return;
  }
  if (d.interior) {
    const int nl = acc[s].nl;
    d.mid = (nl != 0 && nl != size) ? g.start + nl : g.start + size / 2;
    dec[s] = d;
    next[2 * kint[s]] = Seg{g.P, g.start, d.mid, g.P + 2, g.depth + 1, rec, 0, rec + 1};
    next[2 * kint[s] + 1] =
        Seg{g.P + 1, d.mid, g.end, g.P + 2 * (d.mid - g.start), g.depth + 1, rec, 1, rec + (d.mid - g.start)};
  }
  if (g.prec >= 0) {
    const Acc a = acc[s];
    const float x0 = fval(a.mn[0]), y0 = fval(a.mn[1]), z0 = fval(a.mn[2]);
    const float x1 = fval(a.mx[0]), y1 = fval(a.mx[1]), z1 = fval(a.mx[2]);
    const int ref = d.interior ? rec : ~g.start;  // a leaf's slot is its triangle's final position
    float4* R = recs + 4 * (size_t)g.prec;
    float* zr = reinterpret_cast<float*>(R + 2);
    int* refs = reinterpret_cast<int*>(R + 3);
    if (g.side == 0) {
      R[0] = make_float4(x0, x1, y0, y1);
      zr[0] = z0;
      zr[1] = z1;
      refs[0] = ref;
    } else {
      R[1] = make_float4(x0, x1, y0, y1);
      zr[2] = z0;
      zr[3] = z1;
      refs[1] = ref;
    }
  }
}

// Triangles to their child's range, each side in its old order; a range whose
// split leaves one side empty keeps its order (the middle index splits it).
__global__ void k_scatter(int n, const int* __restrict__ seg, const int* __restrict__ obj, const int* __restrict__ flag,
                          const int* __restrict__ scan, const Seg* __restrict__ segs, const Dec* __restrict__ dec,
                          const Acc* __restrict__ acc, const int* __restrict__ kint, int* obj2, int* seg2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int s = seg[p];
  if (s < 0 || !dec[s].interior) {  // done, or a leaf: the triangle stays at its slot
    obj2[p] = obj[p];
    seg2[p] = -1;
    return;
  }
  const Seg g = segs[s];
  const int mid = dec[s].mid;
  const int nl = acc[s].nl, size = g.end - g.start;
  int q = p;
  if (nl != 0 && nl != size) {
    const int lrank = scan[p] - scan[g.start];
    q = flag[p] ? g.start + lrank : mid + ((p - g.start) - lrank);
  }
  obj2[q] = obj[p];
  seg2[q] = 2 * kint[s] + (q < mid ? 0 : 1);
}

__global__ void k_interior(int nseg, const Dec* __restrict__ dec, int* iflag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nseg) iflag[s] = dec[s].interior;
}

__global__ void k_tris(int n, const int* __restrict__ obj, const float4* __restrict__ pts,
                       const Face* __restrict__ faces, float4* tris) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int f = obj[k];
  const Face F = faces[f];
  const float4 p1 = pts[F.vx], p2 = pts[F.vy], p3 = pts[F.vz];
  tris[3 * (size_t)k + 0] = make_float4(p1.x, p1.y, p1.z, __int_as_float(f));
  tris[3 * (size_t)k + 1] = make_float4(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z, 0.f);
  tris[3 * (size_t)k + 2] = make_float4(p3.x - p1.x, p3.y - p1.y, p3.z - p1.z, 0.f);
}

// FP16 records from FP32 ones: lower planes rounded down, upper planes up.
__global__ void k_quantize_fp16(const float4* __restrict__ recs, int nrec, uint4* q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const float4* p = recs + 4 * (size_t)i;
  const float4 n0 = p[0], n1 = p[1], n2 = p[2], n3 = p[3];
  auto pair = [](float lo, float hi) {
    __half2 h = __halves2half2(__float2half_rd(lo), __float2half_ru(hi));
    return *reinterpret_cast<unsigned*>(&h);
  };
  q[2 * (size_t)i + 0] = make_uint4(pair(n0.x, n0.y), pair(n0.z, n0.w), pair(n1.x, n1.y), pair(n1.z, n1.w));
  q[2 * (size_t)i + 1] = make_uint4(pair(n2.x, n2.y), pair(n2.z, n2.w), __float_as_uint(n3.x), __float_as_uint(n3.y));
}

// 4-wide FP16 nodes from FP32 records: node r holds, for each child of record r,
// that child's two children when it is interior, else the child (a leaf), with
// the same outward rounding as the FP16 records.
__global__ void k_quad_fp16(const float4* __restrict__ recs, int nrec, uint4* q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  auto pair = [](float lo, float hi) {
    __half2 h = __halves2half2(__float2half_rd(lo), __float2half_ru(hi));
    return *reinterpret_cast<unsigned*>(&h);
  };
  // a record's children: boxes (lo/hi per axis) and refs
  auto kids = [&](int r, float box[2][6], int ref[2]) {
    const float4* p = recs + 4 * (size_t)r;
    const float4 n0 = p[0], n1 = p[1], n2 = p[2], n3 = p[3];
    const float b[2][6] = {{n0.x, n0.y, n0.z, n0.w, n2.x, n2.y}, {n1.x, n1.y, n1.z, n1.w, n2.z, n2.w}};
    for (int c = 0; c < 2; ++c)
      for (int k = 0; k < 6; ++k) box[c][k] = b[c][k];
    ref[0] = __float_as_int(n3.x);
    ref[1] = __float_as_int(n3.y);
  };
  float box[2][6];
  int ref[2];
  kids(i, box, ref);
  unsigned w[16];
  int n = 0;
  const unsigned empty_box = pair(INFINITY, -INFINITY);
  for (int c = 0; c < 2; ++c) {
    if (ref[c] >= 0) {
      float gb[2][6];
      int gr[2];
      kids(ref[c], gb, gr);
      for (int g = 0; g < 2; ++g, ++n) {
        for (int a = 0; a < 3; ++a) w[3 * n + a] = pair(gb[g][2 * a], gb[g][2 * a + 1]);
        w[12 + n] = (unsigned)gr[g];
      }
    } else {
      for (int a = 0; a < 3; ++a) w[3 * n + a] = pair(box[c][2 * a], box[c][2 * a + 1]);
      w[12 + n] = (unsigned)ref[c];
      ++n;
    }
  }
  for (; n < 4; ++n) {
    for (int a = 0; a < 3; ++a) w[3 * n + a] = empty_box;
    w[12 + n] = (unsigned)kQuadEmpty;
  }
  uint4* o = q + 4 * (size_t)i;
  o[0] = make_uint4(w[0], w[1], w[2], w[3]);
  o[1] = make_uint4(w[4], w[5], w[6], w[7]);
  o[2] = make_uint4(w[8], w[9], w[10], w[11]);
  o[3] = make_uint4(w[12], w[13], w[14], w[15]);
}

// Parent links: up[c] = (r, the other child of r) for each record child c of record r.
__global__ void k_up_links(const float4* __restrict__ recs, int nrec, int root, int2* up) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const float4 n3 = recs[4 * (size_t)i + 3];
  const int l = __float_as_int(n3.x), r = __float_as_int(n3.y);
  if (l >= 0) up[l] = make_int2(i, r);
  if (r >= 0) up[r] = make_int2(i, l);
  if (i == root) up[i] = make_int2(-1, -1);
}

__global__ void k_seed(Seg* segs, int n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) segs[0] = Seg{0, 0, n, 1, 0, -1, 0, 0};
}

inline unsigned blocks(size_t n) { return (unsigned)((n + kT - 1) / kT); }

// exclusive scan of n ints into out (bsum: blocks(n) ints of scratch), total into *total
void scan_ints(cudaStream_t st, const int* in, int n, int* out, int* bsum, int* total) {
  k_scan_blocks<<<blocks(n), kT, 0, st>>>(in, n, out, bsum);
  k_scan_sums<<<1, kT, 0, st>>>(bsum, (int)blocks(n), total);
  k_scan_add<<<blocks(n), kT, 0, st>>>(out, n, bsum);
}

}  // namespace
}  // namespace mt

using namespace mt;

extern "C" int mt_bvh_build_device(mt_scene* s, int32_t* nodes_out, float* bounds_out, int* depth_out) {
  if (!s) return fail(MT_ERR_INVALID, "NULL scene");
  const int n = s->ntri;
  if (n < 1) return fail(MT_ERR_INVALID, "empty scene");
  mt_context* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  CU(cudaSetDevice(ctx->device));
  int q = quiesce(ctx);
  if (q) return q;
  cudaStream_t st = ctx->stream;
  const size_t nn = 2 * (size_t)n - 1;
  const int nrec = n > 1 ? n - 1 : 0;
  float4 *lo = nullptr, *hi = nullptr, *cen = nullptr, *recs = nullptr, *tris = nullptr;
  int *obj = nullptr, *obj2 = nullptr, *seg = nullptr, *seg2 = nullptr, *flag = nullptr, *scan = nullptr;
  int *bsum = nullptr, *iflag = nullptr, *kint = nullptr, *words = nullptr, *ref_nodes = nullptr;
  float* ref_bounds = nullptr;
  Seg *segs = nullptr, *next = nullptr;
  Acc* acc = nullptr;
  Dec* dec = nullptr;
  int r = dalloc(&lo, n);
  if (!r) r = dalloc(&hi, n);
  if (!r) r = dalloc(&cen, n);
  if (!r) r = dalloc(&obj, n);
  if (!r) r = dalloc(&obj2, n);
  if (!r) r = dalloc(&seg, n);
  if (!r) r = dalloc(&seg2, n);
  if (!r) r = dalloc(&flag, n);
  if (!r) r = dalloc(&scan, n);
  if (!r) r = dalloc(&bsum, blocks(n) + 1);
  if (!r) r = dalloc(&iflag, n);
  if (!r) r = dalloc(&kint, n);
  if (!r) r = dalloc(&words, 4);
  if (!r) r = dalloc(&segs, n);
  if (!r) r = dalloc(&next, n);
  if (!r) r = dalloc(&acc, n);
  if (!r) r = dalloc(&dec, n);
  if (!r) r = dalloc(&ref_nodes, 7 * nn);
  if (!r) r = dalloc(&ref_bounds, 8 * nn);
  if (!r) r = dalloc(&recs, 4 * (size_t)std::max(nrec, 1));
  if (!r) r = dalloc(&tris, 3 * (size_t)n);
  auto scratch_free = [&] {
    dfree(lo); dfree(hi); dfree(cen); dfree(obj); dfree(obj2); dfree(seg); dfree(seg2); dfree(flag); dfree(scan);
    dfree(bsum); dfree(iflag); dfree(kint); dfree(words); dfree(segs); dfree(next); dfree(acc); dfree(dec);
    dfree(ref_nodes); dfree(ref_bounds);
  };
  auto fail_all = [&](int code, const char* msg) {
    std::string keep = msg ? std::string(msg) : mt_last_error();
    cudaStreamSynchronize(st);
    scratch_free();
    dfree(recs);
    dfree(tris);
    return fail(code, "%s", keep.c_str());
  };
  if (r) return fail_all(r, nullptr);
  if (cudaMemsetAsync(ref_nodes, 0, 7 * nn * 4, st) != cudaSuccess ||
      cudaMemsetAsync(recs, 0, 4 * (size_t)std::max(nrec, 1) * 16, st) != cudaSuccess ||
      cudaMemsetAsync(words, 0, 16, st) != cudaSuccess)
    return fail_all(MT_ERR_CUDA, "memset");
  // words: [0] deepest level, [1] interior nodes of the level, [2] scan total
  k_prims<<<blocks(n), kT, 0, st>>>(s->d_points, s->d_faces, n, lo, hi, cen, obj, seg);
  k_seed<<<1, 1, 0, st>>>(segs, n);
  int nseg = 1, rec_base = 0;
  for (int level = 0; nseg > 0; ++level) {
    if (level > kStackDepth) return fail_all(MT_ERR_DEPTH, "BVH deeper than the 64-level traversal stack");
    k_acc_init<<<blocks(nseg), kT, 0, st>>>(acc, nseg);
    k_reduce<<<blocks(n), kT, 0, st>>>(n, seg, obj, lo, hi, cen, acc);
    k_decide<<<blocks(nseg), kT, 0, st>>>(nseg, segs, acc, obj, dec, ref_nodes, ref_bounds, words, (long long)nn,
                                          words + 3);
    k_interior<<<blocks(nseg), kT, 0, st>>>(nseg, dec, iflag);
    scan_ints(st, iflag, nseg, kint, bsum, words + 1);
    k_count<<<blocks(n), kT, 0, st>>>(n, seg, obj, cen, dec, acc, flag);
    scan_ints(st, flag, n, scan, bsum, words + 2);
    k_link<<<blocks(nseg), kT, 0, st>>>(nseg, segs, acc, dec, kint, recs, std::max(nrec, 1), next, n,
                                        words + 3);
    k_scatter<<<blocks(n), kT, 0, st>>>(n, seg, obj, flag, scan, segs, dec, acc, kint, obj2, seg2);
    int interior = 0;
    if (cudaMemcpyAsync(&interior, words + 1, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return fail_all(MT_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    std::swap(obj, obj2);
    std::swap(seg, seg2);
    std::swap(segs, next);
    rec_base += interior;
    nseg = 2 * interior;
  }
  k_tris<<<blocks(n), kT, 0, st>>>(n, obj, s->d_points, s->d_faces, tris);
  int w4[4] = {0, 0, 0, 0};
  if (cudaMemcpyAsync(w4, words, 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      (nodes_out && cudaMemcpyAsync(nodes_out, ref_nodes, 7 * nn * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
      (bounds_out && cudaMemcpyAsync(bounds_out, ref_bounds, 8 * nn * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail_all(MT_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  if (w4[3]) return fail_all(MT_ERR_INVALID, "BVH build: a node index left its range");
  const int depth = w4[0];
  scratch_free();
  if (rec_base != nrec) {
    dfree(recs);
    dfree(tris);
    return fail(MT_ERR_INVALID, "BVH build produced %d interior nodes for %d triangles", rec_base, n);
  }
  if (depth > kStackDepth) {
    dfree(recs);
    dfree(tris);
    return fail(MT_ERR_DEPTH, "BVH depth %d exceeds %d", depth, kStackDepth);
  }
  dfree(s->d_nodes);
  dfree(s->d_tris);
  s->d_nodes = recs;
  s->d_tris = tris;
  s->nrec = nrec;
  s->root_ref = n > 1 ? 0 : ~0;
  s->depth = depth;
  s->has_bvh = 1;
  ++s->version;
  if (depth_out) *depth_out = depth;
  return refresh_qnodes(s);
}

bool traversal_bitstack() {
  static const bool on = [] {
    const char* e = std::getenv("MT_TRAVERSAL");
    return e && std::strcmp(e, "bitstack") == 0;
  }();
  return on;
}

int refresh_qnodes(mt_scene* s) {
  dfree(s->d_qnodes);
  dfree(s->d_quad);
  dfree(s->d_up);
  if (traversal_bitstack() && s->has_bvh && s->nrec > 0) {
    int r = dalloc(&s->d_up, (size_t)s->nrec);
    if (r) return r;
    cudaStream_t st = s->ctx->stream;
    k_up_links<<<blocks(s->nrec), kT, 0, st>>>(s->d_nodes, s->nrec, s->root_ref, s->d_up);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
      dfree(s->d_up);
      return fail(MT_ERR_CUDA, "parent links: %s", cudaGetErrorString(cudaGetLastError()));
    }
  }
  if (int w = refresh_wide(s)) return w;
  if (s->precision == 3 && s->has_bvh && s->nrec > 0) {
    int r = dalloc(&s->d_quad, 4 * (size_t)s->nrec);
    if (r) return r;
    cudaStream_t st = s->ctx->stream;
    k_quad_fp16<<<blocks(s->nrec), kT, 0, st>>>(s->d_nodes, s->nrec, s->d_quad);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
      dfree(s->d_quad);
      return fail(MT_ERR_CUDA, "4-wide FP16 nodes: %s", cudaGetErrorString(cudaGetLastError()));
    }
    return MT_OK;
  }
  if (s->precision != 1 || !s->has_bvh || s->nrec == 0) return MT_OK;
  int r = dalloc(&s->d_qnodes, 2 * (size_t)s->nrec);
  if (r) return r;
  cudaStream_t st = s->ctx->stream;
  k_quantize_fp16<<<blocks(s->nrec), kT, 0, st>>>(s->d_nodes, s->nrec, s->d_qnodes);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    dfree(s->d_qnodes);
    return fail(MT_ERR_CUDA, "FP16 records: %s", cudaGetErrorString(cudaGetLastError()));
  }
  return MT_OK;
}
