// The wide BVH of precision 2: the binary tree of the traversal records
// collapsed into nodes of up to eight children with 8-bit child boxes
// (layout: DevScene::wnodes in mt_common.h; traversal: tr::wide_steps).
//
// Built on the host from the device's FP32 records, after every BVH build or
// import (the binary tree is CNormalBVH.build's, src/cl/scene/CNormalBVH.java:45-148;
// its single-triangle leaves stay single-triangle leaves here):
//   * collapse: a node starts with its binary node's two children and, while it
//     has fewer than eight, replaces the interior child of largest surface area
//     by that child's two children;
//   * slots: child i goes to the slot s whose octant direction (x, y, z = -1 where
//     bit 2, 1, 0 of s is set, else +1) best matches the offset of its box centre
//     from the node's, pairs taken greedily by that score, so that taking slots in
//     descending order of s ^ (the ray's octant) visits near children first;
//   * quantisation: per axis, scale = the smallest power of two with extent /
//     scale <= 250 (and no finer than the coordinates' ulp), origin = one step
//     below the node box's lower plane; a child's lower plane is rounded down
//     and its upper plane up to that grid, plus one step each way, so the
//     quantised box contains the FP32 box by a step, which the traversal's plane
//     arithmetic (within half a step) cannot lose (checked in double, where every
//     such plane is exact);
//   * order: the interior children of a node are consecutive nodes (depth-first,
//     a node's children block before its grandchildren); a node's leaf triangles
//     are consecutive entries of the wide triangle array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mt_internal.h"

namespace {

struct WChild {
  float lo[3], hi[3];
  int ref;  // >= 0: binary record, < 0: ~triangle slot
};

struct WideBuilder {
  const float4* rec = nullptr;
  const float4* tris = nullptr;
  std::vector<uint4> nodes;  // kWideWords per node
  std::vector<float4> wt;    // 3 per triangle entry
  int max_depth = 0;
  bool bad = false;

  static bool expandable(const WChild& c) { return c.ref >= 0; }

  void children_of(int r, WChild c[2]) const {
    const float4* p = rec + 4 * (size_t)r;
    c[0] = WChild{{p[0].x, p[0].z, p[2].x}, {p[0].y, p[0].w, p[2].y}, 0};
    c[1] = WChild{{p[1].x, p[1].z, p[2].z}, {p[1].y, p[1].w, p[2].w}, 0};
    int lr, rr;
    std::memcpy(&lr, &p[3].x, 4);
    std::memcpy(&rr, &p[3].y, 4);
    c[0].ref = lr;
    c[1].ref = rr;
  }
  static double area(const WChild& c) {
    const double dx = (double)c.hi[0] - c.lo[0], dy = (double)c.hi[1] - c.lo[1], dz = (double)c.hi[2] - c.lo[2];
    return dx * dy + dy * dz + dz * dx;
  }

  // Writes node w from its child list (n <= 2 on entry); recurses into the
  // interior children it keeps.
  void fill(unsigned w, WChild* ch, int n, int depth) {
    max_depth = std::max(max_depth, depth);
    while (n < 8) {
      int best = -1;
      double ba = -1.0;
      for (int i = 0; i < n; ++i)
        if (expandable(ch[i]) && area(ch[i]) > ba) {
          ba = area(ch[i]);
          best = i;
        }
      if (best < 0) break;
      WChild two[2];
      children_of(ch[best].ref, two);
      ch[best] = two[0];
      ch[n++] = two[1];
    }
    // node box and child centres
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = ch[0].lo[a];
      hi[a] = ch[0].hi[a];
      for (int i = 1; i < n; ++i) {
        lo[a] = std::min(lo[a], ch[i].lo[a]);
        hi[a] = std::max(hi[a], ch[i].hi[a]);
      }
    }
    // slots: greedy by octant score
    int slot_of[8], child_in[8];
    for (int i = 0; i < 8; ++i) slot_of[i] = child_in[i] = -1;
    struct Pair {
      double score;
      int i, s;
    };
    Pair pairs[64];
    int np = 0;
    for (int i = 0; i < n; ++i) {
      double off[3];
      for (int a = 0; a < 3; ++a)
        off[a] = 0.5 * ((double)ch[i].lo[a] + ch[i].hi[a]) - 0.5 * ((double)lo[a] + hi[a]);
      for (int s = 0; s < 8; ++s) {
        const double sc = ((s & 4) ? -off[0] : off[0]) + ((s & 2) ? -off[1] : off[1]) + ((s & 1) ? -off[2] : off[2]);
        pairs[np++] = Pair{sc, i, s};
      }
    }
    std::stable_sort(pairs, pairs + np, [](const Pair& a, const Pair& b) { return a.score > b.score; });
    for (int k = 0; k < np; ++k) {
      const Pair& p = pairs[k];
      if (slot_of[p.i] < 0 && child_in[p.s] < 0) {
        slot_of[p.i] = p.s;
        child_in[p.s] = p.i;
      }
    }
    // quantisation grid per axis: scale 2^e with extent <= 250 steps (and at least
    // an ulp of the node's coordinates), origin one step below the lower plane
    // (rounded down to a float), so every child gets a step of margin on each side
    int ebyte[3];
    double scale[3];
    float org[3];
    for (int a = 0; a < 3; ++a) {
      const double ext = (double)hi[a] - lo[a];
      const double mag = std::max(std::fabs((double)lo[a]), std::fabs((double)hi[a]));
      int e = -126;
      if (ext > 0) e = (int)std::ceil(std::log2(ext / 250.0));
      while (std::ldexp(250.0, e) < ext) ++e;
      if (mag > 0) e = std::max(e, std::ilogb(mag) - 23);
      e = std::max(e, -126);
      if (e > 127) {
        bad = true;
        e = 127;
      }
      ebyte[a] = e + 127;
      scale[a] = std::ldexp(1.0, e);
      const double o = (double)lo[a] - scale[a];
      float of = (float)o;
      if ((double)of > o) of = std::nextafter(of, -INFINITY);
      org[a] = of;
    }
    unsigned char qlo[3][8], qhi[3][8];
    for (int a = 0; a < 3; ++a)
      for (int s = 0; s < 8; ++s) {
        qlo[a][s] = 255;  // an empty slot: an inverted box, never hit
        qhi[a][s] = 0;
      }
    unsigned imask = 0, lmask = 0;
    int ninner = 0;
    for (int s = 0; s < 8; ++s) {
      const int i = child_in[s];
      if (i < 0) continue;
      for (int a = 0; a < 3; ++a) {
        // one step of margin beyond the FP32 planes (the traversal's plane
        // distances are within half a step of the quantised ones)
        const double ql = std::floor(((double)ch[i].lo[a] - org[a]) / scale[a]) - 1.0;
        const double qh = std::ceil(((double)ch[i].hi[a] - org[a]) / scale[a]) + 1.0;
        if (ql < 0 || qh > 255 || (double)org[a] + (ql + 1) * scale[a] > (double)ch[i].lo[a] ||
            (double)org[a] + (qh - 1) * scale[a] < (double)ch[i].hi[a])
          bad = true;
        qlo[a][s] = (unsigned char)std::max(0.0, std::min(255.0, ql));
        qhi[a][s] = (unsigned char)std::max(0.0, std::min(255.0, qh));
      }
      if (expandable(ch[i])) {
        imask |= 1u << s;
        ++ninner;
      } else {
        lmask |= 1u << s;
      }
    }
    const unsigned child_base = (unsigned)(nodes.size() / kWideWords);
    nodes.resize(nodes.size() + kWideWords * (size_t)ninner, make_uint4(0u, 0u, 0u, 0u));
    const unsigned tri_base = (unsigned)(wt.size() / 3);
    for (int s = 0; s < 8; ++s) {  // leaf slot s holds triangle tri_base + (leaf slots below s)
      const int i = child_in[s];
      if (i < 0 || expandable(ch[i])) continue;
      const float4* t = tris + 3 * (size_t)(~ch[i].ref);
      wt.push_back(t[0]);
      wt.push_back(t[1]);
      wt.push_back(t[2]);
    }
    auto word = [](const unsigned char* b) {
      return (unsigned)b[0] | ((unsigned)b[1] << 8) | ((unsigned)b[2] << 16) | ((unsigned)b[3] << 24);
    };
    uint4* o = nodes.data() + kWideWords * (size_t)w;
    unsigned px, py, pz;
    std::memcpy(&px, &org[0], 4);
    std::memcpy(&py, &org[1], 4);
    std::memcpy(&pz, &org[2], 4);
    o[0] = make_uint4(px, py, pz, (unsigned)ebyte[0] | ((unsigned)ebyte[1] << 8) | ((unsigned)ebyte[2] << 16) |
                                      (imask << 24));
    o[1] = make_uint4(child_base, tri_base, lmask, 0u);
    o[2] = make_uint4(word(qlo[0]), word(qlo[0] + 4), word(qlo[1]), word(qlo[1] + 4));
    o[3] = make_uint4(word(qlo[2]), word(qlo[2] + 4), word(qhi[0]), word(qhi[0] + 4));
    o[4] = make_uint4(word(qhi[1]), word(qhi[1] + 4), word(qhi[2]), word(qhi[2] + 4));
    // recurse: interior children in slot order are nodes child_base, child_base + 1, ...
    unsigned k = 0;
    for (int s = 0; s < 8; ++s) {
      const int i = child_in[s];
      if (i < 0 || !expandable(ch[i])) continue;
      WChild gc[8];
      children_of(ch[i].ref, gc);
      fill(child_base + k++, gc, 2, depth + 1);
    }
  }
};

}  // namespace

// Builds (precision 2) or drops the scene's wide BVH from its FP32 records.
int refresh_wide(mt_scene* s) {
  dfree(s->d_wnodes);
  dfree(s->d_wtris);
  s->nwide = 0;
  s->wdepth = 0;
  if (s->precision != 2 || !s->has_bvh) return MT_OK;
  cudaStream_t st = s->ctx->stream;
  std::vector<float4> rec(4 * (size_t)std::max(s->nrec, 1)), tris(3 * (size_t)s->ntri);
  CU(cudaStreamSynchronize(st));
  if (s->nrec) CU(cudaMemcpy(rec.data(), s->d_nodes, 64 * (size_t)s->nrec, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(tris.data(), s->d_tris, 48 * (size_t)s->ntri, cudaMemcpyDeviceToHost));
  WideBuilder b;
  b.rec = rec.data();
  b.tris = tris.data();

  b.nodes.reserve(kWideWords * (size_t)(s->ntri / 3 + 8));
  b.wt.reserve(3 * (size_t)s->ntri);
  b.nodes.resize(kWideWords, make_uint4(0u, 0u, 0u, 0u));
  if (s->root_ref >= 0) {
    WChild c[8];
    b.children_of(s->root_ref, c);
    b.fill(0, c, 2, 0);
  } else {  // one triangle: a root with one leaf
    const float4 p1 = tris[0], e1 = tris[1], e2 = tris[2];
    WChild c[8];
    const float xs[3] = {p1.x, p1.x + e1.x, p1.x + e2.x}, ys[3] = {p1.y, p1.y + e1.y, p1.y + e2.y},
                zs[3] = {p1.z, p1.z + e1.z, p1.z + e2.z};
    const float* v[3] = {xs, ys, zs};
    for (int a = 0; a < 3; ++a) {
      // the edge sums round: widen by a few ulps so the box holds the triangle
      float l = std::min(v[a][0], std::min(v[a][1], v[a][2])), h = std::max(v[a][0], std::max(v[a][1], v[a][2]));
      const float pad = 4.f * std::max(std::fabs(l), std::fabs(h)) * 1.1920929e-7f + 1e-30f;
      c[0].lo[a] = l - pad;
      c[0].hi[a] = h + pad;
    }
    c[0].ref = ~0;
    b.fill(0, c, 1, 0);
  }
  if (b.bad) return fail(MT_ERR_INVALID, "wide BVH: a node's extent does not fit its 8-bit grid");
  if (b.max_depth + 1 > kWideStack)
    return fail(MT_ERR_DEPTH, "wide BVH depth %d exceeds the traversal's %d groups", b.max_depth + 1, kWideStack);
  if ((int)(b.wt.size() / 3) != s->ntri)
    return fail(MT_ERR_INVALID, "wide BVH reaches %zu of %d triangles", b.wt.size() / 3, s->ntri);
  int r = dalloc(&s->d_wnodes, b.nodes.size());
  if (!r) r = dalloc(&s->d_wtris, b.wt.size());
  if (r) return r;
  CU(cudaMemcpy(s->d_wnodes, b.nodes.data(), b.nodes.size() * sizeof(uint4), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(s->d_wtris, b.wt.data(), b.wt.size() * sizeof(float4), cudaMemcpyHostToDevice));
  s->nwide = (int)(b.nodes.size() / kWideWords);
  s->wdepth = b.max_depth + 1;
  return MT_OK;
}
