// BVH traversal on the GPU layout (see DevScene in mt_common.h).
//
// Visit order is the reference's stackless traversal (src/cl/kernel/NormalBVH.cl:14-92):
// at an interior node both child boxes are slab-tested (Util.cl:707-732); when
// both are hit the nearer (right only if strictly nearer) is entered and the
// other is deferred; leaves are single triangles tested with Moller-Trumbore
// (Primitive.cl:3-29) and accepted when tMin < t < tMax (Util.cl:552-555).
// The reference backtracks with a 64-bit bitstack and parent/sibling links; a
// per-thread stack of deferred children (local memory) visits the same nodes in
// the same order without re-reading parents. Identical order and identical
// arithmetic give identical hit ids, including ties.
//
// Binary record formats (DevScene::precision): 0 = FP32 child boxes, 64 bytes per
// record; 1 = FP16 child boxes rounded outward (lower bounds down, upper bounds
// up), 32 bytes per record: the half-size record halves the bytes a visit
// moves through L1/L2. An outward-rounded box contains the FP32 box, and the
// slab arithmetic is monotonic in the planes, so every node the FP32 traversal
// enters is entered too and the closest hit is the same triangle at the same
// distance; only a different visit order can pick another of two triangles hit
// at exactly the same distance.
#pragma once
#include <cuda_fp16.h>

#include "mt_device.cuh"

namespace mt {
namespace tr {

struct RayT {
  float ox, oy, oz;
  float ix, iy, iz;  // 1/d (IEEE division, as initGlobalRay stores inv_d)
  float dx, dy, dz;
  int sx, sy, sz;    // inv_d < 0
  float tmin, tmax;
};

__device__ __forceinline__ RayT make_ray(float4 o, float4 d, float tmin, float tmax) {
  RayT r;
  r.ox = o.x; r.oy = o.y; r.oz = o.z;
  r.dx = d.x; r.dy = d.y; r.dz = d.z;
  r.ix = 1.f / d.x; r.iy = 1.f / d.y; r.iz = 1.f / d.z;
  r.sx = r.ix < 0.f; r.sy = r.iy < 0.f; r.sz = r.iz < 0.f;
  r.tmin = tmin;
  r.tmax = tmax;
  return r;
}

// Util.cl:707-732. lo/hi: the box along each axis; the near plane is picked by
// the direction sign as getExtent(sign) does.
__device__ __forceinline__ bool slab(const RayT& r, float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     float* tnear) {
  float tmin = ((r.sx ? hix : lox) - r.ox) * r.ix;
  float tmax = ((r.sx ? lox : hix) - r.ox) * r.ix;
  float tymin = ((r.sy ? hiy : loy) - r.oy) * r.iy;
  float tymax = ((r.sy ? loy : hiy) - r.oy) * r.iy;
  bool ok = !((tmin > tymax) || (tymin > tmax));
  tmin = (tymin > tmin) ? tymin : tmin;
  tmax = (tymax < tmax) ? tymax : tmax;
  float tzmin = ((r.sz ? hiz : loz) - r.oz) * r.iz;
  float tzmax = ((r.sz ? loz : hiz) - r.oz) * r.iz;
  ok = ok && !((tmin > tzmax) || (tzmin > tmax));
  tmin = (tzmin > tmin) ? tzmin : tmin;
  tmax = (tzmax < tmax) ? tzmax : tmax;
  tmax *= 1.00000024f;
  *tnear = tmin;
  return ok && (tmin < r.tmax) && (tmax > r.tmin);
}

// Primitive.cl:3-29: returns t, or tmax when the triangle is missed. The
// reference's float4 dot adds a w-lane product that is +0 for these operands,
// which changes at most the sign of a zero result and never the outcome.
__device__ __forceinline__ float tri_t(const RayT& r, float4 p1, float4 e1, float4 e2) {
  float hx = r.dy * e2.z - r.dz * e2.y;
  float hy = r.dz * e2.x - r.dx * e2.z;
  float hz = r.dx * e2.y - r.dy * e2.x;
  float a = (e1.x * hx + e1.y * hy) + e1.z * hz;
  if (a > -0.0000001f && a < 0.0000001f) return r.tmax;
  float f = 1.f / a;
  float sx = r.ox - p1.x, sy = r.oy - p1.y, sz = r.oz - p1.z;
  float b1 = f * ((sx * hx + sy * hy) + sz * hz);
  float qx = sy * e1.z - sz * e1.y;
  float qy = sz * e1.x - sx * e1.z;
  float qz = sx * e1.y - sy * e1.x;
  float b2 = f * ((r.dx * qx + r.dy * qy) + r.dz * qz);
  float t = f * ((e2.x * qx + e2.y * qy) + e2.z * qz);
  if (b1 < 0.f || b1 > 1.f || b2 < 0.f || b1 + b2 > 1.f || t < 0.f || t > r.tmax) return r.tmax;
  return t;
}

// Branch-free slab test for rays whose origin and 1/d are finite. With no
// NaN possible, the reference's comparison chain (Util.cl:707-732) reduces to
// max(near) <= min(far) on the three axes (near <= far holds per axis for a
// valid box), and fmaxf/fminf give the same values; the sign of a zero
// distance, which fmaxf may choose differently, never changes a comparison.
// n*/f*: the near and far planes already picked by the direction sign.
__device__ __forceinline__ bool slab_fast(const RayT& r, float nx, float fx, float ny, float fy, float nz, float fz,
                                          float* tnear) {
  float tmin = fmaxf(fmaxf((nx - r.ox) * r.ix, (ny - r.oy) * r.iy), (nz - r.oz) * r.iz);
  float tmax = fminf(fminf((fx - r.ox) * r.ix, (fy - r.oy) * r.iy), (fz - r.oz) * r.iz);
  *tnear = tmin;
  return (tmin <= tmax) && (tmin < r.tmax) && (tmax * 1.00000024f > r.tmin);
}

__device__ __forceinline__ bool ray_is_finite(const RayT& r) {
  return isfinite(r.ix) && isfinite(r.iy) && isfinite(r.iz) && isfinite(r.ox) && isfinite(r.oy) && isfinite(r.oz);
}

// Resumable traversal in the reference's visit order (see the file header).
// Deferred children sit on a per-thread stack of (ref, entry distance). For
// finite rays a deferred interior node whose entry distance is not below the
// current closest hit is dropped when popped: its children's boxes nest in its
// box and the slab arithmetic is monotonic, so both would miss and the
// reference would test no triangle under it. Deferred leaves are always tested.
// Runs at most `steps` node visits or triangle tests; returns true when the
// ray is finished (hit_face / r.tmax hold the result).
// Deferred-node stack entries: (node, entry distance) for closest hits; the
// node alone for any-hit rays, which never cull (their interval is fixed).
template <bool ANY>
struct StackEntry {
  using type = int2;
};
template <>
struct StackEntry<true> {
  using type = int;
};

// A record's two child boxes as n0 = (L.lo.x, L.hi.x, L.lo.y, L.hi.y),
// n1 = the same for R, n2 = (L.lo.z, L.hi.z, R.lo.z, R.hi.z), and its child refs.
// FP16 records: q0 = half2 pairs (L x, L y, R x, R y), q1 = (L z, R z, left, right).
// 32 bytes in one 256-bit read-only load (records are 32-byte aligned: the
// arrays start on 256-byte boundaries and records are 32 or 64 bytes).
__device__ __forceinline__ void ldg32(const void* p, uint4& a, uint4& b) {
  asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
      : "l"(p));
}

template <int PREC>
__device__ __forceinline__ void load_record(const DevScene& S, int ref, float4& n0, float4& n1, float4& n2, int& left,
                                            int& right) {
  if constexpr (PREC == 0) {
    const float4* p = S.nodes + 4 * (size_t)ref;
    uint4 a, b, c, d;
    ldg32(p, a, b);
    ldg32(p + 2, c, d);
    n0 = make_float4(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(a.w));
    n1 = make_float4(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z), __uint_as_float(b.w));
    n2 = make_float4(__uint_as_float(c.x), __uint_as_float(c.y), __uint_as_float(c.z), __uint_as_float(c.w));
    left = (int)d.x;
    right = (int)d.y;
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(S.qnodes) + 2 * (size_t)ref;
    uint4 q0, q1;
    ldg32(p, q0, q1);
    auto h2 = [](unsigned u) { return __half22float2(*reinterpret_cast<const __half2*>(&u)); };
    const float2 lx = h2(q0.x), ly = h2(q0.y), rx = h2(q0.z), ry = h2(q0.w), lz = h2(q1.x), rz = h2(q1.y);
    n0 = make_float4(lx.x, lx.y, ly.x, ly.y);
    n1 = make_float4(rx.x, rx.y, ry.x, ry.y);
    n2 = make_float4(lz.x, lz.y, rz.x, rz.y);
    left = (int)q1.z;
    right = (int)q1.w;
  }
}

// Any-hit rays keep the deferred stack's top entry in a register (top, valid
// while sp > 0) and the entries below it in local memory (stack[0 .. sp - 2]): a
// pop takes its node from the register and loads the next top for a later pop,
// so the load's latency is hidden behind the traversal of the popped subtree
// instead of delaying the next node's load (bounce-1 shadow rays 0.98 against
// 1.15 ms on the 1M soup). Closest-hit rays keep the whole stack in local
// memory: their kernel is bounded to 40 registers, and the register top made it
// spill (1.51 against 1.42 ms).
template <bool ANY, int PREC = 0>
__device__ __forceinline__ bool trav_steps(const DevScene& S, RayT& r, int& ref, int& sp, int& hit_face, bool finite,
                                           typename StackEntry<ANY>::type* stack,
                                           typename StackEntry<ANY>::type& top, int steps, bool* overflow) {
  const float4* __restrict__ tris = S.tris;
  for (int it = 0; it < steps; ++it) {
    if (ref >= 0) {
      float4 n0, n1, n2;
      int left, right;
      load_record<PREC>(S, ref, n0, n1, n2, left, right);
      float tl, trr;
      bool hl, hr;
      if (finite) {
        hl = slab_fast(r, r.sx ? n0.y : n0.x, r.sx ? n0.x : n0.y, r.sy ? n0.w : n0.z, r.sy ? n0.z : n0.w,
                       r.sz ? n2.y : n2.x, r.sz ? n2.x : n2.y, &tl);
        hr = slab_fast(r, r.sx ? n1.y : n1.x, r.sx ? n1.x : n1.y, r.sy ? n1.w : n1.z, r.sy ? n1.z : n1.w,
                       r.sz ? n2.w : n2.z, r.sz ? n2.z : n2.w, &trr);
      } else {
        hl = slab(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, &tl);
        hr = slab(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, &trr);
      }
      if (hl && hr) {
        const bool rfirst = trr < tl;
        if (sp >= kStackDepth) {
          *overflow = true;
          return true;
        }
        if constexpr (ANY) {
          if (sp > 0) stack[sp - 1] = top;
          top = rfirst ? left : right;
          ++sp;
        } else {
          stack[sp++] = make_int2(rfirst ? left : right, __float_as_int(rfirst ? tl : trr));
        }
        ref = rfirst ? right : left;
        continue;
      }
      if (hl) { ref = left; continue; }
      if (hr) { ref = right; continue; }
    } else {
      const float4* tp = tris + 3 * (size_t)(~ref);
      float4 p1 = __ldg(tp + 0), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
      float t = tri_t(r, p1, e1, e2);
      if ((r.tmin < t) && (t < r.tmax)) {
        hit_face = __float_as_int(p1.w);
        if (ANY) return true;
        r.tmax = t;
      }
    }
    if constexpr (ANY) {
      if (sp == 0) return true;
      ref = top;
      if (--sp > 0) top = stack[sp - 1];
    } else {
      for (;;) {
        if (sp == 0) return true;
        const int2 e = stack[--sp];
        if (!finite || e.x < 0 || __int_as_float(e.y) < r.tmax) {
          ref = e.x;
          break;
        }
      }
    }
  }
  return false;
}

// ------------------------------------------------------------ stackless (binary)
// The reference's own traversal (NormalBVH.cl:14-92): no deferred-node stack.
// Each descent pushes one bit on a 64-bit bitstack, 1 when both children were
// hit and the farther one remains; to backtrack, zero bits are popped while
// climbing to the parent (parent links: DevScene::up), and at the first 1 the
// traversal moves to the sibling and clears it. The visit order is the
// reference's and the one of trav_steps, without its culling of deferred nodes
// beyond the closest hit (the sibling's entry distance is not kept). par / sib:
// the current node's parent record and sibling ref, carried in registers from
// the descent, so a backtrack reads a link only per level it climbs.
template <bool ANY, int PREC>
__device__ __forceinline__ bool bitstack_steps(const DevScene& S, RayT& r, int& ref, unsigned long long& bits,
                                               int& par, int& sib, int& hit_face, bool finite, int steps) {
  const float4* __restrict__ tris = S.tris;
  for (int it = 0; it < steps; ++it) {
    if (ref >= 0) {
      float4 n0, n1, n2;
      int left, right;
      load_record<PREC>(S, ref, n0, n1, n2, left, right);
      float tl, trr;
      bool hl, hr;
      if (finite) {
        hl = slab_fast(r, r.sx ? n0.y : n0.x, r.sx ? n0.x : n0.y, r.sy ? n0.w : n0.z, r.sy ? n0.z : n0.w,
                       r.sz ? n2.y : n2.x, r.sz ? n2.x : n2.y, &tl);
        hr = slab_fast(r, r.sx ? n1.y : n1.x, r.sx ? n1.x : n1.y, r.sy ? n1.w : n1.z, r.sy ? n1.z : n1.w,
                       r.sz ? n2.w : n2.z, r.sz ? n2.z : n2.w, &trr);
      } else {
        hl = slab(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, &tl);
        hr = slab(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, &trr);
      }
      if (hl || hr) {
        const bool both = hl && hr;
        const bool rfirst = both ? trr < tl : hr;
        bits = (bits << 1) | (both ? 1ull : 0ull);
        par = ref;
        sib = rfirst ? left : right;
        ref = rfirst ? right : left;
        continue;
      }
    } else {
      const float4* tp = tris + 3 * (size_t)(~ref);
      const float4 p1 = __ldg(tp + 0), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
      const float t = tri_t(r, p1, e1, e2);
      if ((r.tmin < t) && (t < r.tmax)) {
        hit_face = __float_as_int(p1.w);
        if (ANY) return true;
        r.tmax = t;
      }
    }
    // backtrack: climb past the levels with nothing left, then take the sibling
    while ((bits & 1ull) == 0ull) {
      if (bits == 0ull) return true;
      const int2 u = __ldg(S.up + par);
      par = u.x;
      sib = u.y;
      bits >>= 1;
    }
    ref = sib;
    bits ^= 1ull;
  }
  return false;
}

// ------------------------------------------------------------------ 4-wide FP16
// Precision 3: the node of record r holds the children of r's two children
// (a leaf child stands for itself), so one 64-byte node read replaces the two
// dependent record reads of two binary levels. The boxes are the FP32 records'
// child boxes rounded outward to FP16 as in precision 1, tested with the same
// slab arithmetic, so the boxes entered contain those the binary traversal
// enters (a grandchild's box nests in its parent's) and every triangle it tests
// is tested here with the same FP32 Moller-Trumbore: the closest hit is the same
// triangle at the same distance, except among triangles hit at exactly or within
// a few ulps of the same distance (coplanar surfaces), where the order in which
// the boxes are met decides (a box test compares its entry distance with the
// closest hit so far, and a box plane that FP16 represents exactly keeps no
// slack against the triangle's own rounding); with leaves waiting for the warp
// that order can change from run to run. Children hit are taken nearest first;
// the others are deferred with their entry distance (closest hits cull deferred
// interior nodes as above).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float2 half2_bits(unsigned u) {
  return __half22float2(*reinterpret_cast<const __half2*>(&u));
}
__device__ __forceinline__ unsigned long long pack2(float a, float b) {
  unsigned long long v;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(a), "f"(b));
  return v;
}
// (p - o) * i on both lanes, each lane rounded as the scalar subtraction and
// multiplication are (add/mul .rn on f32x2: two IEEE operations per instruction)
__device__ __forceinline__ float2 sub_mul2(unsigned long long p, unsigned long long o, unsigned long long i) {
  unsigned long long t;
  float2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(p), "l"(o));
  asm("mul.rn.f32x2 %0, %0, %1;" : "+l"(t) : "l"(i));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(t));
  return r;
}

// Leaves wait in a one-entry slot (leaf) while the lane goes on with interior
// nodes; the warp tests the waiting leaves together when one of its lanes can
// go no further (its slot is taken and its next entry is a leaf too, or its
// stack is empty), so node visits run on converged lanes and triangle tests on
// many lanes at once instead of a few lanes interleaving the two (Aila, Laine,
// "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009, postponed
// leaves). A closest-hit ray's waiting triangle shortens its interval only when
// tested, so culling is then looser, never tighter.
// ref: the next entry (a node >= 0, a leaf < 0, kQuadEmpty: nothing left);
// leaf: the waiting leaf or kQuadEmpty. cnt (or NULL): [0] += node visits,
// [1] += triangle tests.
template <bool ANY>
__device__ __forceinline__ bool quad_steps(const DevScene& S, RayT& r, int& ref, int& leaf, int& sp, int& hit_face,
                                           bool finite, typename StackEntry<ANY>::type* stack,
                                           typename StackEntry<ANY>::type& top, int steps, bool* overflow,
                                           int* cnt = nullptr) {
  const float4* __restrict__ tris = S.tris;
  // (lo, hi) half pairs swapped to (near, far) by the direction's sign
  const unsigned selx = r.sx ? 0x1032u : 0x3210u, sely = r.sy ? 0x1032u : 0x3210u, selz = r.sz ? 0x1032u : 0x3210u;
  const unsigned long long oxy = pack2(r.ox, r.oy), ixy = pack2(r.ix, r.iy);
  // the next deferred entry, or kQuadEmpty
  auto pop = [&]() -> int {
    if constexpr (ANY) {
      if (sp == 0) return kQuadEmpty;
      const int e = top;
      if (--sp > 0) top = stack[sp - 1];
      return e;
    } else {
      for (;;) {
        if (sp == 0) return kQuadEmpty;
        const int2 e = stack[--sp];
        if (!finite || e.x < 0 || __int_as_float(e.y) < r.tmax) return e.x;
      }
    }
  };
  for (int it = 0; it < steps; ++it) {
    if (ref < 0 && ref != kQuadEmpty && leaf == kQuadEmpty) {
      leaf = ref;
      ref = pop();
    }
    if (ref == kQuadEmpty && leaf == kQuadEmpty) return true;
    if (__any_sync(__activemask(), ref < 0)) {
      // triangle tests: every lane with a waiting leaf
      if (leaf != kQuadEmpty) {
        if (cnt) ++cnt[1];
        const float4* tp = tris + 3 * (size_t)(~leaf);
        const float4 p1 = __ldg(tp + 0), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
        leaf = kQuadEmpty;
        const float t = tri_t(r, p1, e1, e2);
        if ((r.tmin < t) && (t < r.tmax)) {
          hit_face = __float_as_int(p1.w);
          if (ANY) return true;
          r.tmax = t;
        }
      }
      continue;
    }
    // node visit: ref >= 0 on every lane here
    if (cnt) ++cnt[0];
    const uint4* p = S.quad + 4 * (size_t)ref;
    uint4 a, b, c, d;
    ldg32(p, a, b);
    ldg32(p + 2, c, d);
    const unsigned wv[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
    const int cr[4] = {(int)d.x, (int)d.y, (int)d.z, (int)d.w};
    float key[4];
    int kid[4];
    int n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float tn;
      bool h;
      if (finite) {
        // slab_fast on (near, far) planes; an empty slot's (+inf, -inf) box
        // gives an entry distance of +inf and never passes
        const float2 x = half2_bits(__byte_perm(wv[3 * k], 0u, selx));
        const float2 y = half2_bits(__byte_perm(wv[3 * k + 1], 0u, sely));
        const float2 z = half2_bits(__byte_perm(wv[3 * k + 2], 0u, selz));
        const float2 nxy = sub_mul2(pack2(x.x, y.x), oxy, ixy), fxy = sub_mul2(pack2(x.y, y.y), oxy, ixy);
        tn = max3f(nxy.x, nxy.y, (z.x - r.oz) * r.iz);
        const float tf = min3f(fxy.x, fxy.y, (z.y - r.oz) * r.iz);
        h = (tn <= tf) && (tn < r.tmax) && (tf * 1.00000024f > r.tmin);
      } else {
        const float2 x = half2_bits(wv[3 * k]), y = half2_bits(wv[3 * k + 1]), z = half2_bits(wv[3 * k + 2]);
        h = slab(r, x.x, x.y, y.x, y.y, z.x, z.y, &tn) && cr[k] != kQuadEmpty;
        if (tn != tn) tn = -INFINITY;  // order only: a NaN entry distance sorts first
      }
      key[k] = h ? tn : INFINITY;
      kid[k] = cr[k];
      n += h;
    }
    if (n == 0) {
      ref = pop();
      continue;
    }
    // nearest first (children missed carry +inf and sort last)
    auto cx = [&](int i, int j) {
      const bool s = key[j] < key[i];
      const float ki = key[i], kj = key[j];
      const int ri = kid[i], rj = kid[j];
      key[i] = s ? kj : ki;
      key[j] = s ? ki : kj;
      kid[i] = s ? rj : ri;
      kid[j] = s ? ri : rj;
    };
    cx(0, 1);
    cx(2, 3);
    cx(0, 2);
    cx(1, 3);
    cx(1, 2);
    if (sp + n - 1 > kQuadStack) {
      *overflow = true;
      return true;
    }
#pragma unroll
    for (int k = 3; k >= 1; --k) {
      if (k < n) {
        if constexpr (ANY) {
          if (sp > 0) stack[sp - 1] = top;
          top = kid[k];
          ++sp;
        } else {
          stack[sp++] = make_int2(kid[k], __float_as_int(key[k]));
        }
      }
    }
    ref = kid[0];
  }
  return false;
}

// ------------------------------------------------------------------ wide BVH
// Precision 2: the same tree collapsed into nodes of up to eight children whose
// boxes are quantised to 8 bits per plane against the node's FP32 origin and a
// power-of-two scale per axis, rounded outward (Ylitie, Karras, Laine,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs",
// HPG 2017). A node is 80 bytes, padded to 96 (see DevScene::wnodes); leaves stay single
// triangles tested by the same FP32 Moller-Trumbore as above, so a hit is the
// same triangle at the same distance: a quantised box contains the child's
// FP32 box, so every triangle the binary traversal reaches is reached here.
// Only the visit order differs: of two triangles hit at exactly the same
// distance, the one tested first is kept.
//
// A child plane's distance is fma(2^23 + q, a, b') with a = 2^e / d and
// b' = (origin - o) / d - 2^23 a: the float 2^23 + q is the byte q dropped into
// the mantissa of 2^23 (one byte permute), and b' folds the 2^23 back in with
// one rounding, whose error is at most half a grid step (a / 2) plus the
// rounding of (origin - o) / d itself. The builder leaves one grid step of
// margin outside every FP32 box, so the tested box still contains it.
//
// Traversal state: the current node group (first child node, and a 32-bit
// mask: bits 24-31 = interior children still to visit, at bit 24 + (slot ^
// octant), bits 0-7 = the node's interior-slot mask) and triangle group (first
// triangle, bits 0-7 = hit leaf slots still to test, bits 8-15 = the node's
// leaf-slot mask). Interior children are taken in descending bit order, which
// for the ray's direction octant visits the child slots nearest the ray's
// origin first (the builder places a child in the slot of its centre's
// octant). Groups with children left are pushed.
struct WideState {
  uint2 ngroup, tgroup;
  unsigned oct;       // the ray's direction octant: bit 2 x < 0, bit 1 y < 0, bit 0 z < 0
  float jx, jy, jz;   // 1/d with infinities replaced by +-2^100 (box tests only)
};

__device__ __forceinline__ float finite_inv(float i) { return isinf(i) ? copysignf(0x1p100f, i) : i; }

__device__ __forceinline__ void wide_init(const RayT& r, WideState& w) {
  w.oct = (r.dx < 0.f ? 4u : 0u) | (r.dy < 0.f ? 2u : 0u) | (r.dz < 0.f ? 1u : 0u);
  w.jx = finite_inv(r.ix);
  w.jy = finite_inv(r.iy);
  w.jz = finite_inv(r.iz);
  // the root: node 0 as interior slot 0 of a virtual parent whose first child is node 0
  w.ngroup = make_uint2(0u, (1u << (24u + w.oct)) | 1u);
  w.tgroup = make_uint2(0u, 0u);
}

// 2^23 + (byte k of w), exactly: the byte placed in the mantissa of 2^23.
__device__ __forceinline__ float qbyte(unsigned w, int k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + k));
}
// The 8-bit slot mask m with slot s moved to slot s ^ x (x in 0..7).
__device__ __forceinline__ unsigned xor_permute8(unsigned m, unsigned x) {
  if (x & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
  if (x & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
  if (x & 4u) m = ((m & 0x0Fu) << 4) | (m >> 4);
  return m;
}

// Intersects the ray with a wide node's eight child boxes; sets the next node
// and triangle groups from the children hit.
__device__ __forceinline__ void wide_node(const DevScene& S, const RayT& r, WideState& w, unsigned node) {
  const uint4* p = S.wnodes + kWideWords * (size_t)node;
  uint4 w0, w1, w2, w3, w4, w5;
  ldg32(p, w0, w1);
  ldg32(p + 2, w2, w3);
  ldg32(p + 4, w4, w5);
  const unsigned imask = w0.w >> 24, lmask = w1.z & 0xFFu;
  const float ax = __uint_as_float((w0.w & 0xFFu) << 23) * w.jx;
  const float ay = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23) * w.jy;
  const float az = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23) * w.jz;
  const float bx = __fmaf_rn(-8388608.f, ax, (__uint_as_float(w0.x) - r.ox) * w.jx);
  const float by = __fmaf_rn(-8388608.f, ay, (__uint_as_float(w0.y) - r.oy) * w.jy);
  const float bz = __fmaf_rn(-8388608.f, az, (__uint_as_float(w0.z) - r.oz) * w.jz);
  unsigned hits = 0;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    // near / far plane words of this half, picked by the direction's signs
    const unsigned lox = half ? w2.y : w2.x, loy = half ? w2.w : w2.z, loz = half ? w3.y : w3.x;
    const unsigned hix = half ? w3.w : w3.z, hiy = half ? w4.y : w4.x, hiz = half ? w4.w : w4.z;
    const unsigned nx = r.sx ? hix : lox, fx = r.sx ? lox : hix;
    const unsigned ny = r.sy ? hiy : loy, fy = r.sy ? loy : hiy;
    const unsigned nz = r.sz ? hiz : loz, fz = r.sz ? loz : hiz;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float tn = max3f(__fmaf_rn(qbyte(nx, k), ax, bx), __fmaf_rn(qbyte(ny, k), ay, by),
                             __fmaf_rn(qbyte(nz, k), az, bz));
      const float tf = min3f(__fmaf_rn(qbyte(fx, k), ax, bx), __fmaf_rn(qbyte(fy, k), ay, by),
                             __fmaf_rn(qbyte(fz, k), az, bz));
      // the reference's slack on the far distance (Util.cl:707-732)
      if (fmaxf(tn, r.tmin) <= fminf(tf * 1.00000024f, r.tmax)) hits |= 1u << (4 * half + k);
    }
  }
  w.ngroup = make_uint2(w1.x, (xor_permute8(hits & imask, w.oct) << 24) | imask);
  w.tgroup = make_uint2(w1.y, (hits & lmask) | (lmask << 8));
}

// Runs at most `steps` traversal steps (a step tests one triangle and, when the
// current node has no triangle left to test, visits the next node); returns
// true when the ray is finished (hit_face / r.tmax hold the result).
// cnt (work counts, or NULL): [0] += node visits, [1] += triangle tests.
template <bool ANY>
__device__ __forceinline__ bool wide_steps(const DevScene& S, RayT& r, WideState& w, int& sp, int& hit_face,
                                           uint2* stack, int steps, bool* overflow, int* cnt = nullptr) {
  const float4* __restrict__ tris = S.wtris;
  for (int it = 0; it < steps; ++it) {
    if (w.tgroup.y & 0xFFu) {
      if (cnt) ++cnt[1];
      const unsigned k = __ffs(w.tgroup.y) - 1u;
      const unsigned idx = w.tgroup.x + __popc((w.tgroup.y >> 8) & ((1u << k) - 1u));
      w.tgroup.y &= ~(1u << k);
      const float4* tp = tris + 3 * (size_t)idx;
      const float4 p1 = __ldg(tp + 0), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
      const float t = tri_t(r, p1, e1, e2);
      if ((r.tmin < t) && (t < r.tmax)) {
        hit_face = __float_as_int(p1.w);
        if (ANY) return true;
        r.tmax = t;
      }
      if (w.tgroup.y & 0xFFu) continue;
    }
    if (w.ngroup.y <= 0x00FFFFFFu) {
      if (sp == 0) return true;
      w.ngroup = stack[--sp];
    }
    const unsigned b = 31u - __clz(w.ngroup.y);
    const unsigned slot = (b - 24u) ^ w.oct;
    const unsigned node = w.ngroup.x + __popc(w.ngroup.y & ((1u << slot) - 1u) & 0xFFu);
    w.ngroup.y &= ~(1u << b);
    if (w.ngroup.y > 0x00FFFFFFu) {
      if (sp >= kWideStack) {
        *overflow = true;
        return true;
      }
      stack[sp++] = w.ngroup;
    }
    if (cnt) ++cnt[0];
    wide_node(S, r, w, node);
  }
  return false;
}

// Persistent traversal over `count` rays with per-lane refill: every lane that
// finished its ray takes the next one from the global counter, so warps stay
// full while rays of very different lengths run side by side.
// Src: RayT load(int i); Dst: void store(int i, const RayT&, int hit_face).
// steps: traversal steps a lane runs between two refill points (STEPS unless
// given at run time).
template <bool ANY, int STEPS, class Src, class Dst>
__device__ __forceinline__ void trace_persistent_wide(const DevScene& S, int count, int* work, Src src, Dst dst,
                                                      bool* overflow, int steps) {
  const int lane = threadIdx.x & 31;
  uint2 stack[kWideStack];
  int i = -1;
  bool exhausted = false;
  RayT r;
  WideState w;
  int sp = 0, hit = -1;
  for (;;) {
    const bool need = (i < 0) && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(work, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int k = base + __popc(m & ((1u << lane) - 1u));
        if (k < count) {
          i = k;
          r = src(i);
          wide_init(r, w);
          sp = 0;
          hit = -1;
        }
      }
      if (base + __popc(m) >= count) exhausted = true;
    }
    const bool active = i >= 0;
    if (!__any_sync(0xffffffffu, active)) break;
    if (active && wide_steps<ANY>(S, r, w, sp, hit, stack, steps, overflow)) {
      dst(i, r, hit);
      i = -1;
    }
  }
}

template <bool ANY, int STEPS, class Src, class Dst, int PREC>
__device__ __forceinline__ void trace_persistent_binary(const DevScene& S, int count, int* work, Src src, Dst dst,
                                                        bool* overflow, int steps) {
  const int lane = threadIdx.x & 31;
  typename StackEntry<ANY>::type stack[PREC == 3 ? kQuadStack : PREC >= 4 ? 1 : kStackDepth], top;
  int i = -1;
  bool exhausted = false;
  RayT r;
  int ref = 0, sp = 0, hit = -1, leaf = kQuadEmpty, par = -1, sib = -1;
  unsigned long long bits = 0;
  bool finite = true;
  for (;;) {
    const bool need = (i < 0) && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(work, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int k = base + __popc(m & ((1u << lane) - 1u));
        if (k < count) {
          i = k;
          r = src(i);
          finite = ray_is_finite(r);
          ref = S.root_ref;
          leaf = kQuadEmpty;
          sp = 0;
          bits = 0;
          par = sib = -1;
          hit = -1;
        }
      }
      if (base + __popc(m) >= count) exhausted = true;
    }
    const bool active = i >= 0;
    if (!__any_sync(0xffffffffu, active)) break;
    bool done = false;
    if (active) {
      if constexpr (PREC == 3)
        done = quad_steps<ANY>(S, r, ref, leaf, sp, hit, finite, stack, top, steps, overflow);
      else if constexpr (PREC >= 4)
        done = bitstack_steps<ANY, PREC - 4>(S, r, ref, bits, par, sib, hit, finite, steps);
      else
        done = trav_steps<ANY, PREC>(S, r, ref, sp, hit, finite, stack, top, steps, overflow);
    }
    if (done) {
      dst(i, r, hit);
      i = -1;
    }
  }
}

// PREC: 0 FP32 records, 1 FP16 records (binary, the reference's visit order),
// 2 the wide BVH with 8-bit child boxes, 3 4-wide FP16 nodes, 4 / 5 FP32 / FP16
// records traversed without a stack (bitstack_steps).
template <bool ANY, int STEPS, class Src, class Dst, int PREC = 0>
__device__ __forceinline__ void trace_persistent(const DevScene& S, int count, int* work, Src src, Dst dst,
                                                 bool* overflow, int steps = STEPS) {
  if constexpr (PREC == 2)
    trace_persistent_wide<ANY, STEPS>(S, count, work, src, dst, overflow, steps);
  else
    trace_persistent_binary<ANY, STEPS, Src, Dst, PREC>(S, count, work, src, dst, overflow, steps);
}


}  // namespace tr
}  // namespace mt
