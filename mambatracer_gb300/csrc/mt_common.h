// Shared host/device definitions of the GB300 wavefront path tracer.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#include <vector_types.h>
#endif

namespace mt {

constexpr int kMaxDepth = 32;        // bounces per pass (reference: 15)
constexpr int kStackDepth = 64;      // traversal stack = the reference's 64-bit bitstack
constexpr int kWideStack = 32;       // wide-BVH traversal: node groups deferred (<= wide tree depth)
constexpr int kQuadEmpty = (int)0x80000000;  // an unused child slot of a 4-wide node
// 4-wide traversal stack: a 4-wide node spans two binary levels and defers at
// most three children, so a tree within the 64-level bound needs 3 * 32 entries.
constexpr int kQuadStack = 3 * (kStackDepth / 2);
constexpr int kWideWords = 6;        // uint4 per wide-BVH node: 80 bytes used, padded to 96 (three 32-byte loads)
constexpr int kTraceThreads = 128;   // threads per traversal CTA
constexpr int kTraceMinBlocksClosest = 12;  // register bounds of the traversal kernels (CTAs per SM)
constexpr int kTraceMinBlocksShadow = 8;
constexpr int kShadeThreads = 256;   // threads per shade CTA (one compaction tile)
constexpr int kShadeMinBlocks = 4;   // register bound of the shading kernel (CTAs per SM)

// Device error codes latched in Ctrl::error.
constexpr int kDevErrLookback = 1;   // decoupled look-back wait expired
constexpr int kDevErrStack = 2;      // traversal stack overflow (BVH deeper than 64)

// Reference Face (src/cl/kernel/Util.cl:95-102).
struct Face {
  int vx, vy, vz, uvx, uvy, uvz, nx, ny, nz, mat;
};

// Reference SurfaceParameter (src/cl/kernel/Bsdf.cl:24-42), 144 B.
struct Material {
  int isDiffuseTexture, isGlossyTexture, isRoughnessTexture, isMirrorTexture;
  float4 diffuse_color, diffuse_param, glossy_color, glossy_param;
  float4 mirror_color, mirror_param, emission_color, emission_param;
};
static_assert(sizeof(Material) == 144, "Material layout");

// Scene as seen by kernels. Traversal data is the GPU layout:
//   nodes: 4 float4 per interior record (depth-first preorder, root 0):
//     n0 = (L.min.x, L.max.x, L.min.y, L.max.y)
//     n1 = (R.min.x, R.max.x, R.min.y, R.max.y)
//     n2 = (L.min.z, L.max.z, R.min.z, R.max.z)
//     n3 = (bits(left ref), bits(right ref), 0, 0)
//   a child ref >= 0 is a record index, < 0 is ~(triangle slot).
//   tris: 3 float4 per triangle slot (leaf order): (p1.xyz, bits(face id)),
//     (p2 - p1, 0), (p3 - p1, 0), the edges of the reference's Moller-Trumbore.
//   qnodes: FP16 child boxes rounded outward (precision 1), 2 x 16 B per record:
//     (L.x, L.y, R.x, R.y) as (lo, hi) half2 pairs, then (L.z, R.z, left ref, right ref).
//   wnodes: the wide BVH (precision 2), kWideWords uint4 = 96 B per node (the
//     last 16 B unused, so that a node is three aligned 32-byte loads), root 0:
//     w0 = (origin x, y, z as float bits, ex | ey << 8 | ez << 16 | imask << 24):
//          per-axis scale 2^(e - 127), imask bit s = slot s holds an interior node
//     w1 = (first child node, first triangle, lmask, 0): lmask bit s = slot s holds
//          a triangle; the child node in interior slot s is first child + the
//          interior slots below s, the triangle in leaf slot s is wtris entry first
//          triangle + the leaf slots below s
//     w2 = (lo.x slots 0-3, lo.x 4-7, lo.y 0-3, lo.y 4-7), w3 = (lo.z .., hi.x ..),
//     w4 = (hi.y .., hi.z ..): one quantised plane per byte, plane = origin + q 2^(e-127);
//          an empty slot holds lo = 255, hi = 0 (never hit)
//   wtris: the triangles in wide-leaf order, 3 float4 each as in tris.
//   quad: 4-wide FP16 nodes (precision 3), 4 uint4 = 64 B, indexed like nodes: the
//     node of record r holds the grandchildren of r where a child of r is
//     interior and the child itself where it is a leaf, in the order left's
//     children, right's children; words 3c .. 3c + 2 = child c's x, y, z extents
//     as (lo rounded down, hi rounded up) half2 pairs, words 12 + c = child c's
//     ref (a record index, ~triangle slot, or kQuadEmpty: no child).
//   up: per record (parent record, the record's sibling ref), the root (-1, -1):
//     the links of the stackless traversal (bitstack_steps).
struct DevScene {
  const float4* nodes;
  const float4* qnodes;
  const float4* tris;
  const uint4* wnodes;
  const float4* wtris;
  const uint4* quad;
  const int2* up;
  int bitstack;  // binary formats: 1 = the stackless traversal (bitstack and parent links)
  int root_ref;
  int ntri;
  int nrec;
  int precision;  // traversal format: 0 FP32 records, 1 FP16 records, 2 the wide BVH, 3 4-wide FP16 nodes
  // shading data in the reference layout
  const float4* points;
  const float2* uvs;
  const float4* normals;
  const Face* faces;
  const Material* materials;
  const int* light_faces;
  int nlights;
  // textures: ARGB texel pool and, per material, 4 entries (diffuse, glossy,
  // roughness, mirror) of (first texel, width, height, 0); width 0 = no image
  const int* texels;
  const int4* tex_ref;
  int tex_on;
};

struct DevEnv {
  const float4* rgb;
  const float* lum;
  const float* sat;   // FP32 copy of the inclusive SAT used for sampling
  int w, h;
  int present;
  // adaptive light grid (mode 1): nu x nv, rx x ry tiles per cell
  const float* grid_func;
  const float* grid_sat;
  float* grid_accum;
  int grid_on;
  int nu, nv, rx, ry;
  // tabulated CDFs (dv::RegionTab) of each cell's region of the grid and of each
  // tile's region of the map; NULL: computed from the SATs
  const float* cell_marg;
  const float* cell_cond;
  const float* tile_marg;
  const float* tile_cond;
  // the same for the whole map (full-map sampling); NULL: from the SAT
  const float* env_marg;
  const float* env_cond;
};

// Per-pass control block in device memory (zeroed at the start of each pass).
struct Ctrl {
  int count[kMaxDepth + 2];     // queue length entering bounce b (count[1] = pixels)
  int shadow[kMaxDepth + 2];    // shadow rays emitted at bounce b
  int work[2 * (kMaxDepth + 2)];
  int tiles[kMaxDepth + 2];
  int live[kMaxDepth + 2];      // paths that go on after the hit phase of bounce b (two-launch shading)
  int tiles2[kMaxDepth + 2];    // chunk counter of the second shading launch
  int error;
  int pad;
  unsigned long long rays[3];   // primary, extension, shadow traced
};

// Per-pass parameters (uploaded once per pass from pinned host memory).
struct PassParams {
  float cam_m[16];       // view->world matrix rows (Matrix.cl:216-241 mInv)
  float cam_d;           // 1 / tan(radians(fov) / 2)
  float cam_a;           // width / height
  float inv_w, inv_h;    // 1 / width, 1 / height
  float dim_w, dim_h;    // width, height as floats
  float frame_count;     // State.frameCount
  int width, height;
  int max_depth;
  int mode;
  int rr_depth;
  int kahan;
  int grid_accum;        // 1: environment hits add their luminance into the light grid
  float cam_pos[4];      // camera position (LightGrid.cameraPosition)
  int seeds[2 * (1 + 2 * kMaxDepth)];  // mode 0: allocateState() seed pairs
};

}  // namespace mt
