/*
 * mambatracer.h - C-ABI of the GB300 wavefront GI path tracer.
 *
 * Drop-in boundary for MambaTracer's render path: the Java host
 * (src/cl/device/CDeviceGI.java and the classes it drives) reaches these entry
 * points through Panama FFM or JNI in place of JOCL. Plain pointers and sizes
 * only. Every struct that crosses this boundary keeps the reference's OpenCL
 * byte layout:
 *   points    float4 per vertex (w = 0)            src/cl/scene/CMesh.java:339-357
 *   uvs       float2 per uv
 *   normals   float4 per normal
 *   faces     Face, 10 x int32 (40 B)              src/cl/kernel/Util.cl:95-102
 *   materials Material, 144 B                      src/cl/kernel/Bsdf.cl:24-50
 *   nodes     BVHNode, 7 x int32 (28 B)            src/cl/kernel/NormalBVH.cl:1-11
 *   bounds    BoundingBox, 2 x float4 (32 B)       src/cl/kernel/Util.cl:116-121
 *   rays      Ray (80 B)                           src/cl/kernel/Util.cl:129-138
 *   camera    CameraStruct (64 B)                  src/cl/kernel/Util.cl:78-85
 *
 * Errors: every call returns 0 (MT_OK) or a negative MT_ERR_* code; the
 * message of the last failure on the calling thread is mt_last_error(). This
 * replaces the CLException JOCL throws (src/cl/ui/fx/main/TracerAPI.java:79).
 * Device-side failures (a bounded wait that ran out) are latched in the
 * context and returned by the next call that synchronises (MT_ERR_DEVICE).
 *
 * Threading: one CUDA stream per context, calls on one context are serialised
 * by an internal mutex (the reference serialises on one in-order OpenCL queue,
 * src/cl/device/CDeviceGI.java:200-203). Only calls that return data to the
 * host wait for the device.
 */
#ifndef MAMBATRACER_H
#define MAMBATRACER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MT_OK 0
#define MT_ERR_INVALID -1   /* bad argument, malformed array, unknown name */
#define MT_ERR_CUDA -2      /* a CUDA runtime call failed */
#define MT_ERR_NOMEM -3     /* device allocation failed / over budget */
#define MT_ERR_DEPTH -4     /* BVH deeper than the 64-level traversal stack */
#define MT_ERR_DEVICE -5    /* a kernel latched an error (bounded wait expired) */
#define MT_ERR_BUSY -6      /* served mode: admission refused, retry later; a scene still in use */
#define MT_ERR_TIMEOUT -7   /* served mode: a wait ran out before the request finished */

typedef struct mt_context mt_context;
typedef struct mt_buffer mt_buffer;
typedef struct mt_kernel mt_kernel;
typedef struct mt_scene mt_scene;
typedef struct mt_job mt_job;

/* ------------------------------------------------------------ context */

/* OpenCLConfiguration.getDefault (src/cl/ui/fx/main/TracerAPI.java:86-90). */
int mt_ctx_create(int device, mt_context** out);
int mt_ctx_destroy(mt_context* ctx);
/* OpenCLConfiguration.finish (src/cl/device/CDeviceGI.java:428). */
int mt_finish(mt_context* ctx);
const char* mt_last_error(void);
/* Library build string (arch, parity flags). */
const char* mt_version(void);

/* ---------------------------------------- low level: buffers (CMemory) */

/* OpenCLConfiguration.createBufferB/I/F (e.g. src/cl/device/CDeviceGI.java:152-162). */
int mt_buf_alloc(mt_context* ctx, size_t bytes, mt_buffer** out);
/* createFromI/F (e.g. src/cl/scene/CMesh.java:341-345): allocate and upload. */
int mt_buf_create_from(mt_context* ctx, const void* host, size_t bytes, mt_buffer** out);
/* CMemory.transferToDevice / setCL (src/cl/algorithms/CCompact.java:81). */
int mt_buf_write(mt_buffer* buf, size_t offset, const void* host, size_t bytes);
/* CMemory.transferFromDevice / getCL (src/cl/device/CDeviceGI.java:357). */
int mt_buf_read(mt_buffer* buf, size_t offset, void* host, size_t bytes);
/* Fill with a repeated 4-byte pattern (the Init*Data kernels' job). */
int mt_buf_fill32(mt_buffer* buf, uint32_t pattern, size_t offset, size_t bytes);
size_t mt_buf_size(const mt_buffer* buf);
/* CResourceFactory.releaseMemory (src/cl/scene/CNormalBVH.java:56). */
int mt_buf_free(mt_buffer* buf);

/* ----------------------------- low level: kernels by name (CKernel) */

/* OpenCLConfiguration.createKernel(name, args...) (e.g. src/cl/device/CDeviceGI.java:168-178).
 * Names are the reference's __kernel names; the argument list is the
 * reference's (buffers in the reference layouts). Supported: the plain
 * wavefront set listed by mt_kernel_names(). */
int mt_kernel_create(mt_context* ctx, const char* name, mt_kernel** out);
const char* mt_kernel_names(void);
/* CKernel.putArg(i, mem) (src/cl/device/CDeviceGI.java:301). */
int mt_kernel_set_arg_buf(mt_kernel* k, int index, mt_buffer* buf);
/* __local scratch arguments (CLocalMemory.LOCALINT/LOCALFLOAT): size only. */
int mt_kernel_set_arg_local(mt_kernel* k, int index, size_t bytes);
/* OpenCLConfiguration.execute1DKernel(k, global, local): local is a hint;
 * work-items >= global are not launched. */
int mt_launch_1d(mt_kernel* k, size_t global, size_t local);
int mt_kernel_destroy(mt_kernel* k);

/* --------------------------------------------------- scene and BVH */

/* Mesh arrays (CMesh.initCLBuffers, src/cl/scene/CMesh.java:339-357). uvs and
 * normals may be NULL when no face references them (uvx/nx = -1). */
int mt_scene_create(mt_context* ctx, const float* points, int npoints, const float* uvs, int nuvs,
                    const float* normals, int nnormals, const int32_t* faces, int nfaces,
                    const void* materials, int nmaterials, mt_scene** out);
/* OBJ text to the mesh arrays mt_scene_create takes: what TracerAPI.initMesh
 * (src/cl/ui/fx/main/TracerAPI.java:393-438) gets from its OBJ parser into
 * CMesh. v / vt / vn / f (v, v/vt, v//vn, v/vt/vn; negative indices count back;
 * polygons split into triangle fans); each distinct `o` or `g` name is the next
 * material (faces before any name: material 0). counts_out[5] receives the
 * numbers of points, uvs, normals, faces and materials; with the array pointers
 * NULL only the counts are returned, otherwise points (4 floats each), uvs (2),
 * normals (4) and faces (10 ints) are filled. No device work, no context. */
int mt_obj_parse(const char* text, size_t len, int32_t* counts_out, float* points_out, float* uvs_out,
                 float* normals_out, int32_t* faces_out);
/* CNormalBVH.build (src/cl/scene/CNormalBVH.java:45-148) on the host, same
 * node layout; optional copies of nodes (7*(2N-1) ints) and bounds (8*(2N-1)
 * floats) are returned. depth_out: the BVH depth. */
int mt_bvh_build(mt_scene* scene, int32_t* nodes_out, float* bounds_out, int* depth_out);
/* The same build on host arrays only (no device work, no context): fills
 * nodes_out (7*(2N-1) ints) and bounds_out (8*(2N-1) floats) as the Java
 * CNormalBVH fills its CMemory<CNode>/CMemory<CBound> (CNormalBVH.java:59-79). */
int mt_bvh_build_host(const float* points, int npoints, const int32_t* faces, int nfaces, int32_t* nodes_out,
                      float* bounds_out, int* depth_out);
/* The same tree (CNormalBVH.build's splits, node numbering and bounds) built on
 * the GPU, level by level, straight into the traversal layout; nodes_out /
 * bounds_out (may be NULL) receive the reference-layout arrays, equal to
 * mt_bvh_build's. */
int mt_bvh_build_device(mt_scene* scene, int32_t* nodes_out, float* bounds_out, int* depth_out);
/* Copy of the scene's traversal layout: interior records (nrec x 64 B: the two
 * child boxes and child refs) and triangle slots (N x 48 B), either pointer may
 * be NULL; nrec_out / root_ref_out receive the record count and the root ref. */
int mt_scene_layout_read(mt_scene* scene, void* records_out, void* tris_out, int* nrec_out, int* root_ref_out);
/* Use a BVH built elsewhere (the Java builder's nodes/bounds buffers). */
int mt_bvh_import(mt_scene* scene, const int32_t* nodes, const float* bounds, int nnodes);
/* Traversal format: 0 = FP32 child boxes (default, 64-byte records, the
 * reference's visit order); 1 = FP16 child boxes rounded outward (32-byte
 * records); 2 = a wide BVH of up to eight children with 8-bit boxes rounded
 * outward (96-byte nodes); 3 = 4-wide nodes holding a record's grandchildren with
 * FP16 boxes rounded outward (64-byte nodes, leaves tested in warp-wide batches).
 * Formats 1-3 are kept beside the FP32 records and rebuilt with every BVH build
 * or import. Outward-rounded boxes contain the FP32 boxes, so closest hits are
 * the same triangles at the same distances; only which of two triangles hit at
 * exactly the same distance is reported can change with the visit order, and
 * among coplanar triangles hit within a few ulps of each other format 2 keeps
 * the nearer and format 3 either (its choice may change between runs, since
 * its leaf tests wait for the warp). Any-hit answers are the same in every
 * format. */
int mt_scene_set_bvh_precision(mt_scene* scene, int precision);
/* Replace the material table (TracerAPI material edits, src/cl/ui/fx/main/TracerAPI.java:371). */
int mt_scene_set_materials(mt_scene* scene, const void* materials, int nmaterials);
int mt_scene_light_count(const mt_scene* scene);
/* Bind a material's texture image (the images CTextureApplyPass.process reads
 * on the host, src/cl/algorithms/CTextureApplyPass.java:37-92): kind 0 diffuse,
 * 1 glossy, 2 roughness, 3 mirror (kept, never applied, as in the reference);
 * argb: width*height ints in JavaFX PixelReader.getArgb order (row-major,
 * 0xAARRGGBB); NULL removes the image. Materials flag their textures
 * (isDiffuseTexture, ...); renders sample them on the device at the hit's uv. */
int mt_scene_set_texture(mt_scene* scene, int material, int kind, const int32_t* argb, int width, int height);
int mt_scene_destroy(mt_scene* scene);

/* ------------------------------------------------ environment light */

/* CEnvironment.setEnvironmentMap (src/cl/algorithms/CEnvironment.java:46-60):
 * rgb is float4 per texel (lat-long, width x height). The luminance and the
 * inclusive SAT are built on the GPU in FP64 (stored FP32 for sampling). */
int mt_env_set(mt_scene* scene, const float* rgb, int width, int height);
/* Same, with the luminance and SAT given (e.g. the host SAT of the reference). */
int mt_env_set_with_sat(mt_scene* scene, const float* rgb, const float* lum, const float* sat, int width,
                        int height);
int mt_env_clear(mt_scene* scene);
/* Copy out the GPU-built luminance / FP64 SAT (either may be NULL). */
int mt_env_read(mt_scene* scene, float* lum, double* sat64, float* sat32);

/* Adaptive light grid (CAdaptiveEnvironment, src/cl/algorithms/CAdaptiveEnvironment.java:69-145):
 * nu x nv values, (nu/rx) x (nv/ry) cells of rx x ry tiles (reference: 1600 x 1600, 16 x 32;
 * rx, ry in {8, 16, 32}). enable: 0 = off (environment sampled off the full-map SAT, as the
 * reference renders), 1 = grid-guided environment sampling in mode-1 jobs with per-cell SATs in
 * the reference's FP32 order, 2 = the same with FP64 per-cell SATs. Each mode-1 job keeps its own
 * grid (it depends on the job's camera); rx and ry must divide the environment map's size. */
int mt_env_grid_config(mt_scene* scene, int nu, int nv, int rx, int ry, int enable);
/* Per-cell SAT of a given func (prefixSumRowSubgrid + prefixSumColSubgrid,
 * src/cl/kernel/LightGrid.cl:347-400); fp64 != 0 builds it in FP64. */
int mt_env_grid_sat(mt_context* ctx, const float* func, float* sat_out, int nu, int nv, int rx, int ry,
                    int fp64);

/* ---------------------------------------------------------- rendering */

typedef struct mt_render_config {
  int width, height;
  int max_depth;     /* bounces per path (reference: 15, CDeviceGI.java:226) */
  int mode;          /* 0 = reference semantics, 1 = benchmark semantics (pixel-keyed RNG, RR, Q1/Q2 fixed) */
  int rr_depth;      /* mode 1: Russian roulette from this bounce on (0 = off) */
  int film_kahan;    /* 1 = compensated film sums (default), 0 = plain FP32 adds as the reference */
  int spp;           /* passes per mt_render_frame call */
  int use_graph;     /* 1 = replay each frame's launches as a CUDA graph */
  int profile;       /* 1 = time every kernel launch with CUDA events (no graph) */
  int inflight;      /* frames kept in flight on their own streams, 0 or 1 = one (1..8); each
                        in-flight frame has its own path state and film, summed on read.
                        profile = 1 forces one. */
  int grid_updates;  /* mode 1 with the scene's light grid on: the first grid_updates frames add
                        the luminance of environment hits into the grid, which is updated after
                        each of them (CDeviceGI.java:263-264 updates after the first 5) */
} mt_render_config;

/* A render job: film + path state resident on the device (CDeviceGI.setup,
 * src/cl/device/CDeviceGI.java:116-164). */
int mt_job_create(mt_context* ctx, mt_scene* scene, const mt_render_config* cfg, mt_job** out);
int mt_job_destroy(mt_job* job);
/* The job's light grid (nu * nv floats each, NULL to skip): func (the sampled
 * function), its per-cell SAT, and the accumulated environment luminance. */
int mt_job_grid_read(mt_job* job, float* func, float* sat, float* accum);
/* CDeviceGI.updateCamera (src/cl/device/CDeviceGI.java:308-313). */
int mt_job_set_camera(mt_job* job, const void* camera);
/* One GI frame: CDeviceGI.loop (src/cl/device/CDeviceGI.java:214-271) without
 * the texture pass. seeds: in mode 0 the State seed pair of each
 * allocateState() call in launch order (2 * (1 + 2 * max_depth) ints per
 * pass), NULL in mode 1. frame_count: State.frameCount of the first pass. */
int mt_render_frame(mt_job* job, const int32_t* seeds, float frame_count);
/* CImage film: accum (float4 per pixel). resolve != 0 divides by the frame
 * count as averageAccum does (src/cl/kernel/Image.cl:29-67). */
int mt_film_read(mt_job* job, float* rgba, int resolve);
/* The same read, enqueued: copies the film as of every frame submitted so far
 * into rgba (pinned host memory for an asynchronous copy) and returns at once,
 * so the next frames can be submitted while this one finishes. Up to eight
 * reads stay pending; a ninth first completes the oldest. rgba must stay valid
 * until its read completes (mt_film_wait, mt_film_read, mt_film_clear, or the
 * ninth read after it); resolve is applied then. No counterpart in the
 * reference, whose image read (CImage.processImage/readImage) blocks. */
int mt_film_read_async(mt_job* job, float* rgba, int resolve);
int mt_film_wait(mt_job* job);
int mt_film_clear(mt_job* job);
/* The preview device's frame (CDeviceRT.loop, src/cl/device/CDeviceRT.java:176-197,
 * src/cl/kernel/Raytrace.cl): unjittered camera rays, closest hit, quick
 * colour (emission, or diffuse colour x cosine to the camera) or the
 * environment texel with gamma 2.2, as ARGB ints; group (may be NULL): the hit's
 * material index per pixel, -1 on a miss (updateGroupbufferShadeImage). Host
 * arrays of width * height ints; waits for the result. */
int mt_preview_frame(mt_scene* scene, const void* camera, int width, int height, int32_t* argb, int32_t* group);

/* The displayed image: CImage.processImage + CDeviceGI.updateImage
 * (src/cl/image/CImage.java:124-136, src/cl/device/CDeviceGI.java:355-362,
 * src/cl/kernel/Image.cl:29-118): film / frame count, Reinhard on the luminance
 * scaled by exposure / (log-average luminance), gamma, packed as ARGB ints
 * (width * height). Pixels with zero luminance keep their previous value
 * (opaque black after job creation or mt_film_clear). The log-average is taken
 * over the current film on every call (the reference's float scan for it is
 * defective and runs on its first two frames only); log_average (may be NULL)
 * receives it. Reference defaults: exposure 0.18, gamma 2.2. */
int mt_image_argb(mt_job* job, int32_t* argb, float exposure, float gamma, float* log_average);
/* Rays traced so far: [primary, extension, shadow], and the live queue length
 * after each bounce of the last pass (max_depth ints). */
int mt_job_stats(mt_job* job, int64_t* rays3, int32_t* counts);
/* Rays traced since the job was created or its film cleared: [primary,
 * extension, shadow], counted on the device. */
int mt_job_total_rays(mt_job* job, int64_t* rays3);
/* Device time of the last mt_render_frame, in ms (CUDA events on the job's stream). */
int mt_job_last_ms(mt_job* job, float* ms);
/* Kernels the job's frames have launched (graph nodes included): per pass the
 * ray generation, per bounce the closest-hit traversal, shading (one launch or
 * two) and the shadow rays, and the ray totals; per frame the film merge of
 * jobs with frames in flight. Light-grid updates are not counted. */
int mt_job_launches(mt_job* job, int64_t* n);
/* Profiled jobs: device time of each launch of the last frame, in ms, pass by
 * pass: [raygen, then per bounce trace_closest, shade, trace_shadow] =
 * spp * (1 + 3 * max_depth) floats. */
int mt_job_kernel_ms(mt_job* job, float* ms);

/* CUDA event slots on the context's stream (0..7): record, and the device
 * time between two recorded slots. */
int mt_ctx_event_record(mt_context* ctx, int slot);
int mt_ctx_event_elapsed(mt_context* ctx, int from_slot, int to_slot, float* ms);

/* --------------------------------------------------- queue compaction */

/* CompactAtomic (src/cl/kernel/Compact.cl:21-40) as CCompact.execute uses it
 * (src/cl/algorithms/CCompact.java:79-89): keeps the n Intersection records
 * (96 B each) whose hit flag is set, with their pixel ids, writing them from
 * slot *count_io onwards in input order, and adds the kept count to
 * *count_io. All five pointers are device memory (see mt_buf_device_ptr).
 * Input order is the order a serial run of CompactAtomic produces. The call
 * returns when the compaction has finished. */
int mt_compact_isects(mt_context* ctx, const void* isects_in, const int32_t* pixels_in, int n, void* isects_out,
                      int32_t* pixels_out, int32_t* count_io);
/* Device address of a buffer, for entry points that take device memory. */
void* mt_buf_device_ptr(mt_buffer* buf);
/* The same compaction for callers that cannot allocate device memory (a host
 * whose device memory all belongs to another allocator, or a plugin that may
 * not allocate on its caller's behalf). No counterpart in the reference. It
 * needs no context and allocates nothing: its scratch is a fixed array inside
 * the library (128 KiB per GPU that loads it), so n may be at most 4194304
 * records; larger n is refused with MT_ERR_INVALID. The caller passes inputs
 * and outputs in device memory and a CUDA stream (NULL: the default stream);
 * the call returns when the compaction on that stream has finished. It runs in
 * the CUDA context current on the calling thread (the current device's primary
 * context unless the host made another one current). Its first call on a
 * device looks up the scratch array's device address in that context, and
 * looks it up again whenever a different context is current there (another
 * context, or a new primary context after cudaDeviceReset). Every call uses
 * the same array: calls that overlap on the GPU (other streams, other host
 * threads) race. Errors read through mt_last_error(). */
int mt_compact_isects_noalloc(void* stream, const void* isects_in, const int32_t* pixels_in, int n,
                              void* isects_out, int32_t* pixels_out, int32_t* count_io);

/* ------------------------------------------------------ launch shapes */

/* The hot kernels' launch shapes, process-wide (no reference counterpart: its
 * local sizes are fixed, src/cl/device/CDeviceGI.java:122). The reference's
 * block size, queue length and regeneration threshold map to: the traversal
 * and shading builds (resident blocks per SM their registers are bounded
 * for), the persistent traversal grid of a launch that shares the GPU with
 * other frames, and the traversal steps between refills of finished lanes.
 * Every choice renders the same films; mambatracer_gb300.tune searches them
 * and persists the best as JSON. Render jobs capture their graphs again after
 * a change; set it between frames. */
typedef struct mt_tuning {
  int closest_minb, shadow_minb; /* traversal builds: 8, 12 or 16 blocks of 128 threads per SM */
  int closest_grid, shadow_grid; /* blocks per SM of a shared traversal launch, 0..32 (0: half of what fits) */
  int shade_minb;                /* shading build: 3, 4 or 5 blocks of 256 threads per SM */
  int refill_steps;              /* traversal steps between lane refills, 4..1024 */
  int shadow_stream;             /* 1: a frame's shadow rays run beside its next bounce's extension rays; 0 or 1 */
} mt_tuning;
int mt_tuning_get(mt_tuning* out);
int mt_tuning_set(const mt_tuning* in); /* MT_ERR_INVALID when a field is out of range */

/* ------------------------------------------------------- ray queries */

/* Closest hit over n rays in the reference Ray layout (80 B each, tMax is
 * updated as IntersectPrimitives does): t_out and prim_out (-1 on a miss). */
int mt_trace_closest(mt_scene* scene, const void* rays, int n, float* t_out, int32_t* prim_out);
/* Any hit (testOcclusion, src/cl/kernel/NormalBVH.cl:235-317): 1 = occluded. */
int mt_trace_any(mt_scene* scene, const void* rays, int n, int32_t* occluded_out);
/* The same queries with the traversal work each ray costs: counts_out holds
 * 2 ints per ray, interior-node visits and triangle tests, in the scene's
 * record format (FP32 or FP16 binary records: the visits of the reference's
 * stackless traversal, src/cl/kernel/NormalBVH.cl:14-92; the wide BVH: its
 * 96-byte node visits). any != 0: any-hit (t_out unused, prim_out = occluded
 * flags). No reference counterpart: it measures the algorithm's memory work
 * (the roofline's algorithmic bytes). */
int mt_trace_counts(mt_scene* scene, const void* rays, int n, int any, float* t_out, int32_t* prim_out,
                    int32_t* counts_out);
/* Device-resident variant for benchmarks: rays/outputs are mt_buffers. */
int mt_trace_closest_dev(mt_scene* scene, mt_buffer* rays, int n, mt_buffer* t_out, mt_buffer* prim_out,
                         float* ms_out);

/* ---------------------------------------------------------------- served mode
 * Many render requests of different scenes, resolutions and sample counts run
 * concurrently on one GPU (the reference renders one job at a time,
 * CDeviceGI.loop, src/cl/device/CDeviceGI.java:214-271). A request renders spp
 * benchmark-semantics passes (mode 1) of one camera and returns its
 * accumulated film. A scheduler thread admits requests first come, first
 * served onto `lanes` preallocated lanes (stream + path state for the largest
 * frame) within a budget of path-state bytes (200 B per pixel; 0 = no limit);
 * no device memory is allocated while requests run. Scenes used by queued or
 * running requests cannot be destroyed (MT_ERR_BUSY).
 * merged = m (1..lanes): the running requests share wavefront queues (lanes x
 * the largest frame paths, at most 2^30) instead of a lane each; the slots are
 * split over m streams, and each stream issues rounds, a round being one merged
 * pass per scene holding the next pass of every running request of its slots.
 * A request joins at its stream's next round. A cancelled running request
 * stops at the next round (state CANCELLED, no film). Films are the same, bit
 * for bit, in both modes. */
typedef struct mt_server mt_server;
typedef struct mt_server_config {
  int lanes;                 /* requests in flight at once (1..256) */
  int max_width, max_height; /* largest frame (its pixel count bounds every request) */
  int max_spp;               /* largest spp per request */
  int max_depth;             /* bounces per path */
  int rr_depth;              /* Russian roulette from this bounce on (0 = off) */
  int film_kahan;            /* compensated film sums */
  int merged;                /* m >= 1: running requests share wavefront queues on m streams */
  uint64_t budget_bytes;     /* admission budget of path state + film, 0 = unlimited */
} mt_server_config;
typedef struct mt_served_stats {
  int64_t completed, cancelled, failed, queued, running, max_queue;
  int64_t rays[3];  /* primary, extension, shadow rays traced by the server */
  double p50_ms, p95_ms, p99_ms, max_ms;  /* latency, submission to film delivered, of completed requests */
  double span_ms;   /* first submission to last completion */
} mt_served_stats;
int mt_server_create(mt_context* ctx, const mt_server_config* cfg, mt_server** out);

/* ------------------------------------------------------- merged batches */

/* One frame of a merged batch: size, passes, the first pass's frame number
 * (pass p renders frame frame_count + p, as mt_render_frame numbers a job's
 * passes) and its CameraStruct (64 B, src/cl/kernel/Util.cl:78-85). */
typedef struct {
  int width, height, spp;
  float frame_count;
  unsigned char camera[64];
} mt_batch_frame;
/* Render n frames of uneven size of one scene through one set of wavefront
 * queues (benchmark semantics, full-map environment sampling): each bounce is
 * one launch per kernel for all frames still rendering. No reference
 * counterpart (the reference renders one frame at a time); each frame's film
 * equals the frame rendered alone by a job or a served request with the same
 * camera, size, spp, frame number and path settings, bit for bit.
 * films_out: the frames' float4 films back to back in frame order (sum over
 * the frame's passes, not divided); rays_out (may be NULL): [primary,
 * extension, shadow] rays traced. Synchronous; allocates its queues per call. */
int mt_batch_render(mt_context* ctx, mt_scene* scene, const mt_batch_frame* frames, int nframes, int max_depth,
                    int rr_depth, int film_kahan, float* films_out, int64_t* rays_out);
/* Cancels queued requests, waits for running ones, frees the lanes. */
int mt_server_destroy(mt_server* server);
/* Queues a request; film_out (width * height float4, pinned or pageable host
 * memory, may be NULL) receives the accumulated film of its spp passes, whose
 * State.frameCount run from frame_count. No reference counterpart (the
 * reference's host drives its single device directly). */
int mt_job_submit(mt_server* server, mt_scene* scene, const void* camera, int width, int height, int spp,
                  float frame_count, float* film_out, int64_t* id_out);
/* state: 0 queued, 1 running, 2 done, 3 cancelled, 4 failed; latency_ms: -1
 * until done. */
int mt_job_poll(mt_server* server, int64_t id, int* state, double* latency_ms);
/* A queued request is dropped; a running one finishes but delivers nothing. */
int mt_job_cancel(mt_server* server, int64_t id);
/* Waits for a request (timeout_ms < 0: no limit; MT_ERR_TIMEOUT when it runs out). */
int mt_job_wait(mt_server* server, int64_t id, double timeout_ms);
/* Waits until no request is queued or running. */
int mt_server_drain(mt_server* server);
int mt_server_stats(mt_server* server, mt_served_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* MAMBATRACER_H */
