/*
 * flg.h — C ABI of the GB300 acceleration-structure and participating-media
 * library (libflg.so).
 *
 * The library replaces, for one GPU, these reference interfaces (paths are
 * relative to the fledge project root):
 *   - BVHBuilderBase::build / getBound / intersect(BVHRayHit&)
 *       src/experimental/base_bvh.hpp:105-117, implemented by
 *       RadixBVHBuilder (src/experimental/radix_bvh.hpp:32-84,
 *       src/experimental/radix_bvh.cpp:18-245)
 *   - Primitive::intersect / getBound and Accel (src/primitive.hpp:26-72,
 *       src/accel.hpp:12-54) — closest hit that shortens ray.m_tMax
 *   - Volume::tr / Volume::sample (src/volume.hpp:16-30), implemented by
 *       OpenVDBVolume::tr / sample (src/volume.cpp:75-148)
 *
 * Conventions
 *   - Every call returns an int status (flg_status).  No exception and no
 *     abort crosses the ABI; the reference's SErr/assert aborts become codes.
 *   - Device pointers unless a name ends in _host.  Buffers are owned by the
 *     caller; handles own what they allocate.
 *   - Calls are ordered on the context's stream and return without
 *     synchronising unless documented otherwise.  flg_ctx_sync() waits and
 *     reports device-side errors (bounded waits that timed out, traversal
 *     stack overflow).
 *   - One flg_ctx per host thread; handles may be shared read-only between
 *     contexts on the same device once built.
 */
#ifndef FLG_H_
#define FLG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define FLG_API extern "C" __attribute__((visibility("default")))
#else
#define FLG_API extern __attribute__((visibility("default")))
#endif

typedef enum flg_status {
  FLG_OK = 0,
  FLG_ERR_ARG = 1,         /* bad pointer, size or option; nothing launched */
  FLG_ERR_OOM = 2,         /* a device or pinned-host allocation failed */
  FLG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  FLG_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  FLG_ERR_STACK = 5,       /* traversal stack overflow (all stack sizes tried) */
  FLG_ERR_STATE = 6,       /* call not valid in the current state */
  FLG_ERR_UNSUPPORTED = 7  /* option not implemented */
} flg_status;

typedef struct flg_ctx_t *flg_ctx;
typedef struct flg_bvh_t *flg_bvh;
typedef struct flg_grid_t *flg_grid;
typedef struct flg_graph_t *flg_graph;

/* Rays, structure of arrays, n entries each.  tmin / tmax may be NULL, in
 * which case every ray uses tmin_const / tmax_const.  The reference's
 * BVHRayHit (base_bvh.hpp:41-50) holds ray_o, ray_d, tnear, tfar. */
typedef struct flg_rays {
  const float *ox, *oy, *oz;
  const float *dx, *dy, *dz;
  const float *tmin, *tmax;
  float tmin_const, tmax_const;
} flg_rays;

/* Closest-hit results, structure of arrays.  prim is the original index of
 * the triangle within its scene (-1 = miss); t is the hit distance (tmax on a
 * miss); u, v are barycentrics with P = (1-u-v) p0 + u p1 + v p2. */
typedef struct flg_hits {
  int32_t *prim;
  float *t, *u, *v;
} flg_hits;

typedef struct flg_build_opts {
  int32_t node_width;     /* traversal layout: 2, 4 or 8 (0 = 4) */
  int32_t leaf_size;      /* wide layouts: max triangles per leaf range (0 = 1) */
  int32_t keep_topology;  /* unused: flg_bvh_download derives the Karras arrays from the nodes */
  int32_t builder;        /* FLG_BUILDER_LBVH (0, the Karras radix tree), FLG_BUILDER_PLOC,
                             FLG_BUILDER_SAH or FLG_BUILDER_TREELET */
  int32_t treelet_rounds; /* FLG_BUILDER_TREELET: restructuring passes, 1..4 (0 = 3); other
                             builders ignore it */
} flg_build_opts;

/* Tree builders.  FLG_BUILDER_PLOC is a high-quality alternative to the
 * LBVH: parallel locally-ordered clustering over the same Morton order
 * (Meister & Bittner 2018), i.e. repeated merging of mutual nearest clusters
 * within a window of the sorted sequence, by the surface area of the merged
 * box.  Its builds synchronise with the host once per clustering iteration
 * (not capturable), and its handles keep no Karras arrays (flg_bvh_download
 * returns FLG_ERR_UNSUPPORTED).
 * FLG_BUILDER_SAH is BasicBVHBuilder's binned-SAH build
 * (src/experimental/base_bvh.cpp:33-173 with EBVHPartitionMethod::ESAH at
 * every node): top down, 16 buckets of triangle centroids along axis
 * depth % 3, cost 1/8 + (SA_L n_L + SA_R n_R) / SA, leaves at <= 8
 * triangles, depth 26 or no split cheaper than the leaf; stable partitions,
 * bucket indices clamped to [0, 15], and leaves of k > 1 triangles stored as
 * balanced binary subtrees.  Nodes are numbered as in the Karras tree, so
 * flg_bvh_download returns its topology (morton is not filled).  One host
 * synchronisation per tree level (not capturable).
 * FLG_BUILDER_TREELET is the LBVH refined by treelet restructuring (Karras &
 * Aila 2013): treelet_rounds bottom-up passes (3 by default), pass r
 * rebuilding the 7-leaf treelet below every node whose subtree holds at
 * least 7 << r triangles into its topology of least SAH cost (Ci = 1.2,
 * Ct = 1; subset dynamic programming); leaves are then renumbered in
 * depth-first order and nodes in Karras' numbering, so flg_bvh_download
 * returns its topology (morton is not in the new order).  Capturable.  Most
 * of the trace gain comes from the first pass: on 256 scenes of 34.6 M
 * triangles in all, one pass gave a 4.1 % faster trace for 43 ms of
 * restructuring, three passes 5.0 % for 86 ms. */
enum { FLG_BUILDER_LBVH = 0, FLG_BUILDER_PLOC = 1, FLG_BUILDER_SAH = 2, FLG_BUILDER_TREELET = 3 };

typedef struct flg_trace_opts {
  int32_t stack_depth;    /* 32 or 64 (0 = 64); overflowing rays are retried deeper */
  int32_t block_threads;  /* threads per block (0 = 256) */
  int32_t persistent;     /* 0: one ray per thread; 1: persistent work-stealing kernel;
                             2: persistent while-while kernel with speculative leaf
                             postponing (wide layouts) */
  int32_t refill_lanes;   /* persistent: refill a warp once this many lanes idle (0 = 16) */
  int32_t ray_sort;       /* 0: none; 1: sort rays by direction octant and origin cell */
  int32_t tri_test;       /* 0: watertight Pluecker (intersector.hpp:63-101, the experimental
                             path); 1: the live renderer's Moller-Trumbore Triangle::intersect
                             (shape.cpp:100-148; hits need 0 < t < tmax), traced one ray per
                             thread over the BVH2 layout */
} flg_trace_opts;

/* ------------------------------- context -------------------------------- */

/* Creates a context on `device` that issues work on `stream` (a cudaStream_t;
 * NULL creates a private non-blocking stream). */
FLG_API int flg_ctx_create(int32_t device, void *stream, flg_ctx *out);
FLG_API int flg_ctx_destroy(flg_ctx ctx);
/* Waits for the context's stream and returns the first device-side error
 * recorded since the previous sync (FLG_ERR_TIMEOUT, FLG_ERR_STACK). */
FLG_API int flg_ctx_sync(flg_ctx ctx);
FLG_API void *flg_ctx_stream(flg_ctx ctx);
/* Number of kernels the library has launched through this context (each
 * launch of a captured graph counts the kernels once, at capture). */
FLG_API int64_t flg_ctx_launch_count(flg_ctx ctx);
/* Test hook: caps every bounded device-side spin-wait at `spins` iterations
 * (0 restores the default).  Used to inject FLG_ERR_TIMEOUT from the host. */
FLG_API int flg_ctx_set_spin_limit(flg_ctx ctx, uint32_t spins);
/* Stage timing (no counterpart in the reference, which prints whole-build
 * timings only, bvh_test.hpp:30-36): with `on`, every build and trace issued
 * on ctx records a CUDA event at the end of each of its stages (setup,
 * bounds, morton, sort, climb, collapse, trace, trace_retry, trace_finish,
 * and the SAH / PLOC stages); nothing is recorded during a stream capture.
 * Turning it on or off discards the recorded marks. */
FLG_API int flg_ctx_set_stage_timing(flg_ctx ctx, int32_t on);
/* Waits for the last mark and writes the recorded stage times as a JSON
 * object {"stage": {"ms": summed milliseconds, "n": occurrences}, ...} in
 * first-seen order, then discards the marks.  FLG_ERR_ARG if json_len is too
 * small. */
FLG_API int flg_ctx_stage_times(flg_ctx ctx, char *json, size_t json_len);
FLG_API const char *flg_status_string(int status);
/* Test hook: launches one thread that waits, with the library's bounded
 * spin-wait, on a device word that nothing ever sets, then synchronises.
 * Returns FLG_ERR_TIMEOUT after `spins` polls and leaves the context usable. */
FLG_API int flg_debug_wait_unset_flag(flg_ctx ctx, uint32_t spins);
/* Copies the last error message of the context into buf (NUL-terminated). */
FLG_API int flg_ctx_last_error(flg_ctx ctx, char *buf, size_t len);

/* --------------------------------- build -------------------------------- */

/* Karras LBVH of one triangle mesh (RadixBVHBuilder::build,
 * radix_bvh.cpp:18-24,32-200).  pos: 3*n_vert floats (xyz interleaved).  idx:
 * 3*n_tri vertex indices, or NULL for a triangle soup (vertex k of triangle i
 * is 3i+k, n_vert = 3 n_tri).  The mesh arrays are borrowed, not copied, as
 * in the reference (radix_bvh.cpp:42-45): they must outlive the handle. */
FLG_API int flg_bvh_build(flg_ctx ctx, const float *pos, const int32_t *idx, int64_t n_tri,
                          int64_t n_vert, const flg_build_opts *opts, flg_bvh *out);

/* Many independent scenes built in one segmented pass.  Scene s owns
 * triangles [tri_offsets_host[s], tri_offsets_host[s+1]) of the shared
 * arrays; with idx != NULL indices are global vertex indices. */
FLG_API int flg_bvh_build_batched(flg_ctx ctx, const float *pos, const int32_t *idx,
                                  const int64_t *tri_offsets_host, int32_t n_scenes,
                                  int64_t n_vert, const flg_build_opts *opts, flg_bvh *out);

/* Rebuilds an existing handle over new vertex positions of the same size
 * without allocating (usable inside a CUDA graph capture). */
FLG_API int flg_bvh_rebuild(flg_ctx ctx, flg_bvh bvh, const float *pos);

FLG_API int flg_bvh_destroy(flg_bvh bvh);

typedef struct flg_bvh_info {
  int64_t n_tri;          /* all scenes */
  int32_t n_scenes;
  int32_t node_width;
  int64_t n_wide_nodes;
  int64_t device_bytes;   /* memory held by the handle */
  float bound[6];         /* scene 0: lower xyz, upper xyz (getBound()) */
} flg_bvh_info;
FLG_API int flg_bvh_info_get(flg_bvh bvh, flg_bvh_info *out);

/* Karras arrays of one scene, for parity checks (synchronous).  Host
 * pointers; NULL members are skipped.  Internal nodes are numbered as in the
 * reference (root = 0, children split and split+1). */
typedef struct flg_bvh_topology {
  uint32_t *morton;       /* n: sorted Morton codes */
  int32_t *perm;          /* n: sorted position -> original triangle */
  int32_t *split;         /* n-1 */
  uint8_t *leaf_flags;    /* n-1: bit0 left child is a leaf, bit1 right */
  int32_t *range_j;       /* n-1: other end j of the node's range */
  int32_t *parent;        /* n-1: internal-node parents (root: 0) */
  int32_t *leaf_parent;   /* n */
  float *bounds;          /* 6(n-1): node bound lower xyz, upper xyz */
  float *scene_bound;     /* 6: union of triangle bounds (Morton frame) */
} flg_bvh_topology;
FLG_API int flg_bvh_download(flg_bvh bvh, int32_t scene, flg_bvh_topology *out);

/* ------------------------------- traversal ------------------------------ */

/* Closest hit (RadixBVHBuilder::intersect, radix_bvh.cpp:26-30,202-245, with
 * the watertight Pluecker test of intersector.hpp:63-101).  A hit counts if
 * tmin <= t <= tmax; among equal t the first found is kept. */
FLG_API int flg_trace_closest(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n,
                              const flg_trace_opts *opts, flg_hits *out);

/* Any hit (IntersectP; no counterpart in the reference, whose shadow rays use
 * closest hit, integrator.cpp:29-37): occluded[i] = 1 if any triangle is hit
 * with tmin <= t <= tmax. */
FLG_API int flg_trace_any(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n,
                          const flg_trace_opts *opts, uint8_t *occluded);

/* Batched: rays [ray_offsets_host[s], ray_offsets_host[s+1]) go to scene s of
 * a batched handle; one persistent launch traces all scenes. */
FLG_API int flg_trace_closest_batched(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays,
                                      const int64_t *ray_offsets_host,
                                      const flg_trace_opts *opts, flg_hits *out);

/* Same as flg_trace_closest with host (preferably pinned) buffers: the call
 * stages rays to the device in chunks of 2^22 through two buffers, traces
 * each chunk on the context's stream and copies its hits back; every copy
 * runs on the context's copy stream in the order in(0) in(1) out(0) in(2)
 * out(1) ..., so copies overlap the traces but never each other (a
 * host-to-device and a device-to-host copy running at once each lose about
 * two thirds of their bandwidth).  Synchronous. */
FLG_API int flg_trace_closest_host(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays_host,
                                   int64_t n, const flg_trace_opts *opts, flg_hits *out_host);

/* Closest hit that allocates nothing (no counterpart in the reference).  For
 * callers that cannot call cudaMalloc when they trace — under an arena that
 * hands out all device memory up front, or in a frame loop where an
 * allocation would synchronise the device — whereas
 * flg_trace_closest allocates its scratch on a context's first trace.  Same
 * kernels and results as flg_trace_closest with default options; the
 * scratch is a fixed 8 MB device array inside the library, held on every GPU
 * that loads it until exit.  At most 1,048,576 rays per call (larger n:
 * FLG_ERR_ARG).  The first call on a device looks the array up
 * (cudaGetSymbolAddress) and must come before any stream capture (inside a
 * capture it returns FLG_ERR_STATE).  All calls share the array: calls that
 * overlap on the GPU race. */
FLG_API int flg_trace_closest_noalloc(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n,
                                      flg_hits *out);

/* Autotuner of the traversal (no counterpart in the reference): a staged
 * search on the given workload — (1) node width 2/4/8 with leaf ranges of
 * 1..4 triangles under each width's default kernel, (2) on the fastest
 * layout the kernel (one ray per thread, persistent, persistent while-while;
 * refill threshold 4/8/16; stack depth 32/64), (3) 128- or 256-thread
 * blocks, (4) for single-scene traces the ray-sort key.  Each trial is one
 * untimed and `reps` timed launches; its time is their median.  Leaves the
 * handle laid out at the fastest width and leaf size, returns the fastest
 * options in *best and writes a JSON record of every trial (NUL-terminated)
 * to json_out (FLG_ERR_ARG if json_len is too small).  Synchronous; not
 * capturable.  flg_autotune_trace: single-scene handles, reps = 5. */
FLG_API int flg_autotune_trace(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n,
                               flg_trace_opts *best, int32_t *best_node_width, char *json_out,
                               size_t json_len);
/* The same search over a batched handle and its rays (ray_offsets_host as in
 * flg_trace_closest_batched); reps in [1, 64]; also returns the leaf size. */
FLG_API int flg_autotune_trace_batched(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays,
                                       const int64_t *ray_offsets_host, int32_t reps, flg_trace_opts *best,
                                       int32_t *best_node_width, int32_t *best_leaf, char *json_out,
                                       size_t json_len);

/* Re-lays out the traversal nodes of a built handle at another width. */
FLG_API int flg_bvh_set_width(flg_ctx ctx, flg_bvh bvh, int32_t node_width, int32_t leaf_size);

/* Normals of fixed hits of a single-scene handle, for the interfaces that
 * return them with the hit (3 n floats, xyz interleaved; zeros where
 * prim < 0):
 *   FLG_NORMAL_PLUECKER: BVHRayHit::hit_ng (= hit_ns) of
 *     RadixBVHBuilder::intersect (radix_bvh.cpp:229-233): the Pluecker
 *     test's StableTriangleNormal of the ray-relative edges
 *     (intersector.hpp:44-60, 86-88), normalised with the Euclidean norm in
 *     double.  The reference's StableNormalize (common/vector.h:495-503) adds
 *     z instead of z*z; its normals are not unit vectors and it misses the
 *     triangles for which that sum is negative.
 *   FLG_NORMAL_GEOMETRIC: SInteraction::m_ng of the live renderer's
 *     Triangle::intersect (shape.cpp:141): normalize(cross(p1 - p0, p2 - p0))
 *     in fp32 with the reference's operation order.
 * rays: origins are read for FLG_NORMAL_PLUECKER; prim: device, n ids. */
enum { FLG_NORMAL_PLUECKER = 0, FLG_NORMAL_GEOMETRIC = 1 };
FLG_API int flg_hit_normals(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, const int32_t *prim,
                            int32_t kind, float *ng);

/* -------------------------------- adjoint ------------------------------- */

/* Gradient of (t, u, v) of fixed hits with respect to the vertex positions
 * (no counterpart in the reference).  dL_dt/du/dv: n floats (NULL = 0).
 * dL_dpos: 3*n_vert floats, accumulated with fp32 atomics. */
FLG_API int flg_hit_adjoint(flg_ctx ctx, const float *pos, const int32_t *idx, int64_t n_tri,
                            int64_t n_vert, const flg_rays *rays, int64_t n,
                            const flg_hits *hits, const float *dL_dt, const float *dL_du,
                            const float *dL_dv, float *dL_dpos);

/* ------------------------------- volumes -------------------------------- */

typedef struct flg_medium {
  float sigma_s;       /* scattering per unit density */
  float sigma_a;       /* absorption per unit density */
  float g;             /* Henyey-Greenstein asymmetry */
  float rr_threshold;  /* ratio-tracking roulette threshold (0.1 in volume.cpp:98); 0 disables */
  float majorant;      /* <= 0: maximum grid value (volume.cpp:52-59) */
} flg_medium;

/* Dense density grid: nx*ny*nz fp32 samples (x fastest) at the vertices of a
 * regular lattice spanning [box_lo, box_hi]; trilinear interpolation,
 * background 0 outside.  density is borrowed. */
FLG_API int flg_grid_create(flg_ctx ctx, const float *density, int32_t nx, int32_t ny, int32_t nz,
                            const float *box_lo_host, const float *box_hi_host,
                            const flg_medium *medium, flg_grid *out);
/* Sparse grid (the NanoVDBVolume that src/volume.hpp:72-92 declares but does
 * not implement): the lattice is cut into 8^3 bricks; brick_index (device,
 * [ceil(nz/8)][ceil(ny/8)][ceil(nx/8)] int32) holds each brick's slot in
 * bricks (device, n_bricks x 512 floats, z, y, x inside a brick, x fastest)
 * or -1 for a brick of background (0) values.  Lookups, tracking, sampling
 * and the adjoint behave exactly as on the dense grid with those values;
 * adjoint gradients are written in the bricks' layout (empty bricks are not
 * parameters).  Both arrays are borrowed. */
FLG_API int flg_grid_create_sparse(flg_ctx ctx, const int32_t *brick_index, const float *bricks,
                                   int64_t n_bricks, int32_t nx, int32_t ny, int32_t nz, const float *lo,
                                   const float *hi, const flg_medium *medium, flg_grid *out);
/* Converts a dense device grid into that layout: fills brick_index, stores
 * the count of non-empty bricks in *n_bricks (host) and, when bricks is not
 * NULL, copies them (max_bricks slots available).  Synchronises. */
FLG_API int flg_grid_sparsify(flg_ctx ctx, const float *density, int32_t nx, int32_t ny, int32_t nz,
                              int32_t *brick_index, float *bricks, int64_t max_bricks, int64_t *n_bricks);
FLG_API int flg_grid_destroy(flg_grid grid);
FLG_API int flg_grid_majorant(flg_grid grid, float *majorant_host);

/* Per-ray state after the last Russian-roulette survival (t, draw counter,
 * transmittance): the adjoint's checkpoint, 12 bytes per ray. */
typedef struct flg_tr_ckpt {
  float *t;
  uint32_t *k;
  float *c;
} flg_tr_ckpt;

/* Ratio-tracking transmittance (OpenVDBVolume::tr, volume.cpp:75-107).  Ray i
 * draws from Philox-4x32-10 stream (seed, i).  ckpt may be NULL. */
FLG_API int flg_volume_tr(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n,
                          uint64_t seed, float *T, const flg_tr_ckpt *ckpt);

/* Adjoint of flg_volume_tr: dL_dgrid += sum_i dL_dT[i] dT_i/dgrid, majorant
 * held constant.  T is the forward output.  With ckpt == NULL each ray's
 * forward is replayed to find its last roulette segment. */
FLG_API int flg_volume_tr_adjoint(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n,
                                  uint64_t seed, const float *dL_dT, const float *T,
                                  const flg_tr_ckpt *ckpt, float *dL_dgrid);

/* Delta tracking (OpenVDBVolume::sample, volume.cpp:109-148): success[i],
 * collision point p (3n floats, xyz interleaved), weight sigma_s/sigma_t on a
 * collision, 1 otherwise. */
FLG_API int flg_volume_sample(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n,
                              uint64_t seed, uint8_t *success, float *p, float *weight);

/* ---------------------------- path tracing ------------------------------ */

/* The integrator around traversal: PathIntegrator::Li (integrator.cpp:252-326)
 * with one-light next-event estimation (:69-120) over a triangle mesh whose
 * triangles [light_first, light_first + light_count) emit light_le (front
 * side, geometric normal (p1-p0) x (p2-p0)); every other triangle is
 * Lambertian with `albedo`.  Halton samples (sampler.h:143-252) in the
 * per-pixel order of integrator.cpp:136-159; camera as Camera (camera.h). */
typedef struct flg_pt_scene {
  const float *pos;        /* device, 3 * n_vert */
  const int32_t *idx;      /* device, 3 * n_tri, or NULL for a soup */
  int64_t n_tri, n_vert;
  int32_t light_first, light_count;
  float light_le[3];
  float albedo[3];
} flg_pt_scene;

typedef struct flg_pt_camera {
  float eye[3], target[3], up[3];
  float fov_deg;           /* Camera::m_fov (camera.h:25) */
  int32_t width, height;
} flg_pt_camera;

typedef struct flg_pt_stats {
  int64_t closest_rays, shadow_rays;  /* rays traced, all bounces and samples */
} flg_pt_stats;

/* Renders the image into radiance (device, 3 floats per pixel, row-major,
 * mean over spp) as a wavefront: camera rays, closest hit, shading with
 * queue compaction, shadow rays with any hit, per bounce.  bvh must be built
 * over the same mesh.  Synchronises once per bounce. */
FLG_API int flg_pathtrace(flg_ctx ctx, flg_bvh bvh, const flg_pt_scene *scene, const flg_pt_camera *cam,
                          int32_t spp, int32_t max_depth, const flg_trace_opts *opts, float *radiance,
                          flg_pt_stats *stats);

/* Volumetric path tracing (VolPathIntegrator::Li, src/integrator.cpp:407-510):
 * flg_pathtrace with the grid's medium filling the grid's box.  At each
 * surface hit, delta tracking over the segment may move the path vertex to
 * a scattering point (Henyey-Greenstein with the grid's g; beta *= sigma_s /
 * sigma_t); shadow rays are weighted by ratio-tracking transmittance
 * (VolEstimateTr, :40-66).  Tracking draws from Philox streams keyed by seed,
 * pixel, sample, bounce and purpose.  spp <= 65535, max_depth <= 255. */
FLG_API int flg_volpath(flg_ctx ctx, flg_bvh bvh, flg_grid grid, uint64_t seed, const flg_pt_scene *scene,
                        const flg_pt_camera *cam, int32_t spp, int32_t max_depth, const flg_trace_opts *opts,
                        float *radiance, flg_pt_stats *stats);

/* A homogeneous medium bounded by a closed mesh: the reference's HVolume
 * (src/volume.cpp:150-190) attached to a mesh primitive
 * (src/scene.cpp:224-228).  Triangles [first, first + count) of the scene
 * are its boundary; they carry no material. */
typedef struct flg_mesh_medium {
  int32_t first, count;
  float sigma_s[3], sigma_a[3];  /* per RGB channel */
  float g;                       /* Henyey-Greenstein asymmetry, |g| < 1 */
  float density;                 /* > 0 */
} flg_mesh_medium;

/* Volumetric path tracing with that medium (VolPathIntegrator::Li,
 * src/integrator.cpp:407-510): a path that reaches a boundary triangle passes
 * straight through (not counted as a bounce; the reference would dereference
 * the missing material there) and is inside afterwards if it entered
 * (d . ng < 0, ng = (p1 - p0) x (p2 - p0)); a ray leaving any material
 * surface is outside (SInteraction::SpawnRay, src/interaction.cpp:16-38).
 * Inside, HVolume::sample picks a channel and a distance; a scattering vertex
 * takes next-event estimation with the Henyey-Greenstein phase function and
 * a HGSampleP continuation.  Shadow rays follow VolEstimateTr
 * (integrator.cpp:40-66): a material surface blocks, a boundary multiplies
 * HVolume::tr of the segment travelled inside and switches the medium, and
 * the segment after the last boundary is not attenuated.  Tracking draws
 * come from Philox streams keyed by seed, pixel, sample, segment and purpose.
 * Up to 255 segments per path and 64 boundary crossings per shadow ray.
 * Synchronises once per segment; not capturable. */
FLG_API int flg_volpath_mesh(flg_ctx ctx, flg_bvh bvh, const flg_mesh_medium *medium, uint64_t seed,
                             const flg_pt_scene *scene, const flg_pt_camera *cam, int32_t spp, int32_t max_depth,
                             const flg_trace_opts *opts, float *radiance, flg_pt_stats *stats);

/* ---------------------------- mesh ingestion ---------------------------- */

/* A host mesh read from a file; arrays are malloc'ed by the library and
 * released by flg_host_mesh_free.  normal / uv are NULL when the file has
 * none. */
typedef struct flg_host_mesh {
  float *pos;     /* 3 * n_vert */
  float *normal;  /* 3 * n_vert or NULL */
  float *uv;      /* 2 * n_vert or NULL */
  int32_t *idx;   /* 3 * n_tri */
  int64_t n_vert, n_tri;
} flg_host_mesh;

/* Reads a PLY file (ASCII or binary) into a triangle mesh; replaces
 * MakeTriangleMesh (src/plymesh.cpp:19-86).  Faces with more than three
 * corners are fan-triangulated.  Host only (no context, no GPU).  On error
 * returns FLG_ERR_ARG and writes a message into err (err_len bytes). */
FLG_API int flg_ply_read(const char *path, flg_host_mesh *out, char *err, size_t err_len);
FLG_API void flg_host_mesh_free(flg_host_mesh *mesh);

/* ----------------------------- CUDA graphs ------------------------------ */

/* Captures every library call issued on ctx between begin and end into a
 * graph; calls that allocate are refused with FLG_ERR_STATE while capturing. */
FLG_API int flg_graph_begin(flg_ctx ctx);
FLG_API int flg_graph_end(flg_ctx ctx, flg_graph *out);
FLG_API int flg_graph_launch(flg_ctx ctx, flg_graph graph);
FLG_API int flg_graph_destroy(flg_graph graph);

/* --------------------------- synthetic inputs ---------------------------- */
/* Seeded generators of the benchmark workloads, on the device.  Philox
 * streams keyed by seed; identical across runs. */

/* Random triangle soup: centroid U[0,1]^3, vertices centroid + U[-r,r]^3.
 * pos: 9 n_tri floats.  first_tri offsets the stream (batched scenes). */
FLG_API int flg_gen_triangles(flg_ctx ctx, uint64_t seed, int64_t first_tri, int64_t n_tri,
                              float half_extent, float *pos);
/* Rays from a sphere of radius `radius` around `center` toward uniform points
 * of [0,1]^3 (SoA device arrays ox..dz, each n). */
FLG_API int flg_gen_rays(flg_ctx ctx, uint64_t seed, int64_t first_ray, int64_t n,
                         const float *center_host, float radius, float *ox, float *oy, float *oz,
                         float *dx, float *dy, float *dz);
/* 4-octave value noise on an nx*ny*nz lattice over [0,1]^3, remapped to
 * [0, scale]. */
FLG_API int flg_gen_noise_grid(flg_ctx ctx, uint64_t seed, int32_t nx, int32_t ny, int32_t nz,
                               float scale, float *density);

/* Version string of the library. */
FLG_API const char *flg_version(void);

#endif /* FLG_H_ */
