// internal.h — host-side definitions shared by the translation units of
// libflg: context and handle layouts, node records, launch helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/flg.h"

namespace flg {

// BVH2 node: both children's boxes in the parent (one 64-byte fetch tests
// both children).  Child refs: >= 0 internal node (global index); < 0 leaf,
// ~ref = sorted triangle position.
struct alignas(16) Node2 {
  float4 a;  // c0.lo.x c0.hi.x c0.lo.y c0.hi.y
  float4 b;  // c1.lo.x c1.hi.x c1.lo.y c1.hi.y
  float4 c;  // c0.lo.z c0.hi.z c1.lo.z c1.hi.z
  int4 d;    // child0, child1, parent (global, -1 root), scene
};

// Bit pattern of a child box word not yet written by the refit: a NaN whose
// payload min/max of vertex coordinates never produce (they return an input
// or the canonical NaN).
constexpr int32_t kBoxUnset = (int32_t)0xFFC0DEADu;

// Wide node of width W, structure of arrays inside the record (7 / 14
// 16-byte loads per visit).  Child refs: >= 0 wide node index; < 0 leaf range
// ~(first << 3 | (count - 1)) over sorted triangles; kEmptyChild = unused
// slot.  (8-bit quantised child boxes, 64 / 96 bytes, were measured too: no
// gain on incoherent rays, 35 % slower on coherent camera rays, where the
// decode's integer work dominates.)
constexpr int32_t kEmptyChild = 0x7FFFFFFF;
template <int W>
struct alignas(16) NodeW {
  float lox[W], hix[W], loy[W], hiy[W], loz[W], hiz[W];
  int32_t child[W];
};
static_assert(sizeof(NodeW<4>) == 112, "NodeW<4> layout");
static_assert(sizeof(NodeW<8>) == 224, "NodeW<8> layout");

// Sorted triangle record: v0.xyz + original (scene-local) id, v1, v2.
struct alignas(16) TriRec {
  float4 p0, p1, p2;
};

}  // namespace flg

struct flg_ctx_t {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host staging overlap
  bool own_stream = false;
  uint32_t *d_err = nullptr;   // device error word
  uint32_t *h_err = nullptr;   // pinned mirror
  uint32_t spin_limit = 1u << 24;
  bool capturing = false;
  int num_sms = 0;
  int64_t launches = 0;  // kernels launched through this context
  std::string last_error;
  // Traversal scratch: rays whose stack overflowed (retried with a deep
  // stack), the persistent kernels' work counter, per-call ray offsets.
  int64_t *d_ovf = nullptr;
  uint32_t *d_ovf_count = nullptr;
  int64_t ovf_cap = 0;
  unsigned long long *d_work = nullptr;  // [0] persistent ray counter
  int64_t *d_ray_off = nullptr;          // device copy of batched ray offsets
  int64_t ray_off_cap = 0;
  std::vector<int64_t> ray_off_h;        // host copy of what d_ray_off holds
  // Device staging buffers for flg_trace_closest_host (grown on demand).
  void *stage = nullptr;
  size_t stage_bytes = 0;
  // Wavefront queues of flg_pathtrace (grown on demand).
  void *pt_buf = nullptr;
  size_t pt_bytes = 0;
  // Ray-sort scratch of trace_enqueue (grown on demand).
  void *rs_buf = nullptr;
  size_t rs_bytes = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // Stage timing (flg_ctx_set_stage_timing): an event recorded at the end of
  // every stage of builds and traces, named by the stage; pooled events.
  bool stage_timing = false;
  std::vector<cudaEvent_t> stage_pool;
  std::vector<std::pair<const char *, cudaEvent_t>> stage_marks;
};

struct flg_bvh_t {
  flg_ctx ctx = nullptr;
  int64_t n_tri = 0, n_vert = 0, n_nodes = 0;
  int32_t n_scenes = 0;
  const float *pos = nullptr;
  const int32_t *idx = nullptr;
  std::vector<int64_t> tri_off_h, node_off_h;
  int64_t *d_tri_off = nullptr, *d_node_off = nullptr;
  int32_t *d_root = nullptr;     // per scene: root ref (node index, ~leaf, or INT32_MIN)
  float *d_scene_box = nullptr;  // per scene: 6 floats (union of triangle boxes)
  // Sorted codes and order; internal node slots are numbered by sorted
  // triangle position (node_off == tri_off, the last slot of a scene unused).
  uint32_t *d_keys = nullptr;    // sorted Morton codes (after build)
  uint32_t *d_perm = nullptr;    // sorted position -> original global triangle
  uint32_t *d_keys_alt = nullptr, *d_vals_alt = nullptr;
  uint32_t *d_flags = nullptr;   // climb arrival counters (0 between builds)
  float4 *d_slots = nullptr;     // climb hand-over records, 2 per slot (unset between builds)
  uint32_t *d_dirty = nullptr;   // a climb gave up: reset flags and slots before the next
  flg::Node2 *d_nodes2 = nullptr;
  flg::TriRec *d_tris = nullptr;
  // Sort scratch.
  uint32_t *d_hist = nullptr;      // [passes][256] counts, then exclusive offsets
  uint32_t *d_lookback = nullptr;  // [passes][tiles][256]
  uint32_t *d_tile_ctr = nullptr;  // [passes]
  int32_t n_passes = 0, n_morton_passes = 0;
  int64_t n_tiles = 0;
  // Segmented sorts: first sort tile of every scene (n_scenes + 1), per-scene
  // digit counts [scene][pass][256] followed by the buckets' global starts.
  int32_t *d_tile_start = nullptr;
  uint32_t *d_shist = nullptr;
  std::vector<uint32_t> scene_hist_h;  // scene-digit histograms (host)
  // Wide layout.
  int32_t width = 2, leaf_size = 1;
  void *d_wide = nullptr;
  int64_t wide_cap = 0, wide_rec = 0;
  int32_t *d_wide_root = nullptr;  // per scene: wide root ref
  int32_t *d_wide_ctr = nullptr;   // [0] nodes allocated, [1..] queue sizes
  int2 *d_queue[2] = {nullptr, nullptr};
  int2 *d_queue_init = nullptr;
  int32_t n_wide_roots = 0;
  std::vector<void *> allocs;
  int64_t device_bytes = 0;
  bool keep_topology = true;
  // PLOC builds (builder == FLG_BUILDER_PLOC): the leaf range of every BVH2
  // node in the final (depth-first) triangle order, used by the collapse, and
  // the clustering scratch (ping-pong cluster arrays, scan buffers, queues).
  int32_t builder = 0;
  int32_t treelet_rounds = 3;  // FLG_BUILDER_TREELET: restructuring passes
  int32_t *d_rfirst = nullptr, *d_rcount = nullptr;
  float4 *d_cbox[2] = {nullptr, nullptr};  // 2 per cluster: lo, hi
  int32_t *d_cref[2] = {nullptr, nullptr}, *d_ccnt[2] = {nullptr, nullptr}, *d_cscene[2] = {nullptr, nullptr};
  int32_t *d_nn = nullptr, *d_valid = nullptr, *d_pos = nullptr, *d_bsum = nullptr, *d_mctr = nullptr;
  int32_t *d_newpos = nullptr, *d_lcount = nullptr;
  int2 *d_lq[2] = {nullptr, nullptr};
  int32_t n_nonempty = 0;
  // SAH builds (builder == FLG_BUILDER_SAH): per position, ping-pong
  // triangle boxes (2 float4), centroids (xyz + original index) and the
  // level-list index of the position's node; per level, the node list and
  // its 16 bucket records (8 words each); finished ranges, flag scan,
  // counters and the roots' list indices.
  int64_t sah_cap = 0, sah_fin_cap = 0;
  float4 *d_sbox[2] = {nullptr, nullptr}, *d_scen[2] = {nullptr, nullptr};
  int32_t *d_sseg[2] = {nullptr, nullptr};
  void *d_slist[2] = {nullptr, nullptr};
  uint32_t *d_sbins[2] = {nullptr, nullptr};
  int4 *d_sfin = nullptr;
  int32_t *d_sflag = nullptr, *d_sscan = nullptr, *d_ssum = nullptr, *d_sctr = nullptr, *d_sroot = nullptr;
  // Treelet restructuring (builder == FLG_BUILDER_TREELET): per node slot
  // children, parent, leaf count, first leaf, Karras slot (6 x int32), per
  // leaf parent and new position (2 x int32), arrival counters, costs and
  // boxes; the rewritten node records, triangle records and order.
  int32_t *d_tl_i32 = nullptr;
  uint32_t *d_tl_flag = nullptr;
  float *d_tl_cost = nullptr;
  float4 *d_tl_box = nullptr;
  flg::Node2 *d_tl_nodes = nullptr;
  flg::TriRec *d_tl_tris = nullptr;
  uint32_t *d_tl_perm = nullptr;
};

struct flg_grid_t {
  flg_ctx ctx = nullptr;
  const float *rho = nullptr;
  int32_t nx = 0, ny = 0, nz = 0;
  float lo[3], hi[3], scale[3];
  flg_medium medium{};
  float sigma_t = 0.0f;
  float *d_params = nullptr;  // [0] majorant, [1] 1/majorant
  // Sparse grids: brick table [bnz][bny][bnx] (slot or -1) over rho's bricks.
  const int32_t *bidx = nullptr;
  int32_t bnx = 0, bny = 0, bnz = 0;
  int64_t n_bricks = 0;
};

struct flg_graph_t {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace flg {

int set_error(flg_ctx ctx, int code, const char *fmt, ...);
int cuda_fail(flg_ctx ctx, cudaError_t e, const char *what);

#define FLG_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::flg::cuda_fail((ctx), e_, #call); \
  } while (0)

// Placed after every kernel launch: counts the launch on the context and
// turns a launch error into a status.
#define FLG_LAUNCH_CHECK(ctx, what)                                 \
  do {                                                              \
    ++(ctx)->launches;                                              \
    cudaError_t e_ = cudaGetLastError();                            \
    if (e_ != cudaSuccess) return ::flg::cuda_fail((ctx), e_, what); \
  } while (0)

// Stage timing: records an event named `stage` on `st` when the context's
// stage timing is on (never during a capture).  The time between two marks is
// the named stage's; a mark named "start" opens a new sequence.  At most
// kMaxStageMarks marks are kept between two reads.
constexpr size_t kMaxStageMarks = 4096;
inline void stage_mark(flg_ctx ctx, cudaStream_t st, const char *stage) {
  if (!ctx->stage_timing || ctx->capturing || ctx->stage_marks.size() >= kMaxStageMarks) return;
  const size_t k = ctx->stage_marks.size();
  if (k >= ctx->stage_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    ctx->stage_pool.push_back(e);
  }
  if (cudaEventRecord(ctx->stage_pool[k], st) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  ctx->stage_marks.emplace_back(stage, ctx->stage_pool[k]);
}

// Device allocation owned by a handle.
template <class T>
int halloc(flg_bvh b, T **p, size_t count) {
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(b->ctx, FLG_ERR_OOM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  b->allocs.push_back((void *)*p);
  b->device_bytes += (int64_t)bytes;
  return FLG_OK;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Launch-size helper: grid of `n` items, capped at `cap_blocks`.
inline unsigned grid_for(int64_t n, int threads, int64_t cap_blocks = 1 << 30) {
  int64_t g = ceil_div(n > 0 ? n : 1, threads);
  if (g > cap_blocks) g = cap_blocks;
  return (unsigned)g;
}

// Defined in the build / trace translation units.
int build_enqueue(flg_ctx ctx, flg_bvh b);
int collapse_reserve(flg_ctx ctx, flg_bvh b);
int collapse_enqueue(flg_ctx ctx, flg_bvh b, int width, int leaf_size);
int sort_enqueue(flg_ctx ctx, flg_bvh b);
int64_t sort_tiles(int64_t n);
int64_t sort_tile();  // pairs per sort tile
int sort_pairs_enqueue(flg_ctx ctx, cudaStream_t st, int64_t n, int passes, uint32_t *const keys[2],
                       uint32_t *const vals[2], uint32_t *hist, uint32_t *lookback, uint32_t *tile_ctr);
int ploc_reserve(flg_bvh b);
int ploc_build(flg_ctx ctx, flg_bvh b);
int sah_reserve(flg_bvh b);
int sah_build(flg_ctx ctx, flg_bvh b);
int treelet_reserve(flg_bvh b);
int treelet_build(flg_ctx ctx, flg_bvh b);
// Exclusive scan of int32 flags (ploc.cu): per-tile scans and tile sums
// (kFlagScanThreads threads, kFlagScanTile flags per tile), then a one-CTA
// (1024 threads) exclusive scan of the tile sums that also writes the total.
constexpr int kFlagScanThreads = 256;
constexpr int kFlagScanTile = 4096;
#ifdef __CUDACC__
__global__ void k_scan_tiles(const int32_t *in, int n, int32_t *out, int32_t *tsum);
__global__ void k_scan_sums(int32_t *tsum, int nt, int32_t *total_out);
#endif
int trace_enqueue(flg_ctx ctx, cudaStream_t st, int set, flg_bvh b, const flg_rays *rays, int64_t n,
                  const flg_trace_opts *opts, const int64_t *ray_off_dev, int n_scenes, flg_hits *hits,
                  uint8_t *occ);

}  // namespace flg
