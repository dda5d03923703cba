// build.cu — Karras LBVH construction on the GPU (RadixBVHBuilder::build,
// radix_bvh.cpp:18-24,32-200) for one scene or many scenes in one pass.
//
// Pipeline (one CUDA stream, no host synchronisation, no allocation in
// flg_bvh_rebuild so the whole build can be captured in a CUDA graph):
//   1. k_scene_bounds  union of triangle AABBs per scene (prestage reduce,
//                      radix_bvh.cpp:49-60), block reduce + ordered atomics
//   2. k_morton_hist   30-bit Morton code per triangle (radix_bvh.cpp:63-73)
//                      plus the digit histograms of every sort pass
//   3. sort            onesweep radix sort (sort.cu)
//   4. k_karras        one thread per internal node: direction, range, split
//                      (radix_bvh.cpp:118-161) and child/parent links
//   5. k_refit         lanes over sorted leaves: gather the triangle into the
//                      sorted triangle array, then climb with per-node
//                      arrival counters (radix_bvh.cpp:163-199); each child
//                      box is written once, into its parent's record, and
//                      the second arrival polls for its sibling's box (no
//                      fence per level)
//   6. (optional) collapse to 4- or 8-wide nodes (collapse.cu)
#include <cuda/atomic>

#include <algorithm>
#include <climits>
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace flg {

int64_t sort_tiles(int64_t n);

// Ordered float atomics (IEEE order on the sign/magnitude encoding).
__device__ __forceinline__ void atomic_min_f(float *a, float v) {
  if (v >= 0.0f) atomicMin((int *)a, __float_as_int(v));
  else atomicMax((unsigned int *)a, __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
  if (v >= 0.0f) atomicMax((int *)a, __float_as_int(v));
  else atomicMin((unsigned int *)a, __float_as_uint(v));
}

__global__ void k_init_boxes(float *box, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    for (int k = 0; k < 3; ++k) {
      box[6 * i + k] = 3.402823466e+38f;
      box[6 * i + 3 + k] = -3.402823466e+38f;
    }
  }
}

constexpr int kBoundsThreads = 256;
constexpr int kBoundsChunk = 8192;

__global__ void __launch_bounds__(kBoundsThreads)
    k_scene_bounds(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
                   const int64_t *__restrict__ tri_off, int n_scenes, float *scene_box) {
  __shared__ float s_red[6][kBoundsThreads / 32];
  const int64_t start = (int64_t)blockIdx.x * kBoundsChunk;
  const int64_t end = min(start + (int64_t)kBoundsChunk, n_tri);
  if (start >= end) return;
  const int s0 = find_segment(tri_off, n_scenes, start);
  const int s1 = find_segment(tri_off, n_scenes, end - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = s0; s <= s1; ++s) {
    int64_t a0 = max(start, tri_off[s]), a1 = min(end, tri_off[s + 1]);
    float v[6] = {3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f,
                  -3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f};
    for (int64_t t = a0 + threadIdx.x; t < a1; t += kBoundsThreads) {
      float3 p0, p1, p2;
      tri_verts(pos, idx, t, p0, p1, p2);
      float lo[3], hi[3];
      tri_box(p0, p1, p2, lo, hi);
      for (int k = 0; k < 3; ++k) {
        v[k] = fminf(v[k], lo[k]);
        v[3 + k] = fmaxf(v[3 + k], hi[k]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        v[k] = fminf(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
        v[3 + k] = fmaxf(v[3 + k], __shfl_xor_sync(0xFFFFFFFFu, v[3 + k], o));
      }
    }
    if (lane == 0)
      for (int k = 0; k < 6; ++k) s_red[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
      int k = threadIdx.x;
      float r = s_red[k][0];
      for (int w = 1; w < kBoundsThreads / 32; ++w) r = k < 3 ? fminf(r, s_red[k][w]) : fmaxf(r, s_red[k][w]);
      if (a1 > a0) {
        if (k < 3) atomic_min_f(&scene_box[6 * s + k], r);
        else atomic_max_f(&scene_box[6 * s + k], r);
      }
    }
    __syncthreads();
  }
}

// Morton code of every triangle against its scene box (radix_bvh.cpp:63-73,
// experimental_utils.hpp:33-45) and the per-pass digit histograms.
__global__ void __launch_bounds__(256)
    k_morton_hist(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
                  const int64_t *__restrict__ tri_off, int n_scenes, const float *__restrict__ scene_box,
                  uint32_t *__restrict__ keys, uint32_t *__restrict__ hist, int n_hist_passes) {
  __shared__ uint32_t s_hist[4][256];
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
  __syncthreads();
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_tri;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, t);
    float3 p0, p1, p2;
    tri_verts(pos, idx, t, p0, p1, p2);
    float lo[3], hi[3];
    tri_box(p0, p1, p2, lo, hi);
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float slo = scene_box[6 * s + k], shi = scene_box[6 * s + 3 + k];
      float e = shi - slo;
      float c = __fdiv_rn(lo[k] + hi[k], 2.0f);
      float nrm = e == 0.0f ? 0.0f : __fdiv_rn(c - slo, e);
      q[k] = to_u32(nrm * 1024.0f);
    }
    uint32_t code = (left_shift3(q[2]) << 2) | (left_shift3(q[1]) << 1) | left_shift3(q[0]);
    keys[t] = code;
    for (int p = 0; p < n_hist_passes; ++p) atomicAdd(&s_hist[p][(code >> (8 * p)) & 0xFFu], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_hist_passes * 256; i += blockDim.x) {
    uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

// delta(i, j) of radix_bvh.hpp:68-74 on a scene's sorted codes.
struct Delta {
  const uint32_t *code;
  int n;
  __device__ __forceinline__ int operator()(int i, int j) const {
    if (j < 0 || j >= n) return -1;
    uint32_t a = code[i], b = code[j];
    if (a == b) return __clz((uint32_t)(i ^ j)) + 32;
    return __clz(a ^ b);
  }
};

__device__ __forceinline__ int next2pow(int l) {
  return l <= 1 ? 1 : (int)(1u << (32 - __clz((uint32_t)(l - 1))));
}

__global__ void __launch_bounds__(256)
    k_karras(const uint32_t *__restrict__ keys, const int64_t *__restrict__ tri_off,
             const int64_t *__restrict__ node_off, int n_scenes, int64_t n_nodes,
             int32_t *__restrict__ split_o, uint8_t *__restrict__ leaf_o, int32_t *__restrict__ range_o,
             int32_t *__restrict__ parent_o, int32_t *__restrict__ leaf_parent_o, Node2 *__restrict__ nodes,
             uint32_t *__restrict__ flags_o) {
  for (int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < n_nodes;
       gi += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(node_off, n_scenes, gi);
    const int64_t toff = tri_off[s], noff = node_off[s];
    const int n = (int)(tri_off[s + 1] - toff);
    const int i = (int)(gi - noff);
    Delta delta{keys + toff, n};
    // radix_bvh.cpp:119-150
    int dd = delta(i, i + 1) - delta(i, i - 1);
    int d = dd == 0 ? 0 : (dd > 0 ? 1 : -1);
    int delta_min = delta(i, i - d);
    int l_max = 2;
    while (delta(i, i + l_max * d) > delta_min) l_max <<= 1;
    int l = 0;
    for (int t = l_max >> 1; t >= 1; t >>= 1)
      if (delta(i, i + (l + t) * d) > delta_min) l += t;
    int j = i + l * d;
    int delta_node = delta(i, j);
    int sp = 0;
    for (int t = next2pow(l); t >= 1; t >>= 1)
      if (delta(i, i + (sp + t) * d) > delta_node) sp += t;
    int split = i + sp * d + min(d, 0);
    uint8_t lf = 0;
    if (min(i, j) == split) lf |= 1;
    if (max(i, j) == split + 1) lf |= 2;
    split_o[gi] = split;
    leaf_o[gi] = lf;
    range_o[gi] = j;
    // Parent links carry the child's side in bit 0 (0: the child at split,
    // 1: the child at split + 1), so the refit climb needs one load a level.
    int c0, c1;
    if (lf & 1) {
      c0 = ~(int)(toff + split);
      leaf_parent_o[toff + split] = i << 1;
    } else {
      c0 = (int)(noff + split);
      parent_o[noff + split] = i << 1;
      nodes[noff + split].d.z = (int)gi;
    }
    if (lf & 2) {
      c1 = ~(int)(toff + split + 1);
      leaf_parent_o[toff + split + 1] = (i << 1) | 1;
    } else {
      c1 = (int)(noff + split + 1);
      parent_o[noff + split + 1] = (i << 1) | 1;
      nodes[noff + split + 1].d.z = (int)gi;
    }
    // Child boxes start as the "not yet written" pattern the refit polls on.
    const float u = __int_as_float(kBoxUnset);
    float4 *f4 = (float4 *)(nodes + gi);
    f4[0] = f4[1] = f4[2] = make_float4(u, u, u, u);
    nodes[gi].d.x = c0;
    nodes[gi].d.y = c1;
    nodes[gi].d.w = s;
    flags_o[gi] = 0u;
    if (i == 0) {
      nodes[gi].d.z = -1;
      parent_o[gi] = 0;
    }
  }
}

// Child box of side s lives in float4 s (x/y lo-hi) and float2 s of the third
// float4 (z lo-hi).  Stores and polls are relaxed device-scope accesses: the
// climb orders nothing else through them, so no fence is needed.
__device__ __forceinline__ void store_child_box(Node2 *nd, int side, const float *lo, const float *hi) {
  float4 *f4 = (float4 *)nd;
  float2 *f2 = (float2 *)(f4 + 2);
  asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(f4 + side), "f"(lo[0]), "f"(hi[0]),
               "f"(lo[1]), "f"(hi[1])
               : "memory");
  asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(f2 + side), "f"(lo[2]), "f"(hi[2]) : "memory");
}

// One relaxed read of a child box; true when none of its six words holds
// kBoxUnset any more.  Each word is written once, so per-word coherence is
// all the polling relies on (no fence orders the sibling's stores).
__device__ __forceinline__ bool read_child_box(const Node2 *nd, int side, float *lo, float *hi) {
  const float4 *f4 = (const float4 *)nd;
  const float2 *f2 = (const float2 *)(f4 + 2);
  float a0, a1, a2, a3, z0, z1;
  asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(a0), "=f"(a1), "=f"(a2), "=f"(a3)
               : "l"(f4 + side)
               : "memory");
  asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(z0), "=f"(z1) : "l"(f2 + side) : "memory");
  lo[0] = a0; hi[0] = a1; lo[1] = a2; hi[1] = a3; lo[2] = z0; hi[2] = z1;
  return __float_as_int(a0) != kBoxUnset && __float_as_int(a1) != kBoxUnset && __float_as_int(a2) != kBoxUnset &&
         __float_as_int(a3) != kBoxUnset && __float_as_int(z0) != kBoxUnset && __float_as_int(z1) != kBoxUnset;
}

// Polls until read_child_box succeeds; false after `limit` polls.
__device__ __forceinline__ bool wait_child_box(const Node2 *nd, int side, float *lo, float *hi, uint32_t limit) {
  for (uint32_t spins = 0;; ++spins) {
    if (read_child_box(nd, side, lo, hi)) return true;
    if (spins >= limit) return false;
    if (spins > 16) __nanosleep(32);
  }
}

// Bottom-up refit (radix_bvh.cpp:163-199).  Each warp owns a contiguous
// chunk of sorted leaves.  A lane gathers its leaf's triangle into the sorted
// triangle array, then climbs: at every node it writes its own box into the
// parent's record and counts its arrival; the first arrival stops, the second
// waits for the sibling's box, merges and goes on up.  Lanes that stopped
// take new leaves together, once half the warp is idle, so that the gathers
// of a refill run side by side on consecutive leaves.
constexpr int kRefitRefill = 16;

__global__ void __launch_bounds__(256)
    k_refit(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
            const int64_t *__restrict__ tri_off, const int64_t *__restrict__ node_off, int n_scenes,
            const uint32_t *__restrict__ perm, const int32_t *__restrict__ parent,
            const int32_t *__restrict__ leaf_parent, Node2 *nodes, uint32_t *flags, TriRec *__restrict__ tris,
            uint32_t spin_limit, uint32_t *err) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t n_warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t chunk = (n_tri + n_warps - 1) / n_warps;
  int64_t next = warp * chunk;
  const int64_t end = min(next + chunk, n_tri);
  bool climbing = false;
  int cur = 0, side = 0, n = 0, depth = 0;
  int64_t noff = 0;
  float lo[3], hi[3];
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !climbing);
    const int nidle = __popc(idle);
    if (next < end && nidle >= kRefitRefill) {
      const int64_t leaf = next + __popc(idle & lt);
      next += nidle;
      if (!climbing && leaf < end) {
        const int s = find_segment(tri_off, n_scenes, leaf);
        const int64_t toff = tri_off[s];
        noff = node_off[s];
        n = (int)(tri_off[s + 1] - toff);
        const int64_t orig = perm[leaf];
        // A sort that timed out leaves unspecified slots: never follow them.
        if (orig < toff || orig >= toff + n) {
          atomicOr(err, kErrTimeout);
        } else {
          float3 p0, p1, p2;
          tri_verts(pos, idx, orig, p0, p1, p2);
          TriRec r;
          r.p0 = make_float4(p0.x, p0.y, p0.z, __int_as_float((int)(orig - toff)));
          r.p1 = make_float4(p1.x, p1.y, p1.z, 0.0f);
          r.p2 = make_float4(p2.x, p2.y, p2.z, 0.0f);
          tris[leaf] = r;
          if (n >= 2) {
            tri_box(p0, p1, p2, lo, hi);
            const int ps = leaf_parent[leaf];
            cur = ps >> 1;
            side = ps & 1;
            depth = 0;
            climbing = true;
          }
        }
      }
    } else if (nidle == 32) {
      break;  // every leaf of the chunk taken and every climb finished
    }
    if (!climbing) continue;
    // A valid Karras tree is at most 30 + 32 levels deep; the bound only
    // matters if the inputs were corrupted by an earlier timed-out wait.
    if (depth > 96 || cur < 0 || cur >= n - 1) {
      atomicOr(err, kErrTimeout);
      climbing = false;
      continue;
    }
    Node2 *nd = nodes + noff + cur;
    store_child_box(nd, side, lo, hi);
    const int ps = parent[noff + cur];  // in flight with the arrival count
    if (atomicAdd(flags + noff + cur, 1u) == 0u) {
      climbing = false;
      continue;
    }
    float olo[3], ohi[3];
    if (!wait_child_box(nd, side ^ 1, olo, ohi, spin_limit)) {
      atomicOr(err, kErrTimeout);
      climbing = false;
      continue;
    }
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], olo[k]);
      hi[k] = fmaxf(hi[k], ohi[k]);
    }
    if (cur == 0) {
      climbing = false;
      continue;
    }
    cur = ps >> 1;
    side = ps & 1;
    ++depth;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

int build_enqueue(flg_ctx ctx, flg_bvh b) {
  cudaStream_t st = ctx->stream;
  const int64_t n = b->n_tri;
  if (n <= 0) return FLG_OK;
  const unsigned fill_grid = grid_for(b->n_scenes, 128);
  k_init_boxes<<<fill_grid, 128, 0, st>>>(b->d_scene_box, b->n_scenes);
  FLG_LAUNCH_CHECK(ctx, "k_init_boxes");
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_hist, 0, sizeof(uint32_t) * 256 * b->n_morton_passes, st));
  if (b->n_passes > b->n_morton_passes)
    FLG_CUDA(ctx, cudaMemcpyAsync(b->d_hist + 256 * b->n_morton_passes,
                                  b->d_hist + 512 * b->n_passes,
                                  sizeof(uint32_t) * 256 * (b->n_passes - b->n_morton_passes),
                                  cudaMemcpyDeviceToDevice, st));
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_lookback, 0,
                                sizeof(uint32_t) * 256 * (size_t)b->n_tiles * b->n_passes, st));
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_tile_ctr, 0, sizeof(uint32_t) * b->n_passes, st));

  k_scene_bounds<<<grid_for(n, kBoundsChunk), kBoundsThreads, 0, st>>>(b->pos, b->idx, n, b->d_tri_off,
                                                                     b->n_scenes, b->d_scene_box);
  FLG_LAUNCH_CHECK(ctx, "k_scene_bounds");
  uint32_t *morton_out = (b->n_passes % 2 == 0) ? b->d_keys : b->d_keys_alt;
  const unsigned g_elem = grid_for(n, 256, (int64_t)ctx->num_sms * 8);
  k_morton_hist<<<g_elem, 256, 0, st>>>(b->pos, b->idx, n, b->d_tri_off, b->n_scenes, b->d_scene_box,
                                        morton_out, b->d_hist, b->n_morton_passes);
  FLG_LAUNCH_CHECK(ctx, "k_morton_hist");
  int rc = sort_enqueue(ctx, b);
  if (rc) return rc;
  if (b->builder == FLG_BUILDER_PLOC) {
    rc = ploc_build(ctx, b);
    if (rc) return rc;
    if (b->width > 2) return collapse_enqueue(ctx, b, b->width, b->leaf_size);
    return FLG_OK;
  }
  if (b->n_nodes > 0) {
    k_karras<<<grid_for(b->n_nodes, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(
        b->d_keys, b->d_tri_off, b->d_node_off, b->n_scenes, b->n_nodes, b->d_split, b->d_leaf,
        b->d_range_j, b->d_parent, b->d_leaf_parent, b->d_nodes2, b->d_flags);
    FLG_LAUNCH_CHECK(ctx, "k_karras");
  }
  // Lanes take their next leaf as soon as they stop climbing, so one wave
  // of resident CTAs balances better than more CTAs than fit.
  static const int refit_per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_refit, 256, 0) != cudaSuccess || v < 1) v = 1;
    return v;
  }();
  k_refit<<<grid_for(n, 256, (int64_t)ctx->num_sms * refit_per_sm), 256, 0, st>>>(
      b->pos, b->idx, n, b->d_tri_off, b->d_node_off, b->n_scenes, b->d_perm, b->d_parent, b->d_leaf_parent,
      b->d_nodes2, b->d_flags, b->d_tris, ctx->spin_limit, ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_refit");
  if (b->width > 2) return collapse_enqueue(ctx, b, b->width, b->leaf_size);
  return FLG_OK;
}

static int bvh_create(flg_ctx ctx, const float *pos, const int32_t *idx, const int64_t *tri_off_host,
                      int32_t n_scenes, int64_t n_vert, const flg_build_opts *opts, flg_bvh *out) {
  if (!ctx || !out) return FLG_ERR_ARG;
  *out = nullptr;
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "build allocates; not allowed during capture");
  if (n_scenes < 1 || !tri_off_host) return set_error(ctx, FLG_ERR_ARG, "n_scenes must be >= 1");
  if (tri_off_host[0] != 0) return set_error(ctx, FLG_ERR_ARG, "tri_offsets[0] must be 0");
  for (int s = 0; s < n_scenes; ++s) {
    int64_t c = tri_off_host[s + 1] - tri_off_host[s];
    if (c < 0) return set_error(ctx, FLG_ERR_ARG, "tri_offsets must be non-decreasing");
    if (c > INT32_MAX) return set_error(ctx, FLG_ERR_ARG, "scene %d has more than 2^31-1 triangles", s);
  }
  const int64_t n = tri_off_host[n_scenes];
  if (n > ((int64_t)1 << 28))
    return set_error(ctx, FLG_ERR_UNSUPPORTED, "at most 2^28 triangles per build (got %lld)", (long long)n);
  if (n > 0 && !pos) return set_error(ctx, FLG_ERR_ARG, "pos is NULL");
  if (!idx && n_vert != 3 * n) return set_error(ctx, FLG_ERR_ARG, "soup needs n_vert == 3*n_tri");
  int width = opts && opts->node_width ? opts->node_width : 4;
  int leaf_size = opts && opts->leaf_size ? opts->leaf_size : 1;
  if (width != 2 && width != 4 && width != 8) return set_error(ctx, FLG_ERR_ARG, "node_width must be 2, 4 or 8");
  if (leaf_size < 1 || leaf_size > 8) return set_error(ctx, FLG_ERR_ARG, "leaf_size must be in [1, 8]");
  const int builder = opts ? opts->builder : FLG_BUILDER_LBVH;
  if (builder != FLG_BUILDER_LBVH && builder != FLG_BUILDER_PLOC)
    return set_error(ctx, FLG_ERR_ARG, "builder must be FLG_BUILDER_LBVH or FLG_BUILDER_PLOC");

  flg_bvh b = new flg_bvh_t();
  b->ctx = ctx;
  b->n_tri = n;
  b->n_vert = n_vert;
  b->n_scenes = n_scenes;
  b->pos = pos;
  b->idx = idx;
  b->width = width;
  b->leaf_size = leaf_size;
  b->keep_topology = opts ? opts->keep_topology != 0 : true;
  b->builder = builder;
  b->tri_off_h.assign(tri_off_host, tri_off_host + n_scenes + 1);
  b->node_off_h.resize(n_scenes + 1);
  b->node_off_h[0] = 0;
  std::vector<int32_t> root(n_scenes);
  for (int s = 0; s < n_scenes; ++s) {
    int64_t c = tri_off_host[s + 1] - tri_off_host[s];
    b->node_off_h[s + 1] = b->node_off_h[s] + (c >= 2 ? c - 1 : 0);
    root[s] = c >= 2 ? (int32_t)b->node_off_h[s] : c == 1 ? ~(int32_t)tri_off_host[s] : INT32_MIN;
  }
  b->n_nodes = b->node_off_h[n_scenes];
  for (int s = 0; s < n_scenes; ++s) b->n_nonempty += tri_off_host[s + 1] > tri_off_host[s] ? 1 : 0;
  b->n_morton_passes = 4;
  int scene_passes = 0;
  if (n_scenes > 1) scene_passes = n_scenes <= 256 ? 1 : n_scenes <= 65536 ? 2 : 3;
  b->n_passes = b->n_morton_passes + scene_passes;
  b->n_tiles = sort_tiles(n);

  int rc = FLG_OK;
  auto A = [&](auto **p, size_t c) {
    if (rc == FLG_OK) rc = halloc(b, p, c);
  };
  A(&b->d_tri_off, n_scenes + 1);
  A(&b->d_node_off, n_scenes + 1);
  A(&b->d_root, n_scenes);
  A(&b->d_scene_box, 6 * (size_t)n_scenes);
  A(&b->d_keys, n);
  A(&b->d_perm, n);
  A(&b->d_keys_alt, n);
  A(&b->d_vals_alt, n);
  A(&b->d_split, b->n_nodes);
  A(&b->d_leaf, b->n_nodes);
  A(&b->d_range_j, b->n_nodes);
  A(&b->d_parent, b->n_nodes);
  A(&b->d_leaf_parent, n);
  A(&b->d_flags, b->n_nodes);
  A(&b->d_nodes2, b->n_nodes);
  A(&b->d_tris, n);
  // hist: [passes][256] counts, [passes][256] offsets, [passes][256] static scene counts
  A(&b->d_hist, 3 * 256 * (size_t)b->n_passes);
  A(&b->d_lookback, 256 * (size_t)b->n_tiles * b->n_passes);
  A(&b->d_tile_ctr, b->n_passes);
  if (rc == FLG_OK && builder == FLG_BUILDER_PLOC) rc = ploc_reserve(b);
  if (rc) {
    flg_bvh_destroy(b);
    return rc;
  }
  // Scene-digit histograms are fixed by the offsets.
  std::vector<uint32_t> sh(256 * (size_t)b->n_passes, 0u);
  for (int p = b->n_morton_passes; p < b->n_passes; ++p) {
    int shift = 8 * (p - b->n_morton_passes);
    for (int s = 0; s < n_scenes; ++s)
      sh[256 * (size_t)p + ((s >> shift) & 0xFF)] += (uint32_t)(tri_off_host[s + 1] - tri_off_host[s]);
  }
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(b->d_tri_off, tri_off_host, sizeof(int64_t) * (n_scenes + 1),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_node_off, b->node_off_h.data(), sizeof(int64_t) * (n_scenes + 1),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_root, root.data(), sizeof(int32_t) * n_scenes, cudaMemcpyHostToDevice, st);
  // Static scene counts live after counts and offsets; build_enqueue copies
  // the scene passes' part into place each build.
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_hist + 512 * (size_t)b->n_passes, sh.data() + 256 * b->n_morton_passes,
                        sizeof(uint32_t) * 256 * (b->n_passes - b->n_morton_passes), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors go out of scope
  if (e != cudaSuccess) {
    rc = cuda_fail(ctx, e, "bvh upload");
    flg_bvh_destroy(b);
    return rc;
  }
  if (width > 2) {
    rc = collapse_reserve(ctx, b);
    if (rc) {
      flg_bvh_destroy(b);
      return rc;
    }
  }
  rc = build_enqueue(ctx, b);
  if (rc) {
    flg_bvh_destroy(b);
    return rc;
  }
  *out = b;
  return FLG_OK;
}

}  // namespace flg

using namespace flg;

FLG_API int flg_bvh_build(flg_ctx ctx, const float *pos, const int32_t *idx, int64_t n_tri, int64_t n_vert,
                          const flg_build_opts *opts, flg_bvh *out) {
  if (n_tri < 0) return ctx ? set_error(ctx, FLG_ERR_ARG, "n_tri < 0") : FLG_ERR_ARG;
  int64_t off[2] = {0, n_tri};
  return bvh_create(ctx, pos, idx, off, 1, n_vert, opts, out);
}

FLG_API int flg_bvh_build_batched(flg_ctx ctx, const float *pos, const int32_t *idx,
                                  const int64_t *tri_offsets_host, int32_t n_scenes, int64_t n_vert,
                                  const flg_build_opts *opts, flg_bvh *out) {
  return bvh_create(ctx, pos, idx, tri_offsets_host, n_scenes, n_vert, opts, out);
}

FLG_API int flg_bvh_rebuild(flg_ctx ctx, flg_bvh bvh, const float *pos) {
  if (!ctx || !bvh) return FLG_ERR_ARG;
  if (bvh->n_tri > 0 && !pos) return set_error(ctx, FLG_ERR_ARG, "pos is NULL");
  bvh->pos = pos;
  return build_enqueue(ctx, bvh);
}

FLG_API int flg_bvh_destroy(flg_bvh bvh) {
  if (!bvh) return FLG_OK;
  for (void *p : bvh->allocs) cudaFree(p);
  delete bvh;
  return FLG_OK;
}

FLG_API int flg_bvh_info_get(flg_bvh bvh, flg_bvh_info *out) {
  if (!bvh || !out) return FLG_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  out->n_tri = bvh->n_tri;
  out->n_scenes = bvh->n_scenes;
  out->node_width = bvh->width;
  out->device_bytes = bvh->device_bytes;
  if (bvh->width > 2 && bvh->d_wide_ctr) {
    int32_t c = 0;
    if (cudaMemcpyAsync(&c, bvh->d_wide_ctr, sizeof(int32_t), cudaMemcpyDeviceToHost, bvh->ctx->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(bvh->ctx->stream) != cudaSuccess)
      return cuda_fail(bvh->ctx, cudaGetLastError(), "info");
    out->n_wide_nodes = c;
  }
  if (bvh->n_tri > 0) {
    cudaError_t e = cudaMemcpyAsync(out->bound, bvh->d_scene_box, 6 * sizeof(float), cudaMemcpyDeviceToHost,
                                    bvh->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(bvh->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(bvh->ctx, e, "info");
  }
  return FLG_OK;
}

FLG_API int flg_bvh_download(flg_bvh bvh, int32_t scene, flg_bvh_topology *t) {
  if (!bvh || !t) return FLG_ERR_ARG;
  flg_ctx ctx = bvh->ctx;
  if (bvh->builder != FLG_BUILDER_LBVH)
    return set_error(ctx, FLG_ERR_UNSUPPORTED, "only LBVH handles keep the Karras arrays");
  if (scene < 0 || scene >= bvh->n_scenes) return set_error(ctx, FLG_ERR_ARG, "scene out of range");
  cudaStream_t st = ctx->stream;
  const int64_t toff = bvh->tri_off_h[scene], noff = bvh->node_off_h[scene];
  const int64_t n = bvh->tri_off_h[scene + 1] - toff;
  const int64_t m = bvh->node_off_h[scene + 1] - noff;
  cudaError_t e = cudaStreamSynchronize(st);
  auto D = [&](void *dst, const void *src, size_t bytes) {
    if (e == cudaSuccess && dst && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
  };
  D(t->morton, bvh->d_keys + toff, sizeof(uint32_t) * n);
  D(t->perm, bvh->d_perm + toff, sizeof(int32_t) * n);
  D(t->split, bvh->d_split + noff, sizeof(int32_t) * m);
  D(t->leaf_flags, bvh->d_leaf + noff, sizeof(uint8_t) * m);
  D(t->range_j, bvh->d_range_j + noff, sizeof(int32_t) * m);
  D(t->parent, bvh->d_parent + noff, sizeof(int32_t) * m);
  D(t->leaf_parent, bvh->d_leaf_parent + toff, sizeof(int32_t) * n);
  D(t->scene_bound, bvh->d_scene_box + 6 * scene, sizeof(float) * 6);
  if (t->bounds && m > 0) {
    std::vector<Node2> nodes(m);
    D(nodes.data(), bvh->d_nodes2 + noff, sizeof(Node2) * m);
    for (int64_t i = 0; i < m && e == cudaSuccess; ++i) {
      const Node2 &q = nodes[i];
      float *o = t->bounds + 6 * i;
      o[0] = std::min(q.a.x, q.b.x);
      o[3] = std::max(q.a.y, q.b.y);
      o[1] = std::min(q.a.z, q.b.z);
      o[4] = std::max(q.a.w, q.b.w);
      o[2] = std::min(q.c.x, q.c.z);
      o[5] = std::max(q.c.y, q.c.w);
    }
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "download");
  if (t->perm)
    for (int64_t i = 0; i < n; ++i) t->perm[i] -= (int32_t)toff;
  // Device parent links carry the child's side in bit 0.
  if (t->parent)
    for (int64_t i = 0; i < m; ++i) t->parent[i] >>= 1;
  if (t->leaf_parent)
    for (int64_t i = 0; i < n; ++i) t->leaf_parent[i] >>= 1;
  if (t->leaf_parent && n == 1) t->leaf_parent[0] = -1;  // a lone leaf is the root
  return FLG_OK;
}
