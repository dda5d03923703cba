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
//   4. k_climb         the Karras tree (radix_bvh.cpp:118-161) and its refit
//                      (radix_bvh.cpp:163-199) in one bottom-up pass: lanes
//                      over sorted leaves gather the triangle into the sorted
//                      triangle array, then climb with per-node arrival
//                      counters, choosing each node's parent from the two
//                      neighbouring code deltas; the second arrival at a split
//                      polls for its sibling's hand-over record (no fence per
//                      level) and writes the finished node
//   6. (optional) collapse to 4- or 8-wide nodes (collapse.cu)
#include <cuda/atomic>

#include <algorithm>
#include <climits>
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace flg {

int64_t sort_tiles(int64_t n);

// Scene of triangle t given the scene `prev` of an earlier triangle of the
// same thread (-1: none yet): one binary search, then a forward walk.
__device__ __forceinline__ int scene_of(const int64_t *__restrict__ tri_off, int n_scenes, int64_t t, int prev) {
  if (prev < 0) return find_segment(tri_off, n_scenes, t);
  while (prev < n_scenes - 1 && tri_off[prev + 1] <= t) ++prev;
  return prev;
}

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

// Morton code of triangle t against its scene box sb (radix_bvh.cpp:63-73,
// experimental_utils.hpp:33-45).
__device__ __forceinline__ uint32_t morton_of(const float *__restrict__ pos, const int32_t *__restrict__ idx,
                                              int64_t t, const float *__restrict__ sb) {
  float3 p0, p1, p2;
  tri_verts(pos, idx, t, p0, p1, p2);
  float lo[3], hi[3];
  tri_box(p0, p1, p2, lo, hi);
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float slo = sb[k], shi = sb[3 + k];
    float e = shi - slo;
    float c = (lo[k] + hi[k]) * 0.5f;  // = the correctly rounded (lo + hi) / 2: 0.5 is exact
    float nrm = e == 0.0f ? 0.0f : __fdiv_rn(c - slo, e);
    q[k] = to_u32(nrm * 1024.0f);
  }
  return (left_shift3(q[2]) << 2) | (left_shift3(q[1]) << 1) | left_shift3(q[0]);
}

// Morton code of every triangle and the per-pass digit histograms.
__global__ void __launch_bounds__(256)
    k_morton_hist(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
                  const int64_t *__restrict__ tri_off, int n_scenes, const float *__restrict__ scene_box,
                  uint32_t *__restrict__ keys, uint32_t *__restrict__ hist, int n_hist_passes) {
  __shared__ uint32_t s_hist[4][256];
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
  __syncthreads();
  int s = -1;  // scene of t: t only grows, so it is searched once and then advanced
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_tri;
       t += (int64_t)gridDim.x * blockDim.x) {
    s = scene_of(tri_off, n_scenes, t, s);
    const uint32_t code = morton_of(pos, idx, t, scene_box + 6 * s);
    keys[t] = code;
    for (int p = 0; p < n_hist_passes; ++p) atomicAdd(&s_hist[p][(code >> (8 * p)) & 0xFFu], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_hist_passes * 256; i += blockDim.x) {
    uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

// Segmented sorts (batched builds whose scenes span several sort tiles): one
// block per sort tile, tiles aligned to scenes (tile_start[s] = first tile of
// scene s), so each block adds its codes' digit counts to its own scene's
// histograms hist[s][pass][digit].
__global__ void __launch_bounds__(256)
    k_morton_seg(const float *__restrict__ pos, const int32_t *__restrict__ idx, const int64_t *__restrict__ tri_off,
                 int n_scenes, const int32_t *__restrict__ tile_start, int tile, const float *__restrict__ scene_box,
                 uint32_t *__restrict__ keys, uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[4][256];
  __shared__ int s_scene;
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
  if (threadIdx.x == 0) s_scene = find_segment32(tile_start, n_scenes, (int32_t)blockIdx.x);
  __syncthreads();
  const int s = s_scene;
  const int64_t base = tri_off[s] + (int64_t)(blockIdx.x - tile_start[s]) * tile;
  const int64_t end = min(base + tile, tri_off[s + 1]);
  const float *sb = scene_box + 6 * s;
  for (int64_t t = base + threadIdx.x; t < end; t += blockDim.x) {
    const uint32_t code = morton_of(pos, idx, t, sb);
    keys[t] = code;
#pragma unroll
    for (int p = 0; p < 4; ++p) atomicAdd(&s_hist[p][(code >> (8 * p)) & 0xFFu], 1u);
  }
  __syncthreads();
  uint32_t *h = hist + (size_t)s * 4 * 256;
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
    const uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(&h[i], c);
  }
}

// Exclusive scan of each scene's digit counts per pass, offset by the
// scene's first position: the global start of every (scene, pass, digit)
// bucket.  One block of 256 threads per (scene, pass).
__global__ void k_scan_seg(const uint32_t *__restrict__ hist, const int64_t *__restrict__ tri_off,
                           uint32_t *__restrict__ off) {
  __shared__ uint32_t s_w[8];
  const int sp = blockIdx.x, d = threadIdx.x, lane = d & 31, warp = d >> 5;
  const uint32_t c = hist[(size_t)sp * 256 + d];
  uint32_t x = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < warp; ++w) pre += s_w[w];
  off[(size_t)sp * 256 + d] = (uint32_t)tri_off[sp / 4] + pre + x - c;
}

// delta of radix_bvh.hpp:68-74 between neighbouring sorted positions i and
// i + 1 of a scene (codes a, b): the common prefix length of the codes, or
// 32 + that of the positions when the codes are equal.  These are the common
// prefixes of the distinct strings (code, position), so the Karras tree is
// the binary radix tree over them.
__device__ __forceinline__ int delta_next(uint32_t a, uint32_t b, int i) {
  return a == b ? __clz((uint32_t)(i ^ (i + 1))) + 32 : __clz(a ^ b);
}

// Side of node [l, r] of a scene of n sorted codes under its parent: 0 when
// the parent splits at r (the node is a left child), 1 when it splits at l - 1.
__device__ __forceinline__ int parent_side(const uint32_t *__restrict__ code, uint32_t key_l, uint32_t key_r, int l,
                                           int r, int n) {
  const int dr = r < n - 1 ? delta_next(key_r, code[r + 1], r) : -1;
  const int dl = l > 0 ? delta_next(code[l - 1], key_l, l - 1) : -1;
  return dr > dl ? 0 : 1;
}

// The climb's hand-over record of an internal node slot: the first child to
// arrive leaves its box, the far end of its range and the code there; the
// second reads it and writes the unset pattern back, so every slot is unset
// again when a build ends (no clearing pass).  Words: lo.xyz, end | hi.xyz,
// code; kBoxUnset is never a box word (min/max of coordinates), a range end
// (0 .. 2^28) or a 30-bit code.
__device__ __forceinline__ void slot_store(float4 *slot, const float *lo, const float *hi, int end,
                                           uint32_t code) {
  asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(slot), "f"(lo[0]), "f"(lo[1]),
               "f"(lo[2]), "f"(__int_as_float(end))
               : "memory");
  asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(slot + 1), "f"(hi[0]), "f"(hi[1]),
               "f"(hi[2]), "f"(__uint_as_float(code))
               : "memory");
}

// Polls the slot until none of its eight words is unset (per-word coherence
// of relaxed accesses is all this relies on: each word is written once per
// build), then resets it.  False after `limit` polls.
__device__ __forceinline__ bool slot_take(float4 *slot, float *lo, float *hi, int &end, uint32_t &code,
                                          uint32_t limit) {
  for (uint32_t spins = 0;; ++spins) {
    float a0, a1, a2, a3, b0, b1, b2, b3;
    asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(a0), "=f"(a1), "=f"(a2), "=f"(a3)
                 : "l"(slot)
                 : "memory");
    asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(b0), "=f"(b1), "=f"(b2), "=f"(b3)
                 : "l"(slot + 1)
                 : "memory");
    const bool ready = __float_as_int(a0) != kBoxUnset && __float_as_int(a1) != kBoxUnset &&
                       __float_as_int(a2) != kBoxUnset && __float_as_int(a3) != kBoxUnset &&
                       __float_as_int(b0) != kBoxUnset && __float_as_int(b1) != kBoxUnset &&
                       __float_as_int(b2) != kBoxUnset && __float_as_int(b3) != kBoxUnset;
    if (ready) {
      lo[0] = a0; lo[1] = a1; lo[2] = a2; end = __float_as_int(a3);
      hi[0] = b0; hi[1] = b1; hi[2] = b2; code = __float_as_uint(b3);
      const float u = __int_as_float(kBoxUnset);
      asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %1, %1, %1};" ::"l"(slot), "f"(u) : "memory");
      asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %1, %1, %1};" ::"l"(slot + 1), "f"(u) : "memory");
      return true;
    }
    if (spins >= limit) return false;
    if (spins > 16) __nanosleep(32);
  }
}

// Sets every climb slot to the unset pattern and every arrival counter to 0
// (at allocation, and before a build that follows one whose climb gave up).
__global__ void k_climb_reset(float4 *slots, uint32_t *flags, int64_t n, const uint32_t *dirty) {
  if (dirty && *dirty == 0u) return;
  const float u = __int_as_float(kBoxUnset);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    slots[2 * i] = slots[2 * i + 1] = make_float4(u, u, u, u);
    flags[i] = 0u;
  }
}

__global__ void k_climb_clean(uint32_t *dirty) { *dirty = 0u; }

// Karras tree construction fused with the bottom-up refit (radix_bvh.cpp:
// 118-199), built from the leaves up (Apetrei 2014): a node covering sorted
// positions [l, r] of its scene is the left child of the node that splits at
// r when delta(r, r+1) > delta(l-1, l), else the right child of the node that
// splits at l - 1 (one of the two is the parent's split; the other lies
// outside the parent's range and belongs to an ancestor, whose common prefix
// is strictly shorter).  Karras numbering follows: a left child's index is its
// right end, a right child's its left end, the root's 0 — so the second child
// to arrive at a split knows the finished node's index as soon as it has
// chosen that node's parent, and writes the whole Node2 there: both child
// boxes, the child refs (split and split + 1) and the node's range.  Internal
// node slots are numbered by sorted triangle position (node_off == tri_off),
// so a child ref names its range boundary directly.
//
// Each warp owns a contiguous chunk of sorted leaves.  A lane gathers its
// leaf's triangle into the sorted triangle array, then climbs; the first
// child to arrive at a split (arrival counter) leaves its box in the split's
// hand-over slot and stops, the second takes it.  Lanes that stopped take new
// leaves together once 24 of 32 lanes are idle, so that the gathers of a
// refill run side by side on consecutive leaves.
constexpr int kRefitRefill = 24;  // idle lanes before a refill: 24 beat 8 and 16

__global__ void __launch_bounds__(256)
    k_climb(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
            const int64_t *__restrict__ tri_off, int n_scenes, const uint32_t *__restrict__ keys,
            const uint32_t *__restrict__ perm, Node2 *__restrict__ nodes, uint32_t *flags, float4 *slots,
            TriRec *__restrict__ tris, uint32_t spin_limit, uint32_t *err, uint32_t *dirty) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t n_warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t chunk = (n_tri + n_warps - 1) / n_warps;
  int64_t next = warp * chunk;
  const int64_t end = min(next + chunk, n_tri);
  bool climbing = false;
  int n = 0, l = 0, r = 0, depth = 0;
  int up = -1;  // side of the current node under its parent: 0 left, 1 right, -1 not chosen yet
  int sc = -1;  // scene of the lane's last leaf (its leaves only grow)
  int64_t toff = 0;
  uint32_t key_l = 0, key_r = 0;
  float lo[3], hi[3];
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !climbing);
    const int nidle = __popc(idle);
    if (next < end && nidle >= kRefitRefill) {
      const int64_t leaf = next + __popc(idle & lt);
      next += nidle;
      if (!climbing && leaf < end) {
        sc = scene_of(tri_off, n_scenes, leaf, sc);
        const int s = sc;
        toff = tri_off[s];
        n = (int)(tri_off[s + 1] - toff);
        const int64_t orig = perm[leaf];
        // A sort that timed out leaves unspecified slots: never follow them.
        if (orig < toff || orig >= toff + n) {
          atomicOr(err, kErrTimeout);
          *dirty = 1u;
        } else {
          float3 p0, p1, p2;
          tri_verts(pos, idx, orig, p0, p1, p2);
          TriRec rec;
          rec.p0 = make_float4(p0.x, p0.y, p0.z, __int_as_float((int)(orig - toff)));
          rec.p1 = make_float4(p1.x, p1.y, p1.z, 0.0f);
          rec.p2 = make_float4(p2.x, p2.y, p2.z, 0.0f);
          tris[leaf] = rec;
          if (n >= 2) {
            tri_box(p0, p1, p2, lo, hi);
            l = r = (int)(leaf - toff);
            key_l = key_r = keys[leaf];
            depth = 0;
            up = -1;
            climbing = true;
          }
        }
      }
    } else if (nidle == 32) {
      break;  // every leaf of the chunk taken and every climb finished
    }
    // Arrive: node [l, r] (a leaf or a finished internal node) at its
    // parent's split.  Every lane passes the __syncwarp below, so a sibling
    // in the same warp finds the first arrival's record already stored.
    bool take = false, left = false;
    int split = 0;
    if (climbing) {
      if (up < 0) up = parent_side(keys + toff, key_l, key_r, l, r, n);
      left = up == 0;  // the parent splits at r
      split = left ? r : l - 1;
      // A valid tree is at most 62 levels deep; the bound only matters if the
      // inputs were corrupted by an earlier timed-out wait.
      if (depth > 96 || split < 0 || split >= n - 1) {
        atomicOr(err, kErrTimeout);
        *dirty = 1u;
        climbing = false;
      } else if (atomicAdd(flags + toff + split, 1u) == 0u) {
        slot_store(slots + 2 * (toff + split), lo, hi, left ? l : r, left ? key_l : key_r);
        climbing = false;
      } else {
        flags[toff + split] = 0u;  // both arrivals seen: ready for the next build
        take = true;
      }
    }
    __syncwarp();
    if (!take) continue;
    float olo[3], ohi[3];
    int oend = 0;
    uint32_t okey = 0;
    const bool got = slot_take(slots + 2 * (toff + split), olo, ohi, oend, okey, spin_limit);
    // The new node [nl, nr] with children [nl, split] and [split + 1, nr].
    const int nl = left ? l : oend, nr = left ? oend : r;
    if (!got || nl < 0 || nl > split || nr <= split || nr >= n) {
      atomicOr(err, kErrTimeout);
      *dirty = 1u;
      climbing = false;
      continue;
    }
    if (left) key_r = okey;
    else key_l = okey;
    Node2 nd;
    const float *c0lo = left ? lo : olo, *c0hi = left ? hi : ohi;
    const float *c1lo = left ? olo : lo, *c1hi = left ? ohi : hi;
    nd.a = make_float4(c0lo[0], c0hi[0], c0lo[1], c0hi[1]);
    nd.b = make_float4(c1lo[0], c1hi[0], c1lo[1], c1hi[1]);
    nd.c = make_float4(c0lo[2], c0hi[2], c1lo[2], c1hi[2]);
    const int c0 = nl == split ? ~(int)(toff + split) : (int)(toff + split);
    const int c1 = nr == split + 1 ? ~(int)(toff + split + 1) : (int)(toff + split + 1);
    nd.d = make_int4(c0, c1, (int)(toff + nl), (int)(toff + nr));
    l = nl;
    r = nr;
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], olo[k]);
      hi[k] = fmaxf(hi[k], ohi[k]);
    }
    // Its Karras index: 0 for the root, else the end facing its parent.
    int at = 0;
    if (l == 0 && r == n - 1) {
      climbing = false;  // the root: done
    } else {
      up = parent_side(keys + toff, key_l, key_r, l, r, n);
      at = up == 0 ? r : l;
    }
    nodes[toff + at] = nd;
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
  stage_mark(ctx, st, "start");
  const unsigned fill_grid = grid_for(b->n_scenes, 128);
  k_init_boxes<<<fill_grid, 128, 0, st>>>(b->d_scene_box, b->n_scenes);
  FLG_LAUNCH_CHECK(ctx, "k_init_boxes");
  if (b->builder == FLG_BUILDER_SAH) {
    // Top-down from the scene bounds; no Morton codes or sort.
    k_scene_bounds<<<grid_for(n, kBoundsChunk), kBoundsThreads, 0, st>>>(b->pos, b->idx, n, b->d_tri_off,
                                                                       b->n_scenes, b->d_scene_box);
    FLG_LAUNCH_CHECK(ctx, "k_scene_bounds");
    stage_mark(ctx, st, "bounds");
    int rc = sah_build(ctx, b);
    if (rc) return rc;
    if (b->width > 2) return collapse_enqueue(ctx, b, b->width, b->leaf_size);
    return FLG_OK;
  }
  if (b->d_tile_start) {
    FLG_CUDA(ctx, cudaMemsetAsync(b->d_shist, 0, sizeof(uint32_t) * 4 * 256 * (size_t)b->n_scenes, st));
  } else {
    FLG_CUDA(ctx, cudaMemsetAsync(b->d_hist, 0, sizeof(uint32_t) * 256 * b->n_morton_passes, st));
  }
  if (b->n_passes > b->n_morton_passes)
    FLG_CUDA(ctx, cudaMemcpyAsync(b->d_hist + 256 * b->n_morton_passes,
                                  b->d_hist + 512 * b->n_passes,
                                  sizeof(uint32_t) * 256 * (b->n_passes - b->n_morton_passes),
                                  cudaMemcpyDeviceToDevice, st));
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_lookback, 0,
                                sizeof(uint32_t) * 256 * (size_t)b->n_tiles * b->n_passes, st));
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_tile_ctr, 0, sizeof(uint32_t) * b->n_passes, st));
  stage_mark(ctx, st, "setup");

  k_scene_bounds<<<grid_for(n, kBoundsChunk), kBoundsThreads, 0, st>>>(b->pos, b->idx, n, b->d_tri_off,
                                                                     b->n_scenes, b->d_scene_box);
  FLG_LAUNCH_CHECK(ctx, "k_scene_bounds");
  stage_mark(ctx, st, "bounds");
  uint32_t *morton_out = (b->n_passes % 2 == 0) ? b->d_keys : b->d_keys_alt;
  if (b->d_tile_start) {
    k_morton_seg<<<(unsigned)b->n_tiles, 256, 0, st>>>(b->pos, b->idx, b->d_tri_off, b->n_scenes, b->d_tile_start,
                                                      (int)sort_tile(), b->d_scene_box, morton_out, b->d_shist);
    FLG_LAUNCH_CHECK(ctx, "k_morton_seg");
    k_scan_seg<<<(unsigned)(4 * b->n_scenes), 256, 0, st>>>(b->d_shist, b->d_tri_off,
                                                             b->d_shist + 4 * 256 * (size_t)b->n_scenes);
    FLG_LAUNCH_CHECK(ctx, "k_scan_seg");
  } else {
    const unsigned g_elem = grid_for(n, 256, (int64_t)ctx->num_sms * 8);
    k_morton_hist<<<g_elem, 256, 0, st>>>(b->pos, b->idx, n, b->d_tri_off, b->n_scenes, b->d_scene_box,
                                          morton_out, b->d_hist, b->n_morton_passes);
    FLG_LAUNCH_CHECK(ctx, "k_morton_hist");
  }
  stage_mark(ctx, st, "morton");
  int rc = sort_enqueue(ctx, b);
  if (rc) return rc;
  if (b->builder == FLG_BUILDER_PLOC) {
    rc = ploc_build(ctx, b);
    if (rc) return rc;
    stage_mark(ctx, st, "ploc");
    if (b->width > 2) return collapse_enqueue(ctx, b, b->width, b->leaf_size);
    return FLG_OK;
  }
  // Lanes take their next leaf as soon as they stop climbing, so one wave
  // of resident CTAs balances better than more CTAs than fit.
  static const int climb_per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_climb, 256, 0) != cudaSuccess || v < 1) v = 1;
    return v;
  }();
  const unsigned g_nodes = grid_for(b->n_nodes, 256, (int64_t)ctx->num_sms * 8);
  k_climb_reset<<<g_nodes, 256, 0, st>>>(b->d_slots, b->d_flags, b->n_nodes, b->d_dirty);
  FLG_LAUNCH_CHECK(ctx, "k_climb_reset");
  k_climb_clean<<<1, 1, 0, st>>>(b->d_dirty);
  FLG_LAUNCH_CHECK(ctx, "k_climb_clean");
  stage_mark(ctx, st, "climb_reset");
  k_climb<<<grid_for(n, 256, (int64_t)ctx->num_sms * climb_per_sm), 256, 0, st>>>(
      b->pos, b->idx, n, b->d_tri_off, b->n_scenes, b->d_keys, b->d_perm, b->d_nodes2, b->d_flags, b->d_slots,
      b->d_tris, ctx->spin_limit, ctx->d_err, b->d_dirty);
  FLG_LAUNCH_CHECK(ctx, "k_climb");
  stage_mark(ctx, st, "climb");
  if (b->builder == FLG_BUILDER_TREELET) {
    rc = treelet_build(ctx, b);
    if (rc) return rc;
  }
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
  if (builder != FLG_BUILDER_LBVH && builder != FLG_BUILDER_PLOC && builder != FLG_BUILDER_SAH &&
      builder != FLG_BUILDER_TREELET)
    return set_error(ctx, FLG_ERR_ARG,
                     "builder must be FLG_BUILDER_LBVH, FLG_BUILDER_PLOC, FLG_BUILDER_SAH or FLG_BUILDER_TREELET");
  const int tl_rounds = opts && opts->treelet_rounds ? opts->treelet_rounds : 3;
  if (builder == FLG_BUILDER_TREELET && (tl_rounds < 1 || tl_rounds > 4))
    return set_error(ctx, FLG_ERR_ARG, "treelet_rounds must be in [1, 4]");

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
  b->treelet_rounds = tl_rounds;
  b->tri_off_h.assign(tri_off_host, tri_off_host + n_scenes + 1);
  b->node_off_h.resize(n_scenes + 1);
  b->node_off_h[0] = 0;
  std::vector<int32_t> root(n_scenes);
  for (int s = 0; s < n_scenes; ++s) {
    int64_t c = tri_off_host[s + 1] - tri_off_host[s];
    b->node_off_h[s + 1] = tri_off_host[s + 1];  // node slots numbered by sorted position
    root[s] = c >= 2 ? (int32_t)b->node_off_h[s] : c == 1 ? ~(int32_t)tri_off_host[s] : INT32_MIN;
  }
  b->n_nodes = b->node_off_h[n_scenes];
  for (int s = 0; s < n_scenes; ++s) b->n_nonempty += tri_off_host[s + 1] > tri_off_host[s] ? 1 : 0;
  b->n_morton_passes = 4;
  int scene_passes = 0;
  if (n_scenes > 1) scene_passes = n_scenes <= 256 ? 1 : n_scenes <= 65536 ? 2 : 3;
  b->n_tiles = sort_tiles(n);
  // Batched builds whose scenes average at least 4 sort tiles sort each
  // scene in its own run of tiles (per-scene digit offsets, look-back chains
  // restarting at each scene) instead of appending scene passes.
  std::vector<int32_t> tile_start;
  if (n_scenes > 1 && n >= 4 * (int64_t)sort_tile() * n_scenes) {
    tile_start.resize(n_scenes + 1);
    tile_start[0] = 0;
    for (int s = 0; s < n_scenes; ++s)
      tile_start[s + 1] = tile_start[s] + (int32_t)sort_tiles(tri_off_host[s + 1] - tri_off_host[s]);
    b->n_tiles = tile_start[n_scenes];
    scene_passes = 0;
  }
  b->n_passes = b->n_morton_passes + scene_passes;

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
  A(&b->d_flags, b->n_nodes);
  A(&b->d_slots, 2 * (size_t)b->n_nodes);
  A(&b->d_dirty, 1);
  A(&b->d_nodes2, b->n_nodes);
  A(&b->d_tris, n);
  // hist: [passes][256] counts, [passes][256] offsets, [passes][256] static scene counts
  A(&b->d_hist, 3 * 256 * (size_t)b->n_passes);
  if (!tile_start.empty()) {
    A(&b->d_tile_start, n_scenes + 1);
    A(&b->d_shist, 2 * 4 * 256 * (size_t)n_scenes);  // per-scene counts, then bucket starts
  }
  A(&b->d_lookback, 256 * (size_t)b->n_tiles * b->n_passes);
  A(&b->d_tile_ctr, b->n_passes);
  if (rc == FLG_OK && builder == FLG_BUILDER_PLOC) rc = ploc_reserve(b);
  if (rc == FLG_OK && builder == FLG_BUILDER_SAH) rc = sah_reserve(b);
  if (rc == FLG_OK && builder == FLG_BUILDER_TREELET) rc = treelet_reserve(b);
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
  if (e == cudaSuccess && !tile_start.empty())
    e = cudaMemcpyAsync(b->d_tile_start, tile_start.data(), sizeof(int32_t) * (n_scenes + 1),
                        cudaMemcpyHostToDevice, st);
  // Static scene counts live after counts and offsets; build_enqueue copies
  // the scene passes' part into place each build.
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_hist + 512 * (size_t)b->n_passes, sh.data() + 256 * b->n_morton_passes,
                        sizeof(uint32_t) * 256 * (b->n_passes - b->n_morton_passes), cudaMemcpyHostToDevice, st);
  // Node records zeroed (unused slots hold refs 0), climb scratch unset.
  if (e == cudaSuccess && b->n_nodes > 0) e = cudaMemsetAsync(b->d_nodes2, 0, sizeof(Node2) * (size_t)b->n_nodes, st);
  if (e == cudaSuccess) {
    k_climb_reset<<<grid_for(b->n_nodes, 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(b->d_slots, b->d_flags,
                                                                                      b->n_nodes, nullptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_dirty, 0, sizeof(uint32_t), st);
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
  if (bvh->builder == FLG_BUILDER_PLOC)
    return set_error(ctx, FLG_ERR_UNSUPPORTED, "PLOC handles keep no Karras-numbered node records");
  if (scene < 0 || scene >= bvh->n_scenes) return set_error(ctx, FLG_ERR_ARG, "scene out of range");
  cudaStream_t st = ctx->stream;
  const int64_t toff = bvh->tri_off_h[scene];
  const int64_t n = bvh->tri_off_h[scene + 1] - toff;
  const int64_t m = n >= 2 ? n - 1 : 0;  // internal nodes, at slots toff .. toff + m - 1
  cudaError_t e = cudaStreamSynchronize(st);
  auto D = [&](void *dst, const void *src, size_t bytes) {
    if (e == cudaSuccess && dst && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
  };
  D(t->morton, bvh->d_keys + toff, sizeof(uint32_t) * n);
  D(t->perm, bvh->d_perm + toff, sizeof(int32_t) * n);
  D(t->scene_bound, bvh->d_scene_box + 6 * scene, sizeof(float) * 6);
  std::vector<Node2> nodes(m);
  if (m > 0) D(nodes.data(), bvh->d_nodes2 + toff, sizeof(Node2) * m);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "download");
  if (t->perm)
    for (int64_t i = 0; i < n; ++i) t->perm[i] -= (int32_t)toff;
  // The Karras arrays follow from the node records: child refs name the
  // split (left child at split, right at split + 1), d.z / d.w the range.
  if (t->leaf_parent && n == 1) t->leaf_parent[0] = -1;  // a lone leaf is the root
  if (t->parent && m > 0) t->parent[0] = 0;
  for (int64_t i = 0; i < m; ++i) {
    const Node2 &q = nodes[i];
    const int c0 = q.d.x, c1 = q.d.y;
    const int64_t lo = q.d.z - toff, hi = q.d.w - toff;
    const int64_t split = (c0 >= 0 ? c0 : ~c0) - toff;
    if (lo < 0 || hi >= n || split < lo || split >= hi || (lo != i && hi != i))
      return set_error(ctx, FLG_ERR_STATE, "node %lld of scene %d is inconsistent", (long long)i, scene);
    if (t->split) t->split[i] = (int32_t)split;
    if (t->leaf_flags) t->leaf_flags[i] = (uint8_t)((c0 < 0 ? 1 : 0) | (c1 < 0 ? 2 : 0));
    if (t->range_j) t->range_j[i] = (int32_t)(lo == i ? hi : lo);
    const int cr[2] = {c0, c1};
    for (int k = 0; k < 2; ++k) {
      const int64_t c = (cr[k] >= 0 ? cr[k] : ~cr[k]) - toff;
      if (c < 0 || c >= n) return set_error(ctx, FLG_ERR_STATE, "child ref out of scene %d", scene);
      if (cr[k] < 0) {
        if (t->leaf_parent) t->leaf_parent[c] = (int32_t)i;
      } else if (t->parent && c < m) {
        t->parent[c] = (int32_t)i;
      }
    }
    if (t->bounds) {
      float *o = t->bounds + 6 * i;
      o[0] = std::min(q.a.x, q.b.x);
      o[3] = std::max(q.a.y, q.b.y);
      o[1] = std::min(q.a.z, q.b.z);
      o[4] = std::max(q.a.w, q.b.w);
      o[2] = std::min(q.c.x, q.c.z);
      o[5] = std::max(q.c.y, q.c.w);
    }
  }
  return FLG_OK;
}
