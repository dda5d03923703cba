// collapse.cu — re-lays out a built Karras BVH2 as 4- or 8-wide nodes for
// traversal.  Top-down, level by level (one cooperative launch with a grid
// barrier between levels; one launch per level under stream capture): each
// queued BVH2 node becomes a wide node whose children are found by
// repeatedly opening the child with the largest surface area (Wald, Benthin,
// Boulos 2008 style collapsing).
// A BVH2 subtree covers a contiguous run of sorted triangles, so any subtree
// with at most leaf_size triangles becomes a leaf range [first, first+count).
// The Karras topology itself (the parity object) is unchanged.
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr int kMaxLevels = 64;
// Collapse counters: [0] wide nodes allocated, [1 + L] queue size of level L,
// [kMaxLevels + 2 .. + 3] the one-launch collapse's barrier; the initial
// values of these kCtrLive words follow as a static copy.
constexpr int kCtrLive = kMaxLevels + 4;

struct Cand {
  int32_t ref;     // BVH2 ref (>=0 internal, <0 ~leaf position)
  int32_t first;   // first sorted triangle of the subtree
  int32_t count;   // triangles in the subtree
  float lo[3], hi[3];
};

__device__ __forceinline__ float half_area(const Cand &c) {
  float dx = c.hi[0] - c.lo[0], dy = c.hi[1] - c.lo[1], dz = c.hi[2] - c.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// Leaf ranges of internal nodes.  LBVH records carry their own range
// (d.z, d.w: first and last sorted triangle) and split (the left child ref
// names it, node slots being numbered by sorted position), so both children's
// ranges come from the parent's record; PLOC trees keep explicit depth-first
// ranges (rfirst / rcount) per node.
struct Ranges {
  const int32_t *rfirst, *rcount;
};

__device__ __forceinline__ void child_cands(const Node2 &nd, const Ranges &R, Cand &c0, Cand &c1) {
  int32_t r[2] = {nd.d.x, nd.d.y};
  Cand *o[2] = {&c0, &c1};
  const float lo[2][3] = {{nd.a.x, nd.a.z, nd.c.x}, {nd.b.x, nd.b.z, nd.c.z}};
  const float hi[2][3] = {{nd.a.y, nd.a.w, nd.c.y}, {nd.b.y, nd.b.w, nd.c.w}};
  const int32_t split = r[0] >= 0 ? r[0] : ~r[0];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    Cand &c = *o[k];
    c.ref = r[k];
    for (int a = 0; a < 3; ++a) {
      c.lo[a] = lo[k][a];
      c.hi[a] = hi[k][a];
    }
    if (!R.rfirst) {
      c.first = k == 0 ? nd.d.z : split + 1;
      c.count = k == 0 ? split - nd.d.z + 1 : nd.d.w - split;
    } else if (r[k] < 0) {
      c.first = ~r[k];
      c.count = 1;
    } else {
      c.first = R.rfirst[r[k]];
      c.count = R.rcount[r[k]];
    }
  }
}

// One wide node per queued BVH2 node of a level (cnt items in q_in).  The
// new wide slots and queue entries of a warp are claimed with one atomic per
// counter (warp prefix sum of the lanes' internal children): per-child
// atomics on the two shared counters serialised in L2.  Queue entries are
// read through L2 (__ldcg): in the one-launch collapse this SM may still
// hold lines of the same buffer from two levels before.
template <int W>
__device__ __forceinline__ void collapse_level(const Node2 *__restrict__ nodes2, const Ranges &R, int leaf_size,
                                               const int2 *__restrict__ q_in, int cnt, int2 *__restrict__ q_out,
                                               int32_t *q_out_count, int32_t *node_ctr, int64_t cap,
                                               NodeW<W> *__restrict__ wide, uint32_t *err) {
  const int lane = threadIdx.x & 31;
  // Warp-uniform loop: all lanes of a warp share it0.
  for (int it0 = (int)((blockIdx.x * blockDim.x + threadIdx.x) & ~31u); it0 < cnt;
       it0 += gridDim.x * blockDim.x) {
    const int it = it0 + lane;
    const bool valid = it < cnt;
    int2 item = make_int2(0, 0);
    Cand c[W];
    int nc = 0;
    if (valid) {
      item = __ldcg(q_in + it);
      // cap = BVH2 node count + 1: item.x names a BVH2 node, item.y a wide slot.
      if (item.x < 0 || item.y < 0 || item.x >= cap - 1 || item.y >= cap) {
        atomicOr(err, kErrQueue);  // a hole left by an overflowing level
      } else {
        nc = 2;
        child_cands(nodes2[item.x], R, c[0], c[1]);
      }
    }
    // The records of both children that may be opened are fetched together:
    // the first opening takes one of them and the second usually the other,
    // so most wide nodes wait on two dependent loads instead of three.
    Node2 pf0, pf1;
    const int32_t pf0_ref = nc == 2 && c[0].ref >= 0 && c[0].count > leaf_size ? c[0].ref : -1;
    const int32_t pf1_ref = nc == 2 && c[1].ref >= 0 && c[1].count > leaf_size ? c[1].ref : -1;
    if (pf0_ref >= 0) pf0 = nodes2[pf0_ref];
    if (pf1_ref >= 0) pf1 = nodes2[pf1_ref];
    while (nc >= 2 && nc < W) {
      int best = -1;
      float ba = -1.0f;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        if (k < nc && c[k].ref >= 0 && c[k].count > leaf_size) {
          float a = half_area(c[k]);
          if (a > ba) {
            ba = a;
            best = k;
          }
        }
      }
      if (best < 0) break;
      Cand a, b;
      int32_t r = 0;
#pragma unroll
      for (int k = 0; k < W; ++k)
        if (k == best) r = c[k].ref;
      if (r == pf0_ref) child_cands(pf0, R, a, b);
      else if (r == pf1_ref) child_cands(pf1, R, a, b);
      else child_cands(nodes2[r], R, a, b);
#pragma unroll
      for (int k = 0; k < W; ++k) {
        if (k == best) c[k] = a;
        if (k == nc) c[k] = b;
      }
      ++nc;
    }
    // Children that become wide nodes of the next level.
    int need = 0;
#pragma unroll
    for (int k = 0; k < W; ++k)
      if (k < nc && c[k].ref >= 0 && c[k].count > leaf_size) ++need;
    int incl = need;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    int slot0 = 0, q0 = 0;
    if (lane == 31 && total > 0) {
      slot0 = atomicAdd(node_ctr, total);
      q0 = atomicAdd(q_out_count, total);
    }
    slot0 = __shfl_sync(0xFFFFFFFFu, slot0, 31) + incl - need;
    q0 = __shfl_sync(0xFFFFFFFFu, q0, 31) + incl - need;
    if (!valid || nc == 0) continue;
    NodeW<W> out;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      if (k < nc) {
        out.lox[k] = c[k].lo[0];
        out.loy[k] = c[k].lo[1];
        out.loz[k] = c[k].lo[2];
        out.hix[k] = c[k].hi[0];
        out.hiy[k] = c[k].hi[1];
        out.hiz[k] = c[k].hi[2];
        if (c[k].ref < 0 || c[k].count <= leaf_size) {
          out.child[k] = ~((c[k].first << 3) | (c[k].count - 1));
        } else {
          const int slot = slot0++;
          if (slot >= cap) {
            atomicOr(err, kErrQueue);
            if (q0 < cap) q_out[q0] = make_int2(-1, -1);  // the next level skips it
            ++q0;
            out.child[k] = kEmptyChild;
          } else {
            q_out[q0++] = make_int2(c[k].ref, slot);
            out.child[k] = slot;
          }
        }
      } else {
        const float inf = __int_as_float(0x7f800000);
        out.lox[k] = out.loy[k] = out.loz[k] = inf;
        out.hix[k] = out.hiy[k] = out.hiz[k] = inf;
        out.child[k] = kEmptyChild;
      }
    }
    wide[item.y] = out;
  }
}

template <int W>
__global__ void __launch_bounds__(128)
    k_collapse_level(const Node2 *__restrict__ nodes2, Ranges R, int leaf_size,
                     const int2 *__restrict__ q_in, const int32_t *__restrict__ q_in_count, int2 *__restrict__ q_out,
                     int32_t *q_out_count, int32_t *node_ctr, int64_t cap, NodeW<W> *__restrict__ wide,
                     uint32_t *err) {
  // Counts beyond the queue capacity only arise from a corrupted tree.
  const int cnt = (int)min((int64_t)*q_in_count, cap);
  collapse_level<W>(nodes2, R, leaf_size, q_in, cnt, q_out, q_out_count, node_ctr, cap, wide, err);
}

// Barrier over all CTAs of a cooperative launch (all resident): bar[0]
// counts arrivals, bar[1] is the generation.  Fences make each CTA's writes
// of the level visible before it arrives and the others' after it leaves.
// The wait is bounded: on a timeout the error word is set and the CTA goes
// on (the tree is then wrong, the device keeps answering).
__device__ __forceinline__ void grid_barrier(uint32_t *bar, uint32_t limit, uint32_t *err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = ld_volatile(bar + 1);
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      *(volatile uint32_t *)bar = 0u;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      for (uint32_t spins = 0; ld_volatile(bar + 1) == gen; ++spins) {
        if (spins >= limit) {
          atomicOr(err, kErrTimeout);
          break;
        }
        if (spins > 64) __nanosleep(128);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// The whole collapse in one cooperative launch: level after level with a
// grid barrier between them, until a level is empty.  Replaces up to 64
// launches (most of them empty) by one.
template <int W>
__global__ void __launch_bounds__(128)
    k_collapse_all(const Node2 *__restrict__ nodes2, Ranges R, int leaf_size, int2 *q0, int2 *q1, int32_t *ctr,
                   uint32_t *bar, int64_t cap, NodeW<W> *__restrict__ wide, uint32_t spin_limit, uint32_t *err) {
  for (int L = 0; L < kMaxLevels; ++L) {
    // Counts beyond the queue capacity only arise from a corrupted tree.
    const int cnt = (int)min((int64_t)(int32_t)ld_volatile((const uint32_t *)(ctr + 1 + L)), cap);
    if (cnt == 0) break;  // the same value in every CTA: read after the last barrier
    collapse_level<W>(nodes2, R, leaf_size, (L & 1) ? q1 : q0, cnt, (L & 1) ? q0 : q1, ctr + 2 + L, ctr, cap, wide,
                      err);
    grid_barrier(bar, spin_limit, err);
  }
}

__global__ void k_collapse_check(const int32_t *last_count, uint32_t *err) {
  if (*last_count > 0) atomicOr(err, kErrQueue);
}

int collapse_reserve(flg_ctx ctx, flg_bvh b) {
  // Every wide node corresponds to a distinct BVH2 internal node.
  const int64_t cap = b->n_nodes + 1;
  const size_t rec = b->width == 4 ? sizeof(NodeW<4>) : sizeof(NodeW<8>);
  int rc = FLG_OK;
  if (b->d_wide) {
    cudaFree(b->d_wide);
    b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), b->d_wide));
    b->device_bytes -= (int64_t)(b->wide_cap * (b->wide_rec));
    b->d_wide = nullptr;
  }
  uint8_t *w = nullptr;
  rc = halloc(b, &w, rec * (size_t)cap);
  if (rc) return rc;
  b->d_wide = w;
  b->wide_cap = cap;
  b->wide_rec = (int64_t)rec;
  if (!b->d_wide_root) {
    if ((rc = halloc(b, &b->d_wide_root, b->n_scenes))) return rc;
    if ((rc = halloc(b, &b->d_wide_ctr, 2 * kCtrLive))) return rc;
    if ((rc = halloc(b, &b->d_queue[0], cap))) return rc;
    if ((rc = halloc(b, &b->d_queue[1], cap))) return rc;
    if ((rc = halloc(b, &b->d_queue_init, b->n_scenes))) return rc;
    std::vector<int32_t> roots(b->n_scenes);
    std::vector<int2> q;
    for (int s = 0; s < b->n_scenes; ++s) {
      int64_t c = b->tri_off_h[s + 1] - b->tri_off_h[s];
      if (c >= 2) {
        roots[s] = (int32_t)q.size();
        q.push_back(make_int2((int)b->node_off_h[s], (int)q.size()));
      } else if (c == 1) {
        roots[s] = ~(int32_t)(b->tri_off_h[s] << 3);
      } else {
        roots[s] = kEmptyChild;
      }
    }
    b->n_wide_roots = (int32_t)q.size();
    std::vector<int32_t> ctr(2 * kCtrLive, 0);
    ctr[0] = b->n_wide_roots;
    ctr[1] = b->n_wide_roots;
    ctr[kCtrLive] = b->n_wide_roots;
    ctr[kCtrLive + 1] = b->n_wide_roots;
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(b->d_wide_root, roots.data(), sizeof(int32_t) * b->n_scenes,
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !q.empty())
      e = cudaMemcpyAsync(b->d_queue_init, q.data(), sizeof(int2) * q.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->d_wide_ctr, ctr.data(), sizeof(int32_t) * ctr.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "collapse upload");
  }
  return FLG_OK;
}

template <int W>
static int collapse_levels(flg_ctx ctx, flg_bvh b) {
  cudaStream_t st = ctx->stream;
  NodeW<W> *wide = (NodeW<W> *)b->d_wide;
  const Ranges R{b->d_rfirst, b->d_rcount};
  // Level sizes are only known on the device.  Default: one cooperative
  // launch of one resident wave that walks the levels with a grid barrier in
  // between and stops at the first empty one.  Under stream capture: one
  // launch of one resident wave per level (the empty ones after the deepest
  // exit at once).
  static const int all_per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_collapse_all<W>, 128, 0) != cudaSuccess || v < 1)
      v = 1;
    return v;
  }();
  static const int level_per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_collapse_level<W>, 128, 0) != cudaSuccess || v < 1)
      v = 1;
    return v;
  }();
  int32_t *ctr = b->d_wide_ctr;
  if (!ctx->capturing) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctx->num_sms * (unsigned)all_per_sm);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    uint32_t *bar = (uint32_t *)(ctr + kMaxLevels + 2);
    FLG_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_collapse_all<W>, (const Node2 *)b->d_nodes2, R, (int)b->leaf_size,
                                     b->d_queue[0], b->d_queue[1], ctr, bar, (int64_t)b->wide_cap, wide,
                                     ctx->spin_limit, ctx->d_err));
    FLG_LAUNCH_CHECK(ctx, "k_collapse_all");
  } else {
    const unsigned grid = (unsigned)ctx->num_sms * (unsigned)level_per_sm;
    for (int L = 0; L < kMaxLevels; ++L) {
      k_collapse_level<W><<<grid, 128, 0, st>>>(b->d_nodes2, R, b->leaf_size, b->d_queue[L & 1], ctr + 1 + L,
                                                b->d_queue[(L + 1) & 1], ctr + 2 + L, ctr, b->wide_cap, wide,
                                                ctx->d_err);
      FLG_LAUNCH_CHECK(ctx, "k_collapse_level");
    }
  }
  k_collapse_check<<<1, 1, 0, st>>>(ctr + 1 + kMaxLevels, ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_collapse_check");
  return FLG_OK;
}

int collapse_enqueue(flg_ctx ctx, flg_bvh b, int width, int leaf_size) {
  (void)leaf_size;
  if (b->n_wide_roots == 0) return FLG_OK;
  cudaStream_t st = ctx->stream;
  FLG_CUDA(ctx, cudaMemcpyAsync(b->d_wide_ctr, b->d_wide_ctr + kCtrLive, sizeof(int32_t) * kCtrLive,
                                cudaMemcpyDeviceToDevice, st));
  FLG_CUDA(ctx, cudaMemcpyAsync(b->d_queue[0], b->d_queue_init, sizeof(int2) * b->n_wide_roots,
                                cudaMemcpyDeviceToDevice, st));
  const int rc = width == 4 ? collapse_levels<4>(ctx, b) : collapse_levels<8>(ctx, b);
  if (rc == FLG_OK) stage_mark(ctx, st, "collapse");
  return rc;
}

}  // namespace flg

using namespace flg;

FLG_API int flg_bvh_set_width(flg_ctx ctx, flg_bvh bvh, int32_t node_width, int32_t leaf_size) {
  if (!ctx || !bvh) return FLG_ERR_ARG;
  if (node_width != 2 && node_width != 4 && node_width != 8)
    return set_error(ctx, FLG_ERR_ARG, "node_width must be 2, 4 or 8");
  if (leaf_size < 1 || leaf_size > 8) return set_error(ctx, FLG_ERR_ARG, "leaf_size must be in [1, 8]");
  if (node_width == bvh->width && leaf_size == bvh->leaf_size) return FLG_OK;
  const int old_w = bvh->width;
  bvh->width = node_width;
  bvh->leaf_size = leaf_size;
  if (node_width == 2) return FLG_OK;
  if (ctx->capturing && (old_w != node_width || !bvh->d_wide))
    return set_error(ctx, FLG_ERR_STATE, "re-layout allocates; not allowed during capture");
  if (!bvh->d_wide || old_w != node_width) {
    int rc = collapse_reserve(ctx, bvh);
    if (rc) return rc;
  }
  return collapse_enqueue(ctx, bvh, node_width, leaf_size);
}
