// sah.cu — binned-SAH top-down builder (FLG_BUILDER_SAH): the split rule of
// BasicBVHBuilder::recursiveBuilder with EBVHPartitionMethod::ESAH
// (src/experimental/base_bvh.cpp:33-173), applied to every node of every
// scene, one tree level per sequence of launches.
//
// The rule at a node of n triangles at depth d (root 0):
//   * a leaf when n <= 8 or d >= 26 (base_bvh.cpp:44);
//   * otherwise, with B the node's bound (union of its triangles' boxes) and
//     axis a = d % 3, triangle t falls in bucket
//     floor(16 * ((c_t - B.lo) / (B.hi - B.lo))[a]), c_t = (p0 + p1 + p2) / 3
//     (base_bvh.hpp:86-87); for i = 1 .. 14 the cost is
//     1/8 + (SA(L_i) |L_i| + SA(R_i) |R_i|) / SA(B), L_i the buckets 0..i and
//     R_i the rest, SA = 2 (ex ey + ex ez + ey ez) (base_bvh.hpp:58-63); the
//     first minimum wins; the node splits when that cost is below n, else it
//     is a leaf (base_bvh.cpp:109-165).  Every step is evaluated in the
//     reference's order with one rounding per operation, the cost's 1/8 added
//     in double as the reference's `1.0 / 8 + ...` does.
// Where this differs from the reference, its behaviour is undefined or its
// tree is not of this library's form:
//   * a bucket index outside [0, 15] (a centroid rounded past the bound, 0/0
//     on a flat axis) is clamped, NaN to 0; the reference indexes its bucket
//     array out of bounds there (an assert in debug builds);
//   * partitions are stable (std::partition leaves the order unspecified);
//   * a leaf of k > 1 triangles becomes a balanced binary subtree (left part
//     floor(k / 2)), so every BVH2 leaf holds one triangle and the collapse
//     forms the traversal's leaf ranges as it does for the LBVH;
//   * internal nodes are numbered as in the Karras tree: the root by its
//     first position, a left child by its last, a right child by its first.
//     That is a bijection onto the n - 1 slots for any binary tree over a
//     sorted range (boundary b between positions b and b + 1 names the left
//     child b and the right child b + 1 of the node splitting there), so the
//     LBVH's node records, collapse, traversal and topology download apply
//     unchanged.
// The reference's own build() calls the recursion with the default method
// ENone and the recursion does not pass the method on (base_bvh.hpp:153-155,
// base_bvh.cpp:24,167-170), so build() itself splits at object medians; the
// SAH rule is the one the reference writes out for a high-quality build.
//
// One level: k_sah_bin (bucket boxes and counts of every node: shared-memory
// bins when a 2048-position chunk holds at most 32 nodes, global atomics
// otherwise), k_sah_split (one thread per node: the rule above, the node
// record, children queued for the next level or finished), k_sah_flags and
// the flag scan (stable partition ranks), k_sah_scatter (records to their new
// positions; final triangle records of ranges that are finished) and
// k_sah_finish (balanced subtrees over finished ranges of 2..32 triangles).
// Larger leaves (the depth limit, no split below the leaf cost) are halved by
// the same level loop.
#include <cfloat>

#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr int kSahBuckets = 16;
constexpr int kSahLeafMax = 8;     // base_bvh.cpp:44: n <= 8 is a leaf
constexpr int kSahDepthMax = 26;   // base_bvh.cpp:44: depth >= 26 is a leaf
constexpr int kSahFinishMax = 32;  // ranges up to this size are finished by one thread
constexpr int kSahBinThreads = 256, kSahBinItems = 8, kSahChunk = kSahBinThreads * kSahBinItems;
constexpr int kSahBinWords = 8;    // lo key xyz, hi key xyz, count, unused
constexpr int kSahMaxLevels = 128;
enum { kModeBins = 0, kModeHalves = 1 };

// One node of a level's list.  r: first position, count, node slot, mode.
// s (written by k_sah_split): left count (-1: not split this level), last
// bucket of the left side, next-level list index of each child (-1: the
// child is finished or one triangle).
struct alignas(16) SahNode {
  float4 lo, hi;
  int4 r;
  int4 s;
};

// Order-preserving float <-> uint32 keys for atomic min / max.
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__device__ __forceinline__ float comp(const float4 &v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }

// Bucket of a centroid coordinate c in [lo, hi] (base_bvh.cpp:113-114),
// clamped to [0, 15] (NaN to 0).
__device__ __forceinline__ int sah_bucket(float c, float lo, float hi) {
  const float q = __fmul_rn(__fdiv_rn(__fsub_rn(c, lo), __fsub_rn(hi, lo)), (float)kSahBuckets);
  const float f = floorf(q);
  return f >= 0.0f ? (f < (float)kSahBuckets ? (int)f : kSahBuckets - 1) : 0;
}

// BVHBound::surfaceArea (base_bvh.hpp:58-63).
__device__ __forceinline__ float sah_area(const float *lo, const float *hi) {
  const float ex = __fsub_rn(hi[0], lo[0]), ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(ex, ey), __fmul_rn(ex, ez)), __fmul_rn(ey, ez)));
}

__device__ __forceinline__ void bins_init(uint32_t *b) {
  const uint32_t klo = fkey(FLT_MAX), khi = fkey(-FLT_MAX);
  uint4 *v = (uint4 *)b;
#pragma unroll 4
  for (int k = 0; k < kSahBuckets; ++k) {
    v[2 * k] = make_uint4(klo, klo, klo, khi);
    v[2 * k + 1] = make_uint4(khi, khi, 0u, 0u);
  }
}

__device__ __forceinline__ int sah_queue(SahNode *list, int32_t *cnt, int64_t cap, uint32_t *bins, const float *lo,
                                         const float *hi, int first, int count, int slot, int mode, uint32_t *err) {
  const int k = atomicAdd(cnt, 1);
  if (k >= cap) {
    atomicOr(err, kErrQueue);
    return -1;
  }
  SahNode q;
  q.lo = make_float4(lo[0], lo[1], lo[2], 0.0f);
  q.hi = make_float4(hi[0], hi[1], hi[2], 0.0f);
  q.r = make_int4(first, count, slot, mode);
  q.s = make_int4(-1, -1, -1, -1);
  list[k] = q;
  bins_init(bins + (int64_t)k * kSahBuckets * kSahBinWords);
  return k;
}

__device__ __forceinline__ void sah_finish_item(int4 *fin, int32_t *cnt_fin, int64_t fin_cap, int first, int count,
                                                int slot, uint32_t *err) {
  const int k = atomicAdd(cnt_fin, 1);
  if (k >= fin_cap) {
    atomicOr(err, kErrQueue);
    return;
  }
  fin[k] = make_int4(first, count, slot, 0);
}

// Final record of the triangle at sorted position q (original index orig).
__device__ __forceinline__ void sah_final(const float *__restrict__ pos, const int32_t *__restrict__ idx,
                                          const int64_t *__restrict__ tri_off, int n_scenes, int64_t q, int64_t orig,
                                          uint32_t *__restrict__ perm, TriRec *__restrict__ tris) {
  const int s = find_segment(tri_off, n_scenes, q);
  float3 a, b, c;
  tri_verts(pos, idx, orig, a, b, c);
  TriRec r;
  r.p0 = make_float4(a.x, a.y, a.z, __int_as_float((int)(orig - tri_off[s])));
  r.p1 = make_float4(b.x, b.y, b.z, 0.0f);
  r.p2 = make_float4(c.x, c.y, c.z, 0.0f);
  tris[q] = r;
  perm[q] = (uint32_t)orig;
}

// Roots: scenes of 2..8 triangles are leaves (finished now), larger ones
// start the level loop.
__global__ void k_sah_roots(const int64_t *__restrict__ tri_off, int n_scenes, const float *__restrict__ scene_box,
                            SahNode *list, int32_t *cnt, int64_t cap, uint32_t *bins, int4 *fin, int32_t *cnt_fin,
                            int64_t fin_cap, int32_t *__restrict__ root_seg, uint32_t *err) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_scenes) return;
  const int64_t toff = tri_off[s], ns = tri_off[s + 1] - toff;
  root_seg[s] = -1;
  if (ns < 2) return;
  if (ns <= kSahLeafMax) {
    sah_finish_item(fin, cnt_fin, fin_cap, (int)toff, (int)ns, (int)toff, err);
    return;
  }
  const float *b = scene_box + 6 * s;
  root_seg[s] = sah_queue(list, cnt, cap, bins, b, b + 3, (int)toff, (int)ns, (int)toff, kModeBins, err);
}

// Triangle boxes and centroids in input order; positions of finished scenes
// get their final records at once.
__global__ void k_sah_init(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n,
                           const int64_t *__restrict__ tri_off, int n_scenes, const int32_t *__restrict__ root_seg,
                           float4 *__restrict__ box, float4 *__restrict__ cen, int32_t *__restrict__ seg,
                           uint32_t *__restrict__ perm, TriRec *__restrict__ tris) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, p);
    float3 a, b, c;
    tri_verts(pos, idx, p, a, b, c);
    float lo[3], hi[3];
    tri_box(a, b, c, lo, hi);
    box[2 * p] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    box[2 * p + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    // Triangle::center: (a + b + c) / 3 (base_bvh.hpp:86-87)
    cen[p] = make_float4(__fdiv_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), 3.0f),
                         __fdiv_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), 3.0f),
                         __fdiv_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), 3.0f), __int_as_float((int)p));
    const int rs = root_seg[s];
    seg[p] = rs;
    if (rs < 0) {
      TriRec r;
      r.p0 = make_float4(a.x, a.y, a.z, __int_as_float((int)(p - tri_off[s])));
      r.p1 = make_float4(b.x, b.y, b.z, 0.0f);
      r.p2 = make_float4(c.x, c.y, c.z, 0.0f);
      tris[p] = r;
      perm[p] = (uint32_t)p;
    }
  }
}

__device__ __forceinline__ int sah_side_bucket(const SahNode &N, int64_t p, const float4 &c, int axis) {
  if (N.r.w == kModeHalves) return (p - N.r.x) < (N.r.y >> 1) ? 0 : kSahBuckets - 1;
  return sah_bucket(comp(c, axis), comp(N.lo, axis), comp(N.hi, axis));
}

// Bucket boxes and counts.  A CTA takes chunks of 2048 positions and splits
// each into runs of equal list index (nodes are contiguous position ranges,
// so a run is the part of one node inside the chunk).  With at most 32 runs
// the chunk is binned in shared memory and flushed with one atomic per
// non-empty bucket word; otherwise (nodes of a few dozen triangles) every
// position goes to the global bins directly.
constexpr int kSahRuns = 32;
__global__ void __launch_bounds__(kSahBinThreads)
    k_sah_bin(const float4 *__restrict__ box, const float4 *__restrict__ cen, const int32_t *__restrict__ seg,
              int64_t n, const SahNode *__restrict__ list, uint32_t *bins, int axis) {
  __shared__ uint32_t s_bins[kSahRuns * kSahBuckets * kSahBinWords];
  __shared__ uint8_t s_run[kSahChunk];
  __shared__ int32_t s_rseg[kSahRuns];
  __shared__ int32_t s_warp[kSahBinThreads / 32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int64_t c0 = (int64_t)blockIdx.x * kSahChunk; c0 < n; c0 += (int64_t)gridDim.x * kSahChunk) {
    const int64_t c1 = min(c0 + (int64_t)kSahChunk, n) - 1;
    // Run starts over positions c0 + 8t .. c0 + 8t + 7, then a block scan.
    int sv[kSahBinItems];
    int starts = 0;
    uint32_t smask = 0;
#pragma unroll
    for (int j = 0; j < kSahBinItems; ++j) {
      const int64_t p = c0 + (int64_t)kSahBinItems * t + j;
      sv[j] = p <= c1 ? seg[p] : -1;
      const bool st = p <= c1 && (p == c0 || sv[j] != (j > 0 ? sv[j - 1] : seg[p - 1]));
      starts += st ? 1 : 0;
      smask |= st ? (1u << j) : 0u;
    }
    int incl = starts;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int base = 0, runs = 0;
#pragma unroll
    for (int w = 0; w < kSahBinThreads / 32; ++w) {
      base += w < warp ? s_warp[w] : 0;
      runs += s_warp[w];
    }
    const bool local = runs <= kSahRuns;
    if (local) {
      int r = base + incl - starts - 1;
#pragma unroll
      for (int j = 0; j < kSahBinItems; ++j) {
        const int64_t p = c0 + (int64_t)kSahBinItems * t + j;
        if (p > c1) break;
        if (smask & (1u << j)) {
          ++r;
          s_rseg[r] = sv[j];
        }
        s_run[kSahBinItems * t + j] = (uint8_t)r;
      }
      for (int w = t; w < runs * kSahBuckets * kSahBinWords; w += kSahBinThreads) {
        const int k = w % kSahBinWords;
        s_bins[w] = k < 3 ? fkey(FLT_MAX) : k < 6 ? fkey(-FLT_MAX) : 0u;
      }
    }
    __syncthreads();
    for (int k = 0; k < kSahBinItems; ++k) {
      const int64_t p = c0 + (int64_t)k * kSahBinThreads + t;
      if (p > c1) break;
      const int s = seg[p];
      if (s < 0) continue;
      const SahNode N = list[s];
      const int b = sah_side_bucket(N, p, cen[p], axis);
      const float4 bl = box[2 * p], bh = box[2 * p + 1];
      uint32_t *d = local ? s_bins + ((int)s_run[k * kSahBinThreads + t] * kSahBuckets + b) * kSahBinWords
                          : bins + ((int64_t)s * kSahBuckets + b) * kSahBinWords;
      atomicMin(d + 0, fkey(bl.x));
      atomicMin(d + 1, fkey(bl.y));
      atomicMin(d + 2, fkey(bl.z));
      atomicMax(d + 3, fkey(bh.x));
      atomicMax(d + 4, fkey(bh.y));
      atomicMax(d + 5, fkey(bh.z));
      atomicAdd(d + 6, 1u);
    }
    if (local) {
      __syncthreads();
      for (int e = t; e < runs * kSahBuckets * 7; e += kSahBinThreads) {
        const int r = e / (kSahBuckets * 7), b = (e / 7) % kSahBuckets, w = e % 7;
        const int s = s_rseg[r];
        const uint32_t *src = s_bins + (r * kSahBuckets + b) * kSahBinWords;
        if (s >= 0 && src[6] > 0) {
          uint32_t *d = bins + ((int64_t)s * kSahBuckets + b) * kSahBinWords + w;
          if (w < 3) atomicMin(d, src[w]);
          else if (w < 6) atomicMax(d, src[w]);
          else atomicAdd(d, src[w]);
        }
      }
    }
    __syncthreads();
  }
}

// One thread per node of the level: split decision, node record, children.
__global__ void k_sah_split(SahNode *list_in, int n_in, const uint32_t *__restrict__ bins_in, int level,
                            SahNode *list_out, int32_t *cnt_out, uint32_t *bins_out, int64_t cap, int4 *fin,
                            int32_t *cnt_fin, int64_t fin_cap, Node2 *__restrict__ nodes, uint32_t *err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_in; s += gridDim.x * blockDim.x) {
    const SahNode N = list_in[s];
    const int first = N.r.x, count = N.r.y, slot = N.r.z, mode = N.r.w;
    const uint32_t *B = bins_in + (int64_t)s * kSahBuckets * kSahBinWords;
    float blo[kSahBuckets][3], bhi[kSahBuckets][3];
    int bc[kSahBuckets];
    for (int k = 0; k < kSahBuckets; ++k) {
      const uint4 v0 = *(const uint4 *)(B + k * kSahBinWords), v1 = *(const uint4 *)(B + k * kSahBinWords + 4);
      blo[k][0] = fkey_inv(v0.x);
      blo[k][1] = fkey_inv(v0.y);
      blo[k][2] = fkey_inv(v0.z);
      bhi[k][0] = fkey_inv(v0.w);
      bhi[k][1] = fkey_inv(v1.x);
      bhi[k][2] = fkey_inv(v1.y);
      bc[k] = (int)v1.z;
    }
    float llo[3], lhi[3], rlo[3], rhi[3];
    int nl = -1, bucket = -1;
    if (mode == kModeHalves) {
      nl = count >> 1;
      for (int a = 0; a < 3; ++a) {
        llo[a] = blo[0][a];
        lhi[a] = bhi[0][a];
        rlo[a] = blo[kSahBuckets - 1][a];
        rhi[a] = bhi[kSahBuckets - 1][a];
      }
    } else {
      // Suffix unions R_i (base_bvh.cpp:131-136); prefix unions L_i run
      // along the cost loop (:124-129, :138-152).
      float slo[kSahBuckets][3], shi[kSahBuckets][3];
      int sc[kSahBuckets];
      for (int a = 0; a < 3; ++a) {
        slo[kSahBuckets - 1][a] = blo[kSahBuckets - 1][a];
        shi[kSahBuckets - 1][a] = bhi[kSahBuckets - 1][a];
      }
      sc[kSahBuckets - 1] = bc[kSahBuckets - 1];
      for (int k = kSahBuckets - 2; k >= 0; --k) {
        for (int a = 0; a < 3; ++a) {
          slo[k][a] = fminf(slo[k + 1][a], blo[k][a]);
          shi[k][a] = fmaxf(shi[k + 1][a], bhi[k][a]);
        }
        sc[k] = sc[k + 1] + bc[k];
      }
      const float nlo[3] = {N.lo.x, N.lo.y, N.lo.z}, nhi[3] = {N.hi.x, N.hi.y, N.hi.z};
      const float sap = sah_area(nlo, nhi);
      float plo[3], phi[3];
      int pc = bc[0];
      for (int a = 0; a < 3; ++a) {
        plo[a] = blo[0][a];
        phi[a] = bhi[0][a];
      }
      float best = FLT_MAX;
      for (int i = 1; i < kSahBuckets - 1; ++i) {
        for (int a = 0; a < 3; ++a) {
          plo[a] = fminf(plo[a], blo[i][a]);
          phi[a] = fmaxf(phi[a], bhi[i][a]);
        }
        pc += bc[i];
        const float q = __fdiv_rn(__fadd_rn(__fmul_rn(sah_area(plo, phi), (float)pc),
                                            __fmul_rn(sah_area(slo[i + 1], shi[i + 1]), (float)sc[i + 1])),
                                  sap);
        const float cost = __double2float_rn(__dadd_rn(0.125, (double)q));
        if (cost < best) {
          best = cost;
          bucket = i;
          nl = pc;
          for (int a = 0; a < 3; ++a) {
            llo[a] = plo[a];
            lhi[a] = phi[a];
            rlo[a] = slo[i + 1][a];
            rhi[a] = shi[i + 1][a];
          }
        }
      }
      if (!(best < (float)count)) nl = -1;  // no split below the leaf cost: a leaf
      if (nl <= 0 || nl >= count) nl = -1;  // only reachable from corrupted bins
    }
    if (nl < 0) {
      // A leaf of more than 8 triangles: halves from the next level on, or
      // finished at once when small.
      int next = -1;
      const float nlo[3] = {N.lo.x, N.lo.y, N.lo.z}, nhi[3] = {N.hi.x, N.hi.y, N.hi.z};
      if (count <= kSahFinishMax)
        sah_finish_item(fin, cnt_fin, fin_cap, first, count, slot, err);
      else
        next = sah_queue(list_out, cnt_out, cap, bins_out, nlo, nhi, first, count, slot, kModeHalves, err);
      list_in[s].s = make_int4(-1, -1, next, -1);
      continue;
    }
    const int last = first + count - 1, m = first + nl, nr = count - nl;
    Node2 nd;
    nd.a = make_float4(llo[0], lhi[0], llo[1], lhi[1]);
    nd.b = make_float4(rlo[0], rhi[0], rlo[1], rhi[1]);
    nd.c = make_float4(llo[2], lhi[2], rlo[2], rhi[2]);
    nd.d = make_int4(nl == 1 ? ~first : m - 1, nr == 1 ? ~m : m, first, last);
    nodes[slot] = nd;
    int child[2] = {-1, -1};
    for (int k = 0; k < 2; ++k) {
      const int cf = k ? m : first, cc = k ? nr : nl, cs = k ? m : m - 1;
      if (cc < 2) continue;
      const bool bins_mode = mode == kModeBins && cc > kSahLeafMax && level + 1 < kSahDepthMax;
      if (!bins_mode && cc <= kSahFinishMax) {
        sah_finish_item(fin, cnt_fin, fin_cap, cf, cc, cs, err);
      } else {
        child[k] = sah_queue(list_out, cnt_out, cap, bins_out, k ? rlo : llo, k ? rhi : lhi, cf, cc, cs,
                             bins_mode ? kModeBins : kModeHalves, err);
      }
    }
    list_in[s].s = make_int4(nl, bucket, child[0], child[1]);
  }
}

// 1 where a position goes to its node's left child this level.
__global__ void k_sah_flags(const float4 *__restrict__ cen, const int32_t *__restrict__ seg, int64_t n,
                            const SahNode *__restrict__ list, int axis, int32_t *__restrict__ flag) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int s = seg[p];
    int f = 0;
    if (s >= 0) {
      const SahNode N = list[s];
      if (N.s.x >= 0) {
        if (N.r.w == kModeHalves) f = (p - N.r.x) < N.s.x ? 1 : 0;
        else f = sah_bucket(comp(cen[p], axis), comp(N.lo, axis), comp(N.hi, axis)) <= N.s.y ? 1 : 0;
      }
    }
    flag[p] = f;
  }
}

// Stable partition of every split node: left positions keep their order at
// the front, right ones after them.  scan / tsum: exclusive scan of flag in
// tiles of kFlagScanTile plus the scanned tile sums.
__global__ void k_sah_scatter(const float4 *__restrict__ box_in, const float4 *__restrict__ cen_in,
                              const int32_t *__restrict__ seg_in, int64_t n, const SahNode *__restrict__ list,
                              const int32_t *__restrict__ flag, const int32_t *__restrict__ scan,
                              const int32_t *__restrict__ tsum, float4 *__restrict__ box_out,
                              float4 *__restrict__ cen_out, int32_t *__restrict__ seg_out,
                              const float *__restrict__ pos, const int32_t *__restrict__ idx,
                              const int64_t *__restrict__ tri_off, int n_scenes, uint32_t *__restrict__ perm,
                              TriRec *__restrict__ tris, uint32_t *err) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int s = seg_in[p];
    if (s < 0) {
      seg_out[p] = -1;
      continue;
    }
    const SahNode N = list[s];
    const int64_t first = N.r.x, count = N.r.y;
    int64_t q = p;
    int ns = N.s.z;
    if (N.s.x >= 0) {
      const int64_t rl = (int64_t)(scan[p] + tsum[p / kFlagScanTile]) -
                         (int64_t)(scan[first] + tsum[first / kFlagScanTile]);
      const bool left = flag[p] != 0;
      q = left ? first + rl : first + N.s.x + (p - first - rl);
      ns = left ? N.s.z : N.s.w;
    }
    if (q < first || q >= first + count) {
      atomicOr(err, kErrQueue);
      q = p;
    }
    const float4 c = cen_in[p];
    box_out[2 * q] = box_in[2 * p];
    box_out[2 * q + 1] = box_in[2 * p + 1];
    cen_out[q] = c;
    seg_out[q] = ns;
    if (ns < 0) sah_final(pos, idx, tri_off, n_scenes, q, (int64_t)__float_as_int(c.w), perm, tris);
  }
}

// Balanced binary subtree (left part floor(k / 2)) over each finished range
// of k = 2..32 positions, whose boxes are in `box`.
__global__ void k_sah_finish(const int4 *__restrict__ fin, const int32_t *__restrict__ cnt_fin, int64_t fin_cap,
                             int64_t n, const float4 *__restrict__ box, Node2 *__restrict__ nodes, uint32_t *err) {
  // The counter runs past the capacity when the list overflowed (error set).
  const int nf = (int)min((int64_t)*cnt_fin, fin_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
    const int4 it = fin[i];
    if (it.y < 2 || it.y > kSahFinishMax || it.x < 0 || (int64_t)it.x + it.y > n || it.z < it.x ||
        it.z >= it.x + it.y) {
      atomicOr(err, kErrQueue);
      continue;
    }
    int3 stk[8];  // (first, count, slot); depth <= log2(32) + 1
    int sp = 0;
    stk[sp++] = make_int3(it.x, it.y, it.z);
    while (sp > 0) {
      const int3 t = stk[--sp];
      const int h = t.y >> 1, m = t.x + h, nr = t.y - h;
      float lo[2][3], hi[2][3];
      for (int k = 0; k < 2; ++k) {
        const int a = k ? m : t.x, e = k ? t.x + t.y : m;
        for (int c = 0; c < 3; ++c) {
          lo[k][c] = FLT_MAX;
          hi[k][c] = -FLT_MAX;
        }
        for (int j = a; j < e; ++j) {
          const float4 bl = box[2 * (int64_t)j], bh = box[2 * (int64_t)j + 1];
          lo[k][0] = fminf(lo[k][0], bl.x);
          lo[k][1] = fminf(lo[k][1], bl.y);
          lo[k][2] = fminf(lo[k][2], bl.z);
          hi[k][0] = fmaxf(hi[k][0], bh.x);
          hi[k][1] = fmaxf(hi[k][1], bh.y);
          hi[k][2] = fmaxf(hi[k][2], bh.z);
        }
      }
      Node2 nd;
      nd.a = make_float4(lo[0][0], hi[0][0], lo[0][1], hi[0][1]);
      nd.b = make_float4(lo[1][0], hi[1][0], lo[1][1], hi[1][1]);
      nd.c = make_float4(lo[0][2], hi[0][2], lo[1][2], hi[1][2]);
      nd.d = make_int4(h == 1 ? ~t.x : m - 1, nr == 1 ? ~m : m, t.x, t.x + t.y - 1);
      nodes[t.z] = nd;
      if (h >= 2 && sp < 8) stk[sp++] = make_int3(t.x, h, m - 1);
      if (nr >= 2 && sp < 8) stk[sp++] = make_int3(m, nr, m);
    }
  }
}

int sah_reserve(flg_bvh b) {
  const int64_t n = b->n_tri;
  b->sah_cap = n / (kSahLeafMax + 1) + b->n_scenes + 1;
  b->sah_fin_cap = n / 2 + b->n_scenes + 1;
  int rc = FLG_OK;
  auto A = [&](auto **p, size_t c) {
    if (rc == FLG_OK) rc = halloc(b, p, c);
  };
  for (int k = 0; k < 2; ++k) {
    A(&b->d_sbox[k], 2 * (size_t)n);
    A(&b->d_scen[k], (size_t)n);
    A(&b->d_sseg[k], (size_t)n);
    A((SahNode **)&b->d_slist[k], (size_t)b->sah_cap);
    A(&b->d_sbins[k], (size_t)b->sah_cap * kSahBuckets * kSahBinWords);
  }
  A(&b->d_sfin, (size_t)b->sah_fin_cap);
  A(&b->d_sflag, (size_t)n);
  A(&b->d_sscan, (size_t)n);
  A(&b->d_ssum, (size_t)ceil_div(n, kFlagScanTile) + 1);
  A(&b->d_sctr, 4);
  A(&b->d_sroot, (size_t)b->n_scenes);
  return rc;
}

int sah_build(flg_ctx ctx, flg_bvh b) {
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "a SAH build synchronises with the host; not capturable");
  cudaStream_t st = ctx->stream;
  const int64_t n = b->n_tri;
  if (n <= 0) return FLG_OK;
  SahNode *list[2] = {(SahNode *)b->d_slist[0], (SahNode *)b->d_slist[1]};
  int32_t *ctr = b->d_sctr;  // [0], [1] list sizes; [2] finish items; [3] scan total
  const unsigned g_elem = grid_for(n, 256, (int64_t)ctx->num_sms * 16);
  const unsigned g_fin = grid_for(b->sah_fin_cap, 128, (int64_t)ctx->num_sms * 8);
  FLG_CUDA(ctx, cudaMemsetAsync(ctr, 0, 4 * sizeof(int32_t), st));
  // Every level rewrites every position's list index; starting both buffers
  // at -1 keeps even a corrupted level's stale entries inside the list.
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_sseg[1], 0xFF, sizeof(int32_t) * (size_t)n, st));
  k_sah_roots<<<grid_for(b->n_scenes, 128), 128, 0, st>>>(b->d_tri_off, b->n_scenes, b->d_scene_box, list[0], ctr,
                                                          b->sah_cap, b->d_sbins[0], b->d_sfin, ctr + 2,
                                                          b->sah_fin_cap, b->d_sroot, ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_sah_roots");
  k_sah_init<<<g_elem, 256, 0, st>>>(b->pos, b->idx, n, b->d_tri_off, b->n_scenes, b->d_sroot, b->d_sbox[0],
                                     b->d_scen[0], b->d_sseg[0], b->d_perm, b->d_tris);
  FLG_LAUNCH_CHECK(ctx, "k_sah_init");
  k_sah_finish<<<g_fin, 128, 0, st>>>(b->d_sfin, ctr + 2, b->sah_fin_cap, n, b->d_sbox[0], b->d_nodes2,
                                      ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_sah_finish");
  int32_t h_cnt = 0;
  FLG_CUDA(ctx, cudaMemcpyAsync(&h_cnt, ctr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  FLG_CUDA(ctx, cudaStreamSynchronize(st));
  const int nt = (int)ceil_div(n, kFlagScanTile);
  int cur = 0;
  for (int level = 0; h_cnt > 0; ++level) {
    if (level >= kSahMaxLevels || h_cnt > b->sah_cap)
      return set_error(ctx, FLG_ERR_STATE, "SAH build did not finish (level %d, %d nodes)", level, h_cnt);
    const int nxt = cur ^ 1;
    FLG_CUDA(ctx, cudaMemsetAsync(ctr + nxt, 0, sizeof(int32_t), st));
    FLG_CUDA(ctx, cudaMemsetAsync(ctr + 2, 0, sizeof(int32_t), st));
    const int axis = level % 3;
    k_sah_bin<<<grid_for(n, kSahChunk, (int64_t)ctx->num_sms * 8), kSahBinThreads, 0, st>>>(
        b->d_sbox[cur], b->d_scen[cur], b->d_sseg[cur], n, list[cur], b->d_sbins[cur], axis);
    FLG_LAUNCH_CHECK(ctx, "k_sah_bin");
    k_sah_split<<<grid_for(h_cnt, 128), 128, 0, st>>>(list[cur], h_cnt, b->d_sbins[cur], level, list[nxt], ctr + nxt,
                                                      b->d_sbins[nxt], b->sah_cap, b->d_sfin, ctr + 2,
                                                      b->sah_fin_cap, b->d_nodes2, ctx->d_err);
    FLG_LAUNCH_CHECK(ctx, "k_sah_split");
    k_sah_flags<<<g_elem, 256, 0, st>>>(b->d_scen[cur], b->d_sseg[cur], n, list[cur], axis, b->d_sflag);
    FLG_LAUNCH_CHECK(ctx, "k_sah_flags");
    k_scan_tiles<<<nt, kFlagScanThreads, 0, st>>>(b->d_sflag, (int)n, b->d_sscan, b->d_ssum);
    FLG_LAUNCH_CHECK(ctx, "k_scan_tiles");
    k_scan_sums<<<1, 1024, 0, st>>>(b->d_ssum, nt, ctr + 3);
    FLG_LAUNCH_CHECK(ctx, "k_scan_sums");
    k_sah_scatter<<<g_elem, 256, 0, st>>>(b->d_sbox[cur], b->d_scen[cur], b->d_sseg[cur], n, list[cur],
                                          b->d_sflag, b->d_sscan, b->d_ssum, b->d_sbox[nxt], b->d_scen[nxt],
                                          b->d_sseg[nxt], b->pos, b->idx, b->d_tri_off, b->n_scenes, b->d_perm,
                                          b->d_tris, ctx->d_err);
    FLG_LAUNCH_CHECK(ctx, "k_sah_scatter");
    k_sah_finish<<<g_fin, 128, 0, st>>>(b->d_sfin, ctr + 2, b->sah_fin_cap, n, b->d_sbox[nxt], b->d_nodes2,
                                        ctx->d_err);
    FLG_LAUNCH_CHECK(ctx, "k_sah_finish");
    FLG_CUDA(ctx, cudaMemcpyAsync(&h_cnt, ctr + nxt, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(ctx, cudaStreamSynchronize(st));
    cur = nxt;
  }
  stage_mark(ctx, st, "sah_levels");
  return FLG_OK;
}

}  // namespace flg
