// treelet.cu — treelet restructuring of the LBVH (FLG_BUILDER_TREELET):
// Karras & Aila, "Fast Parallel Construction of High-Quality Bounding Volume
// Hierarchies" (HPG 2013).  No counterpart in the reference, whose quality
// builder is the binned SAH of base_bvh.cpp:33-173; this is the LBVH
// refinement that trades build time for trace speed.
//
// After the Karras build (k_climb) the node records are turned into a working
// form (children, parents, leaf counts, boxes, SAH costs).  Each round (3 by
// default, 1 to 4) finishes every node (box, count, cost
// Ci A + C(left) + C(right), A = dx dy + dy dz + dz dx) after its whole
// subtree and, when the subtree holds at least 7 << round triangles, rebuilds
// the treelet of its 7 largest descendants (the treelet leaf of largest area
// is opened until 7 leaves; ties to the first in list order) into the
// topology of least SAH cost by dynamic programming over the 127 subsets of
// the treelet's leaves (splits holding the lowest member, enumerated from
// S - 1 downwards, first minimum kept).  The order is by height: a pass from
// the leaves gives every node the height of its subtree, then one launch per
// height finishes (and rebuilds) the nodes of that height.  Nodes of one
// height lie in disjoint subtrees, and everything below them was finished by
// earlier launches, so the result does not depend on scheduling and no fence
// or arrival protocol is needed.
// Then every node finds its first leaf in depth-first order by climbing to
// its root, the leaves and triangle records are regathered in that order and
// the node records are rewritten in Karras' numbering (root at the scene's
// first slot, a left child at its last position, a right child at its
// first), so traversal, the wide collapse and flg_bvh_download read the tree
// as they read an LBVH.  Morton codes no longer follow the leaf order.
#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr float kTlCi = 1.2f, kTlCt = 1.0f;
constexpr int kTreelet = 7, kTlFull = (1 << kTreelet) - 1;
constexpr int kTlThreads = 128;

struct TlBox {
  float lo[3], hi[3];
};

__device__ __forceinline__ float tl_area(const TlBox &b) {
  const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}
__device__ __forceinline__ void tl_merge(TlBox &a, const TlBox &b) {
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = fminf(a.lo[k], b.lo[k]);
    a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
}

// Heights are below this bound: a valid tree is at most 62 levels deep
// after the LBVH build, and a round rebuilds treelets of 7 leaves.
constexpr int kTlMaxHeight = 128;

// Subsets of the 7 treelet leaves ordered by size: kTlCount[k] subsets of
// size k from kTlOffset[k].
__constant__ uint8_t kTlSubsets[kTlFull] = {
    1,   2,   4,   8,   16,  32,  64,  3,   5,   6,   9,   10,  12,  17,  18,  20,  24,  33,  34,  36,  40,  48,
    65,  66,  68,  72,  80,  96,  7,   11,  13,  14,  19,  21,  22,  25,  26,  28,  35,  37,  38,  41,  42,  44,
    49,  50,  52,  56,  67,  69,  70,  73,  74,  76,  81,  82,  84,  88,  97,  98,  100, 104, 112, 15,  23,  27,
    29,  30,  39,  43,  45,  46,  51,  53,  54,  57,  58,  60,  71,  75,  77,  78,  83,  85,  86,  89,  90,  92,
    99,  101, 102, 105, 106, 108, 113, 114, 116, 120, 31,  47,  55,  59,  61,  62,  79,  87,  91,  93,  94,  103,
    107, 109, 110, 115, 117, 118, 121, 122, 124, 63,  95,  111, 119, 123, 125, 126, 127};
__constant__ int kTlCount[kTreelet + 1] = {0, 7, 21, 35, 35, 21, 7, 1};
__constant__ int kTlOffset[kTreelet + 1] = {0, 0, 7, 28, 63, 98, 119, 126};

// The bits of t deposited, lowest first, at the set bits of mask.
__device__ __forceinline__ int tl_deposit(int t, int mask) {
  int q = 0;
  for (; mask; mask &= mask - 1, t >>= 1)
    if (t & 1) q |= mask & -mask;
  return q;
}

// One warp's treelet in shared memory: the leaves' boxes, costs and counts,
// every subset's area, least cost and split, the grown L / I lists and the
// rebuilt internal nodes.
struct TlWarp {
  float lo[kTreelet][3], hi[kTreelet][3];
  float c[kTlFull + 1], area[kTlFull + 1];
  int32_t ln[kTreelet], L[kTreelet], I[kTreelet - 1], order[kTreelet - 1];
  int orderS[kTreelet - 1];
  uint8_t part[kTlFull + 1];

  // union of the leaves of S: the lowest first, then every member in order
  __device__ __forceinline__ TlBox uni(int S) const {
    const int f = __ffs(S) - 1;
    TlBox u;
    for (int q = 0; q < 3; ++q) {
      u.lo[q] = lo[f][q];
      u.hi[q] = hi[f][q];
    }
    for (int k = 0; k < kTreelet; ++k)
      if ((S >> k) & 1)
        for (int q = 0; q < 3; ++q) {
          u.lo[q] = fminf(u.lo[q], lo[k][q]);
          u.hi[q] = fmaxf(u.hi[q], hi[k][q]);
        }
    return u;
  }
};

// Working form: per node slot children (>= 0 node slot, < 0 ~sorted leaf),
// parent (-1 at a root), leaf count, SAH cost, box; per leaf its parent.
// Reads of what other threads write go through L2 (__ldcg): L1 is not
// coherent across SMs.
struct Tl {
  int32_t *left, *right, *parent, *nleaf, *first, *slot;
  uint32_t *hw;  // per node: both children's heights + 1 and arrival bits; then per height counts, starts, cursors
  float *cost;
  float4 *box;  // 2 per node: lo.xyz, hi.xyz
  int32_t *lpar, *lpos;
  const TriRec *tris;

  __device__ __forceinline__ TlBox leaf_box(int32_t pos) const {
    const TriRec t = tris[pos];
    TlBox b;
    b.lo[0] = fminf(fminf(t.p0.x, t.p1.x), t.p2.x);
    b.lo[1] = fminf(fminf(t.p0.y, t.p1.y), t.p2.y);
    b.lo[2] = fminf(fminf(t.p0.z, t.p1.z), t.p2.z);
    b.hi[0] = fmaxf(fmaxf(t.p0.x, t.p1.x), t.p2.x);
    b.hi[1] = fmaxf(fmaxf(t.p0.y, t.p1.y), t.p2.y);
    b.hi[2] = fmaxf(fmaxf(t.p0.z, t.p1.z), t.p2.z);
    return b;
  }
  __device__ __forceinline__ TlBox bx(int32_t r) const {
    if (r < 0) return leaf_box(~r);
    const float4 a = __ldcg(box + 2 * r), b = __ldcg(box + 2 * r + 1);
    TlBox o;
    o.lo[0] = a.x; o.lo[1] = a.y; o.lo[2] = a.z;
    o.hi[0] = b.x; o.hi[1] = b.y; o.hi[2] = b.z;
    return o;
  }
  __device__ __forceinline__ float cs(int32_t r) const {
    return r < 0 ? kTlCt * tl_area(leaf_box(~r)) : __ldcg(cost + r);
  }
  __device__ __forceinline__ int32_t nl(int32_t r) const { return r < 0 ? 1 : __ldcg(nleaf + r); }
  __device__ __forceinline__ void set_parent(int32_t r, int32_t p) const {
    if (r >= 0) parent[r] = p;
    else lpar[~r] = p;
  }
  __device__ __forceinline__ void store(int32_t x, const TlBox &b, float c, int32_t n) const {
    box[2 * x] = make_float4(b.lo[0], b.lo[1], b.lo[2], 0.0f);
    box[2 * x + 1] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.0f);
    cost[x] = c;
    nleaf[x] = n;
  }

  __device__ int32_t finish(int32_t x) const {
    const int32_t l = __ldcg(left + x), r = __ldcg(right + x);
    TlBox b = bx(l);
    tl_merge(b, bx(r));
    const int32_t n = nl(l) + nl(r);
    store(x, b, kTlCi * tl_area(b) + (cs(l) + cs(r)), n);
    return n;
  }

  // Rebuilds the treelet rooted at R with the whole warp (R uniform, every
  // lane calls).  Decisions equal the serial rule: the growing picks the
  // first treelet leaf of largest area, a subset's split is the first
  // minimum in the order P = (S - 1) & S downwards; lanes split the
  // candidates and reduce (cost, position in that order).
  __device__ void restructure(int32_t R, TlWarp &w, int lane) const {
    if (lane == 0) {
      w.L[0] = __ldcg(left + R);
      w.L[1] = __ldcg(right + R);
      w.I[0] = R;
    }
    __syncwarp();
    for (int nL = 2; nL < kTreelet; ++nL) {
      const int32_t mine = lane < nL ? w.L[lane] : -1;
      float a = -2.0f;
      int k = 32;
      if (mine >= 0) {
        const float v = tl_area(bx(mine));
        if (v > -1.0f) {
          a = v;
          k = lane;
        }
      }
      for (int o = 4; o; o >>= 1) {
        const float oa = __shfl_xor_sync(0xffffffffu, a, o);
        const int ok = __shfl_xor_sync(0xffffffffu, k, o);
        if (oa > a || (oa == a && ok < k)) {
          a = oa;
          k = ok;
        }
      }
      k = __shfl_sync(0xffffffffu, k, 0);
      if (k == 32) return;  // every treelet leaf is a triangle
      __syncwarp();
      if (lane == 0) {
        const int32_t x = w.L[k];
        w.I[nL - 1] = x;
        w.L[k] = __ldcg(left + x);
        w.L[nL] = __ldcg(right + x);
      }
      __syncwarp();
    }
    if (lane < kTreelet) {
      const int32_t r = w.L[lane];
      const TlBox b = bx(r);
      for (int q = 0; q < 3; ++q) {
        w.lo[lane][q] = b.lo[q];
        w.hi[lane][q] = b.hi[q];
      }
      w.c[1 << lane] = cs(r);
      w.part[1 << lane] = 0;
      w.ln[lane] = nl(r);
    }
    __syncwarp();
    for (int S = lane + 1; S <= kTlFull; S += 32) w.area[S] = tl_area(w.uni(S));
    __syncwarp();
    // sizes 2..7: 21, 35, 35, 21, 7, 1 subsets; 1, 1, 1, 1, 4, 32 lanes each
    for (int k = 2; k <= kTreelet; ++k) {
      const int m = kTlCount[k], g = k == 7 ? 32 : k == 6 ? 4 : 1, np = (1 << (k - 1)) - 1;
      for (int base = 0; base < m; base += 32 / g) {
        const int si = base + lane / g, r = lane % g;
        const bool ok = si < m;
        const int S = ok ? (int)kTlSubsets[kTlOffset[k] + si] : 0;
        const int low = S & -S, rest = S ^ low;
        float best = 3.402823466e+38f;
        int bj = np, bp = 0;
        if (ok) {
          // The j-th split holding `low` is low | Q, Q the (np - 1 - j)-th
          // subset of rest; Q = (Q - 1) & rest steps to the next j.
          int Q = tl_deposit(np - 1 - r, rest);
          for (int j = r; j < np; j += g) {
            const int P = low | Q;
            const float v = w.c[P] + w.c[S ^ P];
            if (v < best) {
              best = v;
              bj = j;
              bp = P;
            }
            if (g == 32) {
              Q = tl_deposit(np - 1 - (j + g), rest);
            } else {
              for (int q = 0; q < g; ++q) Q = (Q - 1) & rest;
            }
          }
        }
        for (int o = g >> 1; o; o >>= 1) {
          const float ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
          const int op = __shfl_xor_sync(0xffffffffu, bp, o);
          if (ob < best || (ob == best && oj < bj)) {
            best = ob;
            bj = oj;
            bp = op;
          }
        }
        if (ok && r == 0) {
          w.c[S] = kTlCi * w.area[S] + best;
          w.part[S] = (uint8_t)bp;
        }
      }
      __syncwarp();
    }
    // Rebuild: internal nodes taken from I as their parents are expanded
    // (left child first), expansion by a stack with the left subtree on top.
    if (lane == 0) {
      int next = 1, sp = 0, no = 0;
      int stS[kTreelet];
      int32_t stN[kTreelet];
      stS[sp] = kTlFull;
      stN[sp++] = R;
      while (sp) {
        --sp;
        const int S = stS[sp];
        const int32_t node = stN[sp];
        w.order[no] = node;
        w.orderS[no++] = S;
        const int P = w.part[S], Q = S ^ P;
        const int32_t c0 = __popc(P) == 1 ? w.L[__ffs(P) - 1] : w.I[next++];
        const int32_t c1 = __popc(Q) == 1 ? w.L[__ffs(Q) - 1] : w.I[next++];
        left[node] = c0;
        right[node] = c1;
        set_parent(c0, node);
        set_parent(c1, node);
        if (__popc(Q) > 1) {
          stS[sp] = Q;
          stN[sp++] = c1;
        }
        if (__popc(P) > 1) {
          stS[sp] = P;
          stN[sp++] = c0;
        }
      }
    }
    __syncwarp();
    // boxes, counts and costs of the treelet's six internal nodes
    if (lane < kTreelet - 1) {
      const int S = w.orderS[lane];
      int32_t n = 0;
      for (int j = 0; j < kTreelet; ++j)
        if ((S >> j) & 1) n += w.ln[j];
      store(w.order[lane], w.uni(S), w.c[S], n);
    }
    __syncwarp();
  }
};

// A child ref of a node of the scene [toff, toff + n): a node slot in
// [toff, toff + n - 1) or ~position in [toff, toff + n).
__device__ __forceinline__ bool tl_ref_ok(int32_t r, int64_t toff, int64_t n) {
  return r >= 0 ? (r >= toff && r < toff + n - 1) : (~r >= toff && ~r < toff + n);
}

__global__ void __launch_bounds__(256)
    k_tl_init(const Node2 *__restrict__ nodes, int64_t n_nodes, const int64_t *__restrict__ tri_off, int n_scenes,
              Tl T, uint32_t *err) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, g);
    const int64_t toff = tri_off[s], n = tri_off[s + 1] - toff;
    if (g >= toff + n - 1) continue;  // a scene's last slot is unused
    const int4 d = nodes[g].d;
    // only a build whose bounded waits gave up leaves refs outside the scene
    if (!tl_ref_ok(d.x, toff, n) || !tl_ref_ok(d.y, toff, n)) {
      atomicOr(err, kErrTimeout);
      T.left[g] = T.right[g] = ~(int32_t)toff;
      continue;
    }
    T.left[g] = d.x;
    T.right[g] = d.y;
    T.set_parent(d.x, (int32_t)g);
    T.set_parent(d.y, (int32_t)g);
  }
}

// Height of every node (a leaf's is 0) for the order of a round.  A thread
// per leaf climbs; each child ORs its height + 1 and its side's bit into the
// parent's word (bits 0-7 and 16 from the left child, 8-15 and 17 from the
// right); the second arrival reads its sibling's height from the value the
// OR returns and climbs on with the larger.  Everything travels in the
// atomic word, so relaxed atomics suffice.
__global__ void __launch_bounds__(256)
    k_tl_height(int64_t n_tri, Tl T, uint32_t *hw) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n_tri;
       pos += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = ~(int32_t)pos, x = __ldcg(T.lpar + pos);
    uint32_t h = 0;
    for (int depth = 0; x >= 0 && depth < kTlMaxHeight - 1; ++depth) {
      const bool lft = __ldcg(T.left + x) == c;
      const uint32_t old = atomicOr(hw + x, lft ? ((h + 1) | 0x10000u) : (((h + 1) << 8) | 0x20000u));
      if (!(old & (lft ? 0x20000u : 0x10000u))) break;  // first arrival
      h = max(h + 1, lft ? (old >> 8) & 0xFFu : old & 0xFFu);
      c = x;
      x = __ldcg(T.parent + x);
    }
  }
}

// Height of a node from its word; 0 unless both children arrived (a scene's
// unused last slot, a node of an inconsistent tree).
__device__ __forceinline__ uint32_t tl_height(uint32_t v) {
  return (v & 0x30000u) == 0x30000u ? max(v & 0xFFu, (v >> 8) & 0xFFu) : 0u;
}

// Nodes listed by height (counting sort; the order within a height does not
// matter): per-block counts, one global add per height and block.
// `hc` = count[kTlMaxHeight], start[kTlMaxHeight], cursor[kTlMaxHeight].
__global__ void __launch_bounds__(256)
    k_tl_hcount(int64_t n_nodes, const uint32_t *__restrict__ hw, uint32_t *hc) {
  __shared__ uint32_t cnt[kTlMaxHeight];
  for (int t = threadIdx.x; t < kTlMaxHeight; t += blockDim.x) cnt[t] = 0u;
  __syncthreads();
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t h = tl_height(hw[g]);
    if (h) atomicAdd(cnt + h, 1u);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kTlMaxHeight; t += blockDim.x)
    if (cnt[t]) atomicAdd(hc + t, cnt[t]);
}

__global__ void k_tl_hscan(uint32_t *hc) {
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int h = 0; h < kTlMaxHeight; ++h) {
      hc[kTlMaxHeight + h] = hc[2 * kTlMaxHeight + h] = run;
      run += hc[h];
    }
  }
}

// Same slices as k_tl_hcount: a block reserves its range per height with
// one global add, then places its nodes through shared cursors.
__global__ void __launch_bounds__(256)
    k_tl_hplace(int64_t n_nodes, const uint32_t *__restrict__ hw, uint32_t *hc, int32_t *__restrict__ list) {
  __shared__ uint32_t cnt[kTlMaxHeight];
  for (int t = threadIdx.x; t < kTlMaxHeight; t += blockDim.x) cnt[t] = 0u;
  __syncthreads();
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t h = tl_height(hw[g]);
    if (h) atomicAdd(cnt + h, 1u);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kTlMaxHeight; t += blockDim.x)
    if (cnt[t]) cnt[t] = atomicAdd(hc + 2 * kTlMaxHeight + t, cnt[t]);
  __syncthreads();
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t h = tl_height(hw[g]);
    if (h) list[atomicAdd(cnt + h, 1u)] = (int32_t)g;
  }
}

// One height of a round: every node of height h is finished; those whose
// subtree holds >= gamma triangles are then rebuilt by the whole warp, one
// after the other.  Their children were finished by earlier launches.  The
// list is dealt to the warps round robin (entry i to warp i mod W), so that a
// short list gives each warp at most one rebuild instead of leaving a few
// warps with 32 each.
__global__ void __launch_bounds__(kTlThreads)
    k_tl_wave(uint32_t h, int32_t gamma, Tl T, const uint32_t *__restrict__ hc, const int32_t *__restrict__ list) {
  const int64_t m = hc[h], first = hc[kTlMaxHeight + h];
  if (m == 0) return;
  __shared__ TlWarp warps[kTlThreads / 32];
  TlWarp &w = warps[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int64_t k = 0; wid + k * nw < m; k += 32) {
    const int64_t i = wid + (k + lane) * nw;
    const int32_t x = i < m ? list[first + i] : -1;
    const bool big = x >= 0 && T.finish(x) >= gamma;
    for (unsigned need = __ballot_sync(0xffffffffu, big); need; need &= need - 1)
      T.restructure(__shfl_sync(0xffffffffu, x, __ffs(need) - 1), w, lane);
  }
}

// Depth-first position of every node's first leaf (climb to the root adding
// the left siblings' leaf counts) and the internal nodes' Karras slots.
__global__ void __launch_bounds__(256)
    k_tl_first(int64_t n_nodes, int64_t n_tri, const int64_t *__restrict__ tri_off, int n_scenes, Tl T) {
  const int64_t total = n_nodes + n_tri;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const bool leaf = k >= n_nodes;
    const int64_t g = leaf ? k - n_nodes : k;
    const int s = find_segment(tri_off, n_scenes, g);
    const int64_t toff = tri_off[s];
    if (!leaf && g >= tri_off[s + 1] - 1) continue;
    int32_t x = leaf ? ~(int32_t)g : (int32_t)g;
    int32_t p = leaf ? T.lpar[g] : T.parent[g];
    int64_t f = 0;
    bool is_left = true;
    int depth = 0;
    for (int32_t c = x, q = p; q >= 0 && depth < 128; ++depth) {
      const bool right = T.right[q] == c;
      if (c == x) is_left = !right;
      if (right) f += T.left[q] < 0 ? 1 : T.nleaf[T.left[q]];
      c = q;
      q = T.parent[q];
    }
    const int64_t n = tri_off[s + 1] - toff;
    if (leaf) {
      T.lpos[g] = f < n ? (int32_t)(toff + f) : -1;
    } else {
      const int64_t last = f + T.nleaf[g] - 1;
      const int64_t sl = p < 0 ? 0 : is_left ? last : f;
      const bool ok = f >= 0 && last < n && sl < n - 1;
      T.first[g] = ok ? (int32_t)f : -1;
      T.slot[g] = ok ? (int32_t)(toff + sl) : -1;
    }
  }
}

__global__ void __launch_bounds__(256)
    k_tl_emit(int64_t n_nodes, const int64_t *__restrict__ tri_off, int n_scenes, Tl T, Node2 *__restrict__ out) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, g);
    const int64_t toff = tri_off[s];
    if (g >= tri_off[s + 1] - 1) continue;
    const int32_t l = T.left[g], r = T.right[g];
    if (T.slot[g] < 0) continue;  // an inconsistent tree (timed-out build): the flagged error stands
    const TlBox b0 = T.bx(l), b1 = T.bx(r);
    Node2 nd;
    nd.a = make_float4(b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
    nd.b = make_float4(b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
    nd.c = make_float4(b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
    const int32_t c0 = l < 0 ? ~T.lpos[~l] : T.slot[l];
    const int32_t c1 = r < 0 ? ~T.lpos[~r] : T.slot[r];
    const int32_t f = (int32_t)(toff + T.first[g]);
    nd.d = make_int4(c0, c1, f, f + T.nleaf[g] - 1);
    out[T.slot[g]] = nd;
  }
}

__global__ void __launch_bounds__(256)
    k_tl_leaves(int64_t n_tri, Tl T, const uint32_t *__restrict__ perm, uint32_t *__restrict__ perm_out,
                TriRec *__restrict__ tris_out) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n_tri;
       pos += (int64_t)gridDim.x * blockDim.x) {
    const int32_t np = T.lpos[pos];
    if (np < 0 || np >= n_tri) continue;
    perm_out[np] = perm[pos];
    tris_out[np] = T.tris[pos];
  }
}

static Tl tl_arrays(flg_bvh b) {
  Tl T;
  T.left = b->d_tl_i32;
  T.right = T.left + b->n_nodes;
  T.parent = T.right + b->n_nodes;
  T.nleaf = T.parent + b->n_nodes;
  T.first = T.nleaf + b->n_nodes;
  T.slot = T.first + b->n_nodes;
  T.lpar = T.slot + b->n_nodes;
  T.lpos = T.lpar + b->n_tri;
  T.hw = b->d_tl_flag;
  T.cost = b->d_tl_cost;
  T.box = b->d_tl_box;
  T.tris = b->d_tris;
  return T;
}

int treelet_reserve(flg_bvh b) {
  int rc = FLG_OK;
  auto A = [&](auto **p, size_t c) {
    if (rc == FLG_OK) rc = halloc(b, p, c);
  };
  A(&b->d_tl_i32, 6 * (size_t)b->n_nodes + 2 * (size_t)b->n_tri);
  A(&b->d_tl_flag, b->n_nodes + 3 * kTlMaxHeight);  // heights, then counts, starts, cursors per height
  A(&b->d_tl_cost, b->n_nodes);
  A(&b->d_tl_box, 2 * (size_t)b->n_nodes);
  A(&b->d_tl_nodes, b->n_nodes);
  A(&b->d_tl_tris, b->n_tri);
  A(&b->d_tl_perm, b->n_tri);
  return rc;
}

int treelet_build(flg_ctx ctx, flg_bvh b) {
  cudaStream_t st = ctx->stream;
  const int64_t n = b->n_tri, nn = b->n_nodes;
  if (n <= 1) return FLG_OK;
  Tl T = tl_arrays(b);
  // parents of roots (and of one-triangle scenes' leaves) stay -1
  FLG_CUDA(ctx, cudaMemsetAsync(T.parent, 0xFF, sizeof(int32_t) * (size_t)nn, st));
  FLG_CUDA(ctx, cudaMemsetAsync(T.lpar, 0xFF, sizeof(int32_t) * (size_t)n, st));
  const unsigned g = grid_for(nn, 256, (int64_t)ctx->num_sms * 8);
  k_tl_init<<<g, 256, 0, st>>>(b->d_nodes2, nn, b->d_tri_off, b->n_scenes, T, ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_tl_init");
  static const int wave_per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_tl_wave, kTlThreads, 0) != cudaSuccess || v < 1) v = 1;
    return v;
  }();
  const unsigned gw = grid_for(nn, kTlThreads, (int64_t)ctx->num_sms * wave_per_sm);
  const unsigned gn = grid_for(nn, 256, (int64_t)ctx->num_sms * 8);
  uint32_t *hc = T.hw + nn;
  int32_t *list = T.first;  // free until k_tl_first
  for (int r = 0; r < b->treelet_rounds; ++r) {
    // heights of the tree as the previous round left it, nodes listed by height
    FLG_CUDA(ctx, cudaMemsetAsync(T.hw, 0, sizeof(uint32_t) * ((size_t)nn + 3 * kTlMaxHeight), st));
    k_tl_height<<<grid_for(n, 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(n, T, T.hw);
    FLG_LAUNCH_CHECK(ctx, "k_tl_height");
    k_tl_hcount<<<gn, 256, 0, st>>>(nn, T.hw, hc);
    FLG_LAUNCH_CHECK(ctx, "k_tl_hcount");
    k_tl_hscan<<<1, 32, 0, st>>>(hc);
    FLG_LAUNCH_CHECK(ctx, "k_tl_hscan");
    k_tl_hplace<<<gn, 256, 0, st>>>(nn, T.hw, hc, list);
    FLG_LAUNCH_CHECK(ctx, "k_tl_hplace");
    // a fixed launch count keeps the build capturable; empty heights return
    // at once
    for (uint32_t h = 1; h < (uint32_t)kTlMaxHeight; ++h) {
      k_tl_wave<<<gw, kTlThreads, 0, st>>>(h, kTreelet << r, T, hc, list);
      FLG_LAUNCH_CHECK(ctx, "k_tl_wave");
    }
  }
  stage_mark(ctx, st, "treelet");
  k_tl_first<<<grid_for(nn + n, 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(nn, n, b->d_tri_off, b->n_scenes, T);
  FLG_LAUNCH_CHECK(ctx, "k_tl_first");
  stage_mark(ctx, st, "treelet_first");
  k_tl_emit<<<g, 256, 0, st>>>(nn, b->d_tri_off, b->n_scenes, T, b->d_tl_nodes);
  FLG_LAUNCH_CHECK(ctx, "k_tl_emit");
  k_tl_leaves<<<grid_for(n, 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(n, T, b->d_perm, b->d_tl_perm,
                                                                           b->d_tl_tris);
  FLG_LAUNCH_CHECK(ctx, "k_tl_leaves");
  FLG_CUDA(ctx, cudaMemcpyAsync(b->d_nodes2, b->d_tl_nodes, sizeof(Node2) * (size_t)nn, cudaMemcpyDeviceToDevice, st));
  FLG_CUDA(ctx, cudaMemcpyAsync(b->d_perm, b->d_tl_perm, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st));
  FLG_CUDA(ctx, cudaMemcpyAsync(b->d_tris, b->d_tl_tris, sizeof(TriRec) * (size_t)n, cudaMemcpyDeviceToDevice, st));
  stage_mark(ctx, st, "treelet_emit");
  return FLG_OK;
}

}  // namespace flg
