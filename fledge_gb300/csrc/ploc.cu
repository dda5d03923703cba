// ploc.cu — the high-quality tree builder next to the LBVH: parallel
// locally-ordered clustering (Meister & Bittner, "Parallel Locally-Ordered
// Clustering for Bounding Volume Hierarchy Construction", TVCG 2018) over the
// same Morton order as the Karras build.  It plays the role of the
// reference's SAH BasicBVHBuilder (src/experimental/base_bvh.cpp:33-188):
// slower to build than the LBVH, better trees for traversal.
//
//   k_ploc_init     one leaf cluster per sorted triangle (box, ref, count,
//                   scene)
//   per iteration   k_ploc_nn      nearest neighbour of every cluster among
//                                  the clusters within kPlocRadius positions
//                                  of the same scene, by the surface area of
//                                  the merged box (shared-memory window)
//                   k_ploc_merge   mutual nearest neighbours merge into a new
//                                  BVH2 node; the lower position keeps it
//                   scan + k_ploc_compact  drop the merged-away clusters
//   k_ploc_layout   top down, level by level: the leaf range of every node in
//                   depth-first order (left subtree first)
//   k_ploc_tris     triangles gathered into that order; k_ploc_fixrefs turns
//                   the nodes' leaf refs into positions of that order
//
// Node ids: the k-th merge of scene s takes node_off[s] + n_s - 2 - k, so the
// last merge — the root — lands on node_off[s], where the Karras root is;
// roots, wide roots and the collapse work unchanged.  Every subtree covers a
// contiguous range of the final triangle order, which the collapse turns into
// leaf ranges (rfirst / rcount instead of the Karras range ends).
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
static_assert(kScanThreads == kFlagScanThreads && kScanTile == kFlagScanTile, "flag scan shape");

__device__ __forceinline__ float merged_half_area(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  const float dx = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
  const float dy = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
  const float dz = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
  return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_init(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n,
                            const uint32_t *__restrict__ perm, const int64_t *__restrict__ tri_off, int n_scenes,
                            float4 *__restrict__ box, int32_t *__restrict__ ref, int32_t *__restrict__ cnt,
                            int32_t *__restrict__ scene) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, p);
    int64_t orig = perm[p];
    if (orig < 0 || orig >= n) orig = p;  // a timed-out sort (error word set): stay in bounds
    float3 a, b, c;
    tri_verts(pos, idx, orig, a, b, c);
    float lo[3], hi[3];
    tri_box(a, b, c, lo, hi);
    box[2 * p] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    box[2 * p + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    ref[p] = ~(int32_t)p;
    cnt[p] = 1;
    scene[p] = s;
  }
}

// Nearest neighbour within +-kPlocRadius positions (same scene); ties go to
// the lower position, and a NaN area counts as +inf.  -1 when no other
// cluster of the scene is in reach.  With this tie rule the closest reachable
// pair of a scene (lowest index first) is always mutual, so every iteration
// merges at least once in every unfinished scene.
__global__ void __launch_bounds__(kPlocThreads)
    k_ploc_nn(const float4 *__restrict__ box, const int32_t *__restrict__ scene, int n, int32_t *__restrict__ nn) {
  constexpr int kWin = kPlocThreads + 2 * kPlocRadius;
  __shared__ float4 s_lo[kWin], s_hi[kWin];
  __shared__ int32_t s_sc[kWin];
  const int base = blockIdx.x * kPlocThreads - kPlocRadius;
  for (int k = threadIdx.x; k < kWin; k += kPlocThreads) {
    const int g = base + k;
    if (g >= 0 && g < n) {
      s_lo[k] = box[2 * (int64_t)g];
      s_hi[k] = box[2 * (int64_t)g + 1];
      s_sc[k] = scene[g];
    } else {
      s_sc[k] = -1;
    }
  }
  __syncthreads();
  const int i = blockIdx.x * kPlocThreads + threadIdx.x;
  if (i >= n) return;
  const int li = threadIdx.x + kPlocRadius;
  const float4 lo = s_lo[li], hi = s_hi[li];
  const int sc = s_sc[li];
  float best = __int_as_float(0x7f800000);
  int bj = -1;
#pragma unroll 4
  for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {
    if (d == 0 || s_sc[li + d] != sc) continue;
    float a = merged_half_area(lo, hi, s_lo[li + d], s_hi[li + d]);
    if (!(a == a)) a = __int_as_float(0x7f800000);
    if (bj < 0 || a < best) {
      best = a;
      bj = i + d;
    }
  }
  nn[i] = bj;
}

// Mutual nearest neighbours (i < j) merge into node node_off[s] + n_s - 2 - k
// (k-th merge of scene s); cluster i becomes the new node, j is dropped.
// Only thread i touches cluster i's arrays, and the partner j only reads nn.
__global__ void k_ploc_merge(float4 *__restrict__ box, int32_t *__restrict__ ref, int32_t *__restrict__ cnt,
                             const int32_t *__restrict__ scene, const int32_t *__restrict__ nn, int n,
                             const int64_t *__restrict__ tri_off, const int64_t *__restrict__ node_off,
                             int32_t *__restrict__ mctr, Node2 *__restrict__ nodes, int32_t *__restrict__ rcount,
                             int32_t *__restrict__ valid, uint32_t *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = nn[i];
  const bool mutual = j >= 0 && j < n && nn[j] == i;
  if (mutual && j < i) {
    valid[i] = 0;
    return;
  }
  valid[i] = 1;
  if (!mutual) return;
  const int s = scene[i];
  const int64_t ns = tri_off[s + 1] - tri_off[s];
  const int k = atomicAdd(mctr + s, 1);
  if (k > ns - 2) {  // more merges than the scene has internal nodes: corrupted input
    atomicOr(err, kErrQueue);
    return;
  }
  const int64_t id = node_off[s] + (ns - 2 - k);
  const float4 alo = box[2 * (int64_t)i], ahi = box[2 * (int64_t)i + 1];
  const float4 blo = box[2 * (int64_t)j], bhi = box[2 * (int64_t)j + 1];
  Node2 nd;
  nd.a = make_float4(alo.x, ahi.x, alo.y, ahi.y);
  nd.b = make_float4(blo.x, bhi.x, blo.y, bhi.y);
  nd.c = make_float4(alo.z, ahi.z, blo.z, bhi.z);
  nd.d = make_int4(ref[i], ref[j], -1, s);
  nodes[id] = nd;
  const int32_t c = cnt[i] + cnt[j];
  rcount[id] = c;
  box[2 * (int64_t)i] = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.0f);
  box[2 * (int64_t)i + 1] = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.0f);
  ref[i] = (int32_t)id;
  cnt[i] = c;
}

// Exclusive scan of int32 flags: per-tile sums, a one-CTA scan of the tile
// sums (which also yields the total), then each tile's scan plus its offset.
__device__ __forceinline__ int32_t block_exclusive(int32_t v, int32_t *s_w, int32_t &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  int32_t pre = 0, tot = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    if (w < warp) pre += s_w[w];
    tot += s_w[w];
  }
  __syncthreads();
  total = tot;
  return pre + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
    k_scan_tiles(const int32_t *__restrict__ in, int n, int32_t *__restrict__ out, int32_t *__restrict__ tsum) {
  __shared__ int32_t s_w[kScanThreads / 32];
  const int64_t b0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems], sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = b0 + k < n ? in[b0 + k] : 0;
    sum += v[k];
  }
  int32_t total;
  int32_t run = block_exclusive(sum, s_w, total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (b0 + k < n) out[b0 + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int32_t *tsum, int nt, int32_t *total_out) {
  __shared__ int32_t s_w[32];
  const int per = (nt + 1023) / 1024;
  const int a = threadIdx.x * per, e = min(a + per, nt);
  int32_t sum = 0;
  for (int k = a; k < e; ++k) sum += tsum[k];
  int32_t total;
  int32_t run = block_exclusive(sum, s_w, total);
  for (int k = a; k < e; ++k) {
    const int32_t x = tsum[k];
    tsum[k] = run;
    run += x;
  }
  if (threadIdx.x == 0) *total_out = total;
}

__global__ void k_scan_add(int32_t *out, int n, const int32_t *__restrict__ tsum) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tsum[i / kScanTile];
}

__global__ void k_ploc_compact(const float4 *__restrict__ box, const int32_t *__restrict__ ref,
                               const int32_t *__restrict__ cnt, const int32_t *__restrict__ scene,
                               const int32_t *__restrict__ valid, const int32_t *__restrict__ pos, int n,
                               float4 *__restrict__ box_o, int32_t *__restrict__ ref_o, int32_t *__restrict__ cnt_o,
                               int32_t *__restrict__ scene_o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !valid[i]) return;
  const int o = pos[i];
  box_o[2 * (int64_t)o] = box[2 * (int64_t)i];
  box_o[2 * (int64_t)o + 1] = box[2 * (int64_t)i + 1];
  ref_o[o] = ref[i];
  cnt_o[o] = cnt[i];
  scene_o[o] = scene[i];
}

// Roots of the layout: node node_off[s] starts at tri_off[s]; a one-triangle
// scene keeps its triangle in place.
__global__ void k_ploc_layout_init(const int64_t *__restrict__ tri_off, const int64_t *__restrict__ node_off,
                                   int n_scenes, int32_t *__restrict__ rfirst, int32_t *__restrict__ newpos,
                                   int2 *__restrict__ q, int32_t *qcount) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_scenes) return;
  const int64_t ns = tri_off[s + 1] - tri_off[s];
  if (ns == 1) newpos[tri_off[s]] = (int32_t)tri_off[s];
  if (ns < 2) return;
  rfirst[node_off[s]] = (int32_t)tri_off[s];
  q[atomicAdd(qcount, 1)] = make_int2((int)node_off[s], (int)tri_off[s]);
}

// One level: a node starting at `off` puts its left subtree at off and its
// right subtree after the left subtree's leaves.
__global__ void k_ploc_layout(const Node2 *__restrict__ nodes, const int32_t *__restrict__ rcount,
                              const int2 *__restrict__ q_in, int n_in, int2 *__restrict__ q_out, int32_t *q_count,
                              int64_t q_cap, int32_t *__restrict__ rfirst, int32_t *__restrict__ newpos,
                              uint32_t *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_in) return;
  const int2 it = q_in[i];
  const int4 d = nodes[it.x].d;
  const int32_t cl = d.x < 0 ? 1 : rcount[d.x];
  const int32_t ch[2] = {d.x, d.y};
  const int32_t off[2] = {it.y, it.y + cl};
  for (int k = 0; k < 2; ++k) {
    if (ch[k] < 0) {
      newpos[~ch[k]] = off[k];
    } else {
      rfirst[ch[k]] = off[k];
      const int slot = atomicAdd(q_count, 1);
      if (slot < q_cap) q_out[slot] = make_int2(ch[k], off[k]);
      else atomicOr(err, kErrQueue);
    }
  }
}

__global__ void k_ploc_tris(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n,
                            const uint32_t *__restrict__ perm, const int64_t *__restrict__ tri_off, int n_scenes,
                            const int32_t *__restrict__ newpos, TriRec *__restrict__ tris, uint32_t *err) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int s = find_segment(tri_off, n_scenes, p);
    const int64_t toff = tri_off[s], tend = tri_off[s + 1];
    const int64_t q = newpos[p];
    const int64_t orig = perm[p];
    if (q < toff || q >= tend || orig < toff || orig >= tend) {
      atomicOr(err, kErrQueue);
      continue;
    }
    float3 a, b, c;
    tri_verts(pos, idx, orig, a, b, c);
    TriRec r;
    r.p0 = make_float4(a.x, a.y, a.z, __int_as_float((int)(orig - toff)));
    r.p1 = make_float4(b.x, b.y, b.z, 0.0f);
    r.p2 = make_float4(c.x, c.y, c.z, 0.0f);
    tris[q] = r;
  }
}

__global__ void k_ploc_fixrefs(Node2 *nodes, int64_t n_nodes, int64_t n, const int32_t *__restrict__ newpos) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes;
       i += (int64_t)gridDim.x * blockDim.x) {
    int4 d = nodes[i].d;
    if (d.x < 0 && ~d.x < n) d.x = ~newpos[~d.x];
    if (d.y < 0 && ~d.y < n) d.y = ~newpos[~d.y];
    nodes[i].d = d;
  }
}

int ploc_reserve(flg_bvh b) {
  const int64_t n = b->n_tri;
  int rc = FLG_OK;
  auto A = [&](auto **p, size_t c) {
    if (rc == FLG_OK) rc = halloc(b, p, c);
  };
  for (int k = 0; k < 2; ++k) {
    A(&b->d_cbox[k], 2 * (size_t)n);
    A(&b->d_cref[k], n);
    A(&b->d_ccnt[k], n);
    A(&b->d_cscene[k], n);
    A(&b->d_lq[k], b->n_nodes);
  }
  A(&b->d_nn, n);
  A(&b->d_valid, n);
  A(&b->d_pos, n);
  A(&b->d_bsum, ceil_div(n, kScanTile) + 1);
  A(&b->d_mctr, b->n_scenes);
  A(&b->d_newpos, n);
  A(&b->d_lcount, 2);
  A(&b->d_rfirst, b->n_nodes);
  A(&b->d_rcount, b->n_nodes);
  return rc;
}

// Exclusive scan of b->d_valid[0, n) into b->d_pos; the total lands in *d_total.
static int scan_valid(flg_ctx ctx, flg_bvh b, int n, int32_t *d_total) {
  cudaStream_t st = ctx->stream;
  const int nt = (int)ceil_div(n, kScanTile);
  k_scan_tiles<<<nt, kScanThreads, 0, st>>>(b->d_valid, n, b->d_pos, b->d_bsum);
  FLG_LAUNCH_CHECK(ctx, "k_scan_tiles");
  k_scan_sums<<<1, 1024, 0, st>>>(b->d_bsum, nt, d_total);
  FLG_LAUNCH_CHECK(ctx, "k_scan_sums");
  k_scan_add<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(b->d_pos, n, b->d_bsum);
  FLG_LAUNCH_CHECK(ctx, "k_scan_add");
  return FLG_OK;
}

int ploc_build(flg_ctx ctx, flg_bvh b) {
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "a PLOC build synchronises with the host; not capturable");
  cudaStream_t st = ctx->stream;
  const int64_t n = b->n_tri;
  if (n <= 0) return FLG_OK;
  k_ploc_init<<<grid_for(n, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(
      b->pos, b->idx, n, b->d_perm, b->d_tri_off, b->n_scenes, b->d_cbox[0], b->d_cref[0], b->d_ccnt[0],
      b->d_cscene[0]);
  FLG_LAUNCH_CHECK(ctx, "k_ploc_init");
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_mctr, 0, sizeof(int32_t) * b->n_scenes, st));
  int cur = 0;
  int n_c = (int)n;
  int32_t h_total = 0;
  // Every iteration merges in every unfinished scene, so the count strictly
  // falls; the checks below only guard against corrupted input.
  while (n_c > b->n_nonempty) {
    const unsigned g = (unsigned)ceil_div(n_c, kPlocThreads);
    k_ploc_nn<<<g, kPlocThreads, 0, st>>>(b->d_cbox[cur], b->d_cscene[cur], n_c, b->d_nn);
    FLG_LAUNCH_CHECK(ctx, "k_ploc_nn");
    k_ploc_merge<<<g, kPlocThreads, 0, st>>>(b->d_cbox[cur], b->d_cref[cur], b->d_ccnt[cur], b->d_cscene[cur],
                                             b->d_nn, n_c, b->d_tri_off, b->d_node_off, b->d_mctr, b->d_nodes2,
                                             b->d_rcount, b->d_valid, ctx->d_err);
    FLG_LAUNCH_CHECK(ctx, "k_ploc_merge");
    int rc = scan_valid(ctx, b, n_c, b->d_lcount);
    if (rc) return rc;
    k_ploc_compact<<<g, kPlocThreads, 0, st>>>(b->d_cbox[cur], b->d_cref[cur], b->d_ccnt[cur], b->d_cscene[cur],
                                               b->d_valid, b->d_pos, n_c, b->d_cbox[cur ^ 1], b->d_cref[cur ^ 1],
                                               b->d_ccnt[cur ^ 1], b->d_cscene[cur ^ 1]);
    FLG_LAUNCH_CHECK(ctx, "k_ploc_compact");
    FLG_CUDA(ctx, cudaMemcpyAsync(&h_total, b->d_lcount, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_total >= n_c || h_total < b->n_nonempty)
      return set_error(ctx, FLG_ERR_STATE, "clustering made no progress (%d clusters)", n_c);
    n_c = h_total;
    cur ^= 1;
  }
  // Depth-first leaf ranges, level by level.
  FLG_CUDA(ctx, cudaMemsetAsync(b->d_lcount, 0, 2 * sizeof(int32_t), st));
  k_ploc_layout_init<<<grid_for(b->n_scenes, 128), 128, 0, st>>>(b->d_tri_off, b->d_node_off, b->n_scenes,
                                                                  b->d_rfirst, b->d_newpos, b->d_lq[0], b->d_lcount);
  FLG_LAUNCH_CHECK(ctx, "k_ploc_layout_init");
  int qa = 0;
  int32_t n_in = 0;
  FLG_CUDA(ctx, cudaMemcpyAsync(&n_in, b->d_lcount, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  FLG_CUDA(ctx, cudaStreamSynchronize(st));
  for (int64_t level = 0; n_in > 0; ++level) {
    if (level > b->n_nodes) return set_error(ctx, FLG_ERR_STATE, "layout did not finish");
    FLG_CUDA(ctx, cudaMemsetAsync(b->d_lcount + 1, 0, sizeof(int32_t), st));
    k_ploc_layout<<<(unsigned)ceil_div(n_in, 256), 256, 0, st>>>(b->d_nodes2, b->d_rcount, b->d_lq[qa], n_in,
                                                                 b->d_lq[qa ^ 1], b->d_lcount + 1, b->n_nodes,
                                                                 b->d_rfirst, b->d_newpos, ctx->d_err);
    FLG_LAUNCH_CHECK(ctx, "k_ploc_layout");
    FLG_CUDA(ctx, cudaMemcpyAsync(&n_in, b->d_lcount + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(ctx, cudaStreamSynchronize(st));
    if ((int64_t)n_in > b->n_nodes) return set_error(ctx, FLG_ERR_STATE, "layout queue overflow");
    qa ^= 1;
  }
  k_ploc_tris<<<grid_for(n, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(
      b->pos, b->idx, n, b->d_perm, b->d_tri_off, b->n_scenes, b->d_newpos, b->d_tris, ctx->d_err);
  FLG_LAUNCH_CHECK(ctx, "k_ploc_tris");
  if (b->n_nodes > 0) {
    k_ploc_fixrefs<<<grid_for(b->n_nodes, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(b->d_nodes2, b->n_nodes,
                                                                                          n, b->d_newpos);
    FLG_LAUNCH_CHECK(ctx, "k_ploc_fixrefs");
  }
  return FLG_OK;
}

}  // namespace flg
