// sort.cu — onesweep LSD radix sort of (Morton code, triangle index) pairs
// with decoupled look-back (Adinets & Merrill, "Onesweep: A Faster Least
// Significant Digit Radix Sort for GPUs", 2022).  Replaces the reference's
// tbb::parallel_sort of 32-byte RadixTriangle records (radix_bvh.cpp:77-81);
// the sort is stable, so equal codes keep ascending original index.
//
// One launch per 8-bit digit.  Each CTA claims a tile of 4096 pairs in launch
// order, ranks its keys with warp match-any, publishes its per-digit counts,
// resolves its global offsets by looking back over earlier tiles, reorders
// the tile in shared memory and writes runs of equal digits contiguously.
// Batched builds append passes whose digit is the scene of the pair (from
// the triangle offsets), which regroups the scenes after the Morton passes.
#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;

__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) { *(volatile uint32_t *)p = v; }

__device__ __forceinline__ uint32_t sort_digit(uint32_t key, uint32_t val, int shift, int scene_mode,
                                               const int64_t *tri_off, int n_scenes) {
  if (!scene_mode) return (key >> shift) & 0xFFu;
  uint32_t s = (uint32_t)find_segment(tri_off, n_scenes, (int64_t)val);
  return (s >> shift) & 0xFFu;
}

template <bool kFirst>
__global__ void __launch_bounds__(kSortThreads)
    k_onesweep(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
               uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n, int shift,
               int scene_mode, const int64_t *__restrict__ tri_off, int n_scenes,
               const uint32_t *__restrict__ pass_off, uint32_t *lookback, uint32_t *tile_ctr,
               uint32_t *err, uint32_t spin_limit) {
  __shared__ uint32_t s_keys[kSortTile];
  __shared__ uint32_t s_vals[kSortTile];
  __shared__ uint8_t s_dig[kSortTile];
  __shared__ uint32_t s_whist[kSortWarps][kRadix];
  __shared__ uint32_t s_tile_start[kRadix];
  __shared__ int32_t s_glob[kRadix];
  __shared__ uint32_t s_wsum[kSortWarps];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
  for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) (&s_whist[0][0])[i] = 0u;
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * kSortTile;
  const int64_t wbase = base + (int64_t)warp * (kSortItems * 32);

  uint32_t k[kSortItems], v[kSortItems], dg[kSortItems], rank[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    int64_t idx = wbase + j * 32 + lane;
    bool valid = idx < n;
    k[j] = valid ? keys_in[idx] : 0xFFFFFFFFu;
    v[j] = valid ? (kFirst ? (uint32_t)idx : vals_in[idx]) : 0u;
  }
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    int64_t idx = wbase + j * 32 + lane;
    bool valid = idx < n;
    uint32_t d = valid ? sort_digit(k[j], v[j], shift, scene_mode, tri_off, n_scenes) : 256u;
    dg[j] = d;
    uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    uint32_t cnt = valid ? s_whist[warp][d] : 0u;
    __syncwarp();
    rank[j] = cnt + __popc(peers & lt);
    if (valid && (peers & lt) == 0u) s_whist[warp][d] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Column scan over warps: per-warp exclusive offsets, tile count per digit.
  const int d = tid;
  uint32_t tile_count = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    uint32_t c = s_whist[w][d];
    s_whist[w][d] = tile_count;
    tile_count += c;
  }
  uint32_t *lb = lookback + (size_t)tile * kRadix;
  st_volatile(lb + d, tile_count | (tile == 0 ? kFlagPrefix : kFlagAgg));

  // Exclusive scan of the tile counts over digits (shared-memory reorder).
  uint32_t x = tile_count;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_wsum[warp] = x;
  __syncthreads();
  uint32_t wpre = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w)
    if (w < warp) wpre += s_wsum[w];
  const uint32_t tstart = wpre + x - tile_count;
  s_tile_start[d] = tstart;

  // Decoupled look-back over earlier tiles.  Each wait is bounded: on a
  // timeout the error word is set and a (wrong) prefix is still published so
  // later tiles do not wait on this one; writes stay bounds-checked.
  uint32_t excl = 0;
  if (tile > 0) {
    int64_t p = tile - 1;
    while (p >= 0) {
      uint32_t s = wait_flag(lookback + (size_t)p * kRadix + d, kFlagMask, spin_limit, err);
      excl += s & kValMask;
      if (s == 0u || (s & kFlagPrefix)) break;
      --p;
    }
    st_volatile(lb + d, ((excl + tile_count) & kValMask) | kFlagPrefix);
  }
  s_glob[d] = (int32_t)(pass_off[d] + excl) - (int32_t)tstart;
  __syncthreads();

#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    if (dg[j] < 256u) {
      uint32_t pos = s_tile_start[dg[j]] + s_whist[warp][dg[j]] + rank[j];
      s_keys[pos] = k[j];
      s_vals[pos] = v[j];
      s_dig[pos] = (uint8_t)dg[j];
    }
  }
  __syncthreads();
  int64_t rem = n - base;
  const int tile_valid = rem < kSortTile ? (int)rem : kSortTile;
  for (int i = tid; i < tile_valid; i += kSortThreads) {
    int64_t out = (int64_t)s_glob[s_dig[i]] + i;
    if (out >= 0 && out < n) {
      keys_out[out] = s_keys[i];
      vals_out[out] = s_vals[i];
    }
  }
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void k_scan_hist(const uint32_t *__restrict__ hist, uint32_t *__restrict__ off) {
  __shared__ uint32_t s_w[8];
  const int p = blockIdx.x, d = threadIdx.x, lane = d & 31, warp = d >> 5;
  uint32_t c = hist[p * kRadix + d];
  uint32_t x = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < warp; ++w) pre += s_w[w];
  off[p * kRadix + d] = pre + x - c;
}

int64_t sort_tiles(int64_t n) { return ceil_div(n, kSortTile); }

// Enqueues the passes.  Expects: b->d_kbuf[0] holds the unsorted codes and
// b->d_hist[0 .. n_morton_passes) the code histograms; the scene-pass
// histograms are already in place.  Leaves the sorted pairs in
// (b->d_keys, b->d_perm).
int sort_enqueue(flg_ctx ctx, flg_bvh b) {
  const int64_t n = b->n_tri;
  if (n <= 0) return FLG_OK;
  uint32_t *hist = b->d_hist;
  uint32_t *off = b->d_hist + (size_t)b->n_passes * kRadix;
  k_scan_hist<<<b->n_passes, kRadix, 0, ctx->stream>>>(hist, off);
  FLG_LAUNCH_CHECK(ctx, "k_scan_hist");
  const unsigned grid = (unsigned)b->n_tiles;
  // Ping-pong: pass p reads buffer (p & 1) and writes buffer ((p + 1) & 1).
  uint32_t *kb[2] = {b->n_passes % 2 == 0 ? b->d_keys : b->d_keys_alt,
                     b->n_passes % 2 == 0 ? b->d_keys_alt : b->d_keys};
  uint32_t *vb[2] = {b->n_passes % 2 == 0 ? b->d_perm : b->d_vals_alt,
                     b->n_passes % 2 == 0 ? b->d_vals_alt : b->d_perm};
  for (int p = 0; p < b->n_passes; ++p) {
    const bool scene_pass = p >= b->n_morton_passes;
    const int shift = scene_pass ? 8 * (p - b->n_morton_passes) : 8 * p;
    uint32_t *lb = b->d_lookback + (size_t)p * b->n_tiles * kRadix;
    uint32_t *in_k = kb[p & 1], *out_k = kb[(p + 1) & 1];
    uint32_t *in_v = vb[p & 1], *out_v = vb[(p + 1) & 1];
    if (p == 0) {
      k_onesweep<true><<<grid, kSortThreads, 0, ctx->stream>>>(
          in_k, nullptr, out_k, out_v, n, shift, scene_pass ? 1 : 0, b->d_tri_off, b->n_scenes,
          off + (size_t)p * kRadix, lb, b->d_tile_ctr + p, ctx->d_err, ctx->spin_limit);
    } else {
      k_onesweep<false><<<grid, kSortThreads, 0, ctx->stream>>>(
          in_k, in_v, out_k, out_v, n, shift, scene_pass ? 1 : 0, b->d_tri_off, b->n_scenes,
          off + (size_t)p * kRadix, lb, b->d_tile_ctr + p, ctx->d_err, ctx->spin_limit);
    }
    FLG_LAUNCH_CHECK(ctx, "k_onesweep");
  }
  return FLG_OK;
}

// Generic (key, index) sort used by the ray sort: keys[0] holds n keys and
// hist[0 .. passes) their per-pass digit counts; the sorted keys and the
// original indices end in keys[passes & 1] / vals[passes & 1].  hist needs
// 2 * passes * 256 words, lookback passes * tiles * 256, tile_ctr passes.
int sort_pairs_enqueue(flg_ctx ctx, cudaStream_t st, int64_t n, int passes, uint32_t *const keys[2],
                       uint32_t *const vals[2], uint32_t *hist, uint32_t *lookback, uint32_t *tile_ctr) {
  if (n <= 0) return FLG_OK;
  const int64_t tiles = sort_tiles(n);
  uint32_t *off = hist + (size_t)passes * kRadix;
  FLG_CUDA(ctx, cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * kRadix * (size_t)tiles * passes, st));
  FLG_CUDA(ctx, cudaMemsetAsync(tile_ctr, 0, sizeof(uint32_t) * passes, st));
  k_scan_hist<<<passes, kRadix, 0, st>>>(hist, off);
  FLG_LAUNCH_CHECK(ctx, "k_scan_hist");
  for (int p = 0; p < passes; ++p) {
    uint32_t *lb = lookback + (size_t)p * tiles * kRadix;
    if (p == 0)
      k_onesweep<true><<<(unsigned)tiles, kSortThreads, 0, st>>>(keys[0], nullptr, keys[1], vals[1], n, 0, 0, nullptr,
                                                                  1, off, lb, tile_ctr, ctx->d_err, ctx->spin_limit);
    else
      k_onesweep<false><<<(unsigned)tiles, kSortThreads, 0, st>>>(keys[p & 1], vals[p & 1], keys[(p + 1) & 1],
                                                                   vals[(p + 1) & 1], n, 8 * p, 0, nullptr, 1,
                                                                   off + (size_t)p * kRadix, lb, tile_ctr + p,
                                                                   ctx->d_err, ctx->spin_limit);
    FLG_LAUNCH_CHECK(ctx, "k_onesweep");
  }
  return FLG_OK;
}

}  // namespace flg
