// sort.cu — onesweep LSD radix sort of (Morton code, triangle index) pairs
// with decoupled look-back (Adinets & Merrill, "Onesweep: A Faster Least
// Significant Digit Radix Sort for GPUs", 2022).  Replaces the reference's
// tbb::parallel_sort of 32-byte RadixTriangle records (radix_bvh.cpp:77-81);
// the sort is stable, so equal codes keep ascending original index.
//
// One launch per 8-bit digit.  Each CTA claims a tile of 3072 pairs (256
// threads x 12) in launch order, ranks its keys with warp ballots and
// shared-memory atomics, publishes its per-digit counts,
// resolves its global offsets by looking back over earlier tiles, reorders
// the tile in shared memory and writes runs of equal digits contiguously.
// Batched builds either sort every scene in its own run of tiles (per-scene
// digit offsets, look-back chains restarting at each scene's first tile: when
// scenes average at least 4 tiles) or append passes whose digit is the scene
// of the pair (from the triangle offsets), which regroup the scenes after the
// Morton passes.
#include "common.cuh"
#include "internal.h"

namespace flg {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 12;  // 12 x 4 CTAs per SM beat 8 / 16 items and 2 / 3 CTAs
constexpr int kSortMinBlocks = 4;  // CTAs per SM the register budget allows
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr int kLookback = 4;  // predecessor tiles read per look-back step
constexpr int kSceneStage = 2048;  // scene passes stage up to this many offsets in shared memory
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;

__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) { *(volatile uint32_t *)p = v; }

// Digit of a pair in this pass: a byte of the key, or (scene passes) a byte
// of the scene that the pair's triangle index falls in.
template <bool kScene>
__device__ __forceinline__ uint32_t sort_digit(uint32_t key, uint32_t val, int shift, const int64_t *tri_off,
                                               int n_scenes) {
  if (!kScene) return (key >> shift) & 0xFFu;
  const uint32_t s = (uint32_t)find_segment(tri_off, n_scenes, (int64_t)val);
  return (s >> shift) & 0xFFu;
}

// One pass over one tile.  Phases: (1) each warp loads 32 x kSortItems
// consecutive pairs (coalesced, no bounds checks on full tiles); (2) ranks
// them: per item, the lanes holding the same digit find each other with
// eight ballots and their lowest lane adds the group's size to the warp's
// counter for that digit with a shared-memory atomic whose old value is the
// group's base.  The atomics of successive items of a warp are issued back
// to back (nothing waits for the previous item's counter), and a warp's
// shared-memory operations are performed in issue order, so ranks follow
// item order and the sort stays stable; (3) column scan of the warp counters
// (warp offsets) and scan over digits (tile start), folded into one offset
// per (warp, digit); (4) publish the tile's counts and look back for the
// global offsets; (5) scatter the pairs into shared memory in digit order
// (one 8-byte store each) and write them out in runs of equal digits.
template <bool kFirst, bool kScene>
__global__ void __launch_bounds__(kSortThreads, kSortMinBlocks)
    k_onesweep(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
               uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n, int shift,
               const int64_t *__restrict__ tri_off, int n_scenes, const uint32_t *__restrict__ pass_off,
               const int32_t *__restrict__ tile_start, int64_t scene_stride, uint32_t *lookback, uint32_t *tile_ctr,
               uint32_t *err, uint32_t spin_limit) {
  __shared__ uint2 s_kv[kSortTile];
  __shared__ uint8_t s_dig[kScene ? kSortTile : 1];
  __shared__ uint32_t s_whist[kSortWarps][kRadix];
  __shared__ int32_t s_glob[kRadix];
  __shared__ uint32_t s_wsum[kSortWarps];
  __shared__ uint32_t s_tile;
  __shared__ int32_t s_off[kScene ? kSceneStage : 1];  // scene passes: the scene offsets
  __shared__ int32_t s_seg;                             // segmented sorts: the tile's scene

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    s_tile = atomicAdd(tile_ctr, 1u);
    if (tile_start) s_seg = find_segment32(tile_start, n_scenes, (int32_t)s_tile);
  }
  for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) (&s_whist[0][0])[i] = 0u;
  const bool staged = kScene && n_scenes <= kSceneStage;
  if (staged)
    for (int i = tid; i < n_scenes; i += kSortThreads) s_off[kScene ? i : 0] = (int32_t)tri_off[i];
  __syncthreads();
  const int64_t tile = s_tile;
  // A segmented sort keeps every scene in its own run of tiles: the tile
  // covers part of [tri_off[s], tri_off[s+1]), the look-back stops at the
  // scene's first tile and the digit offsets are the scene's.
  int64_t first_tile = 0, base = tile * kSortTile, seg_end = n;
  if (tile_start) {
    const int sc = s_seg;
    first_tile = tile_start[sc];
    base = tri_off[sc] + (tile - first_tile) * kSortTile;
    seg_end = tri_off[sc + 1];
    pass_off += (size_t)sc * scene_stride;
  }
  const bool full = base + kSortTile <= seg_end;
  const int64_t wbase = base + (int64_t)warp * (kSortItems * 32) + lane;
  // Pairs of this lane left in the input, as a 32-bit bound for the checks.
  const int64_t wrem64 = seg_end - wbase;
  const int wrem = wrem64 > kSortTile ? kSortTile : (wrem64 < 0 ? 0 : (int)wrem64);
  const uint32_t *kin = keys_in + wbase;
  const uint32_t *vin = kFirst ? nullptr : vals_in + wbase;

  uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
  uint32_t dg[kScene ? kSortItems : 1];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const bool valid = full || j * 32 < wrem;
    k[j] = valid ? kin[j * 32] : 0xFFFFFFFFu;
    v[j] = valid ? (kFirst ? (uint32_t)wbase + (uint32_t)(j * 32) : vin[j * 32]) : 0u;
  }
  if (kScene) {
    // Scene of every pair: with the offsets in shared memory, a binary search
    // of fixed depth whose steps are interleaved over the thread's pairs
    // (largest s with off[s] <= value, as find_segment).
    if (staged) {
      int sc[kScene ? kSortItems : 1];
#pragma unroll
      for (int j = 0; j < kSortItems; ++j) sc[kScene ? j : 0] = 0;
      for (int step = n_scenes > 1 ? 1 << (31 - __clz(n_scenes - 1)) : 0; step >= 1; step >>= 1) {
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
          const int c = sc[kScene ? j : 0] + step;
          if (c < n_scenes && s_off[kScene ? c : 0] <= (int32_t)v[j]) sc[kScene ? j : 0] = c;
        }
      }
#pragma unroll
      for (int j = 0; j < kSortItems; ++j) dg[kScene ? j : 0] = ((uint32_t)sc[kScene ? j : 0] >> shift) & 0xFFu;
    } else {
#pragma unroll
      for (int j = 0; j < kSortItems; ++j) dg[kScene ? j : 0] = sort_digit<true>(k[j], v[j], shift, tri_off, n_scenes);
    }
  }
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const bool valid = full || j * 32 < wrem;
    const uint32_t d = !valid ? 256u : kScene ? dg[kScene ? j : 0] : ((k[j] >> shift) & 0xFFu);
    // Lanes holding the same digit: one ballot per digit bit (and one for
    // validity on a partial tile), about twice as fast as match-any here.
    uint32_t peers = 0xFFFFFFFFu;
    if (!full) {
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, valid);
      peers = valid ? m : ~m;
    }
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
      peers &= ((d >> b) & 1u) ? m : ~m;
    }
    const int leader = __ffs(peers) - 1;
    uint32_t gbase = 0u;
    if (lane == leader && d < 256u) gbase = atomicAdd(&s_whist[warp][d], (uint32_t)__popc(peers));
    gbase = __shfl_sync(0xFFFFFFFFu, gbase, leader);
    rank[j] = gbase + __popc(peers & lt);
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
  st_volatile(lb + d, tile_count | (tile == first_tile ? kFlagPrefix : kFlagAgg));

  // Exclusive scan of the tile counts over digits: the digit's start in the
  // tile's shared-memory reorder, added to every warp's offset.
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
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) s_whist[w][d] += tstart;

  // Decoupled look-back over earlier tiles, kLookback predecessors per step:
  // their flags are read with independent loads, so a walk over m tiles that
  // have only published aggregates costs m / kLookback L2 round trips instead
  // of m.  A word read early stays usable (an aggregate never changes; only
  // its flag may since have become a prefix); an unpublished one is waited
  // on.  The first tile (of the scene) always holds a prefix, so the walk
  // ends there at the latest.
  // Each wait is bounded: on a timeout the error word is set and a (wrong)
  // prefix is still published so later tiles do not wait on this one;
  // writes stay bounds-checked.
  uint32_t excl = 0;
  if (tile > first_tile) {
    int64_t p = tile - 1;
    bool done = false;
    while (!done) {
      uint32_t s[kLookback];
#pragma unroll
      for (int i = 0; i < kLookback; ++i)
        s[i] = p - i >= first_tile ? ld_volatile(lookback + (size_t)(p - i) * kRadix + d) : 0u;
#pragma unroll
      for (int i = 0; i < kLookback; ++i) {
        if (!done && p - i >= first_tile) {
          uint32_t w = s[i];
          if (!(w & kFlagMask)) w = wait_flag(lookback + (size_t)(p - i) * kRadix + d, kFlagMask, spin_limit, err);
          excl += w & kValMask;
          if (w == 0u || (w & kFlagPrefix)) done = true;
        }
      }
      p -= kLookback;
      if (p < first_tile) done = true;
    }
    st_volatile(lb + d, ((excl + tile_count) & kValMask) | kFlagPrefix);
  }
  s_glob[d] = (int32_t)(pass_off[d] + excl) - (int32_t)tstart;
  __syncthreads();

#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t dj = kScene ? dg[kScene ? j : 0] : ((k[j] >> shift) & 0xFFu);
    if (full || j * 32 < wrem) {
      const uint32_t pos = s_whist[warp][dj] + rank[j];
      s_kv[pos] = make_uint2(k[j], v[j]);
      if (kScene) s_dig[kScene ? pos : 0] = (uint8_t)dj;
    }
  }
  __syncthreads();
  const int64_t rem = seg_end - base;
  const int tile_valid = rem < kSortTile ? (int)rem : kSortTile;
  for (int i = tid; i < tile_valid; i += kSortThreads) {
    const uint2 kv = s_kv[i];
    const uint32_t di = kScene ? (uint32_t)s_dig[kScene ? i : 0] : ((kv.x >> shift) & 0xFFu);
    const int64_t out = (int64_t)s_glob[di] + i;
    if (out >= 0 && out < n) {
      keys_out[out] = kv.x;
      vals_out[out] = kv.y;
    }
  }
}

// Launches one pass (the template pair for first / scene passes).
static void launch_pass(cudaStream_t st, unsigned grid, bool first, bool scene, const uint32_t *in_k,
                        const uint32_t *in_v, uint32_t *out_k, uint32_t *out_v, int64_t n, int shift,
                        const int64_t *tri_off, int n_scenes, const uint32_t *pass_off, const int32_t *tile_start,
                        int64_t scene_stride, uint32_t *lb, uint32_t *tile_ctr, uint32_t *err, uint32_t spin_limit) {
  if (first && scene)
    k_onesweep<true, true><<<grid, kSortThreads, 0, st>>>(in_k, in_v, out_k, out_v, n, shift, tri_off, n_scenes,
                                                          pass_off, tile_start, scene_stride, lb, tile_ctr, err,
                                                          spin_limit);
  else if (first)
    k_onesweep<true, false><<<grid, kSortThreads, 0, st>>>(in_k, in_v, out_k, out_v, n, shift, tri_off, n_scenes,
                                                           pass_off, tile_start, scene_stride, lb, tile_ctr, err,
                                                           spin_limit);
  else if (scene)
    k_onesweep<false, true><<<grid, kSortThreads, 0, st>>>(in_k, in_v, out_k, out_v, n, shift, tri_off, n_scenes,
                                                           pass_off, tile_start, scene_stride, lb, tile_ctr, err,
                                                           spin_limit);
  else
    k_onesweep<false, false><<<grid, kSortThreads, 0, st>>>(in_k, in_v, out_k, out_v, n, shift, tri_off, n_scenes,
                                                            pass_off, tile_start, scene_stride, lb, tile_ctr, err,
                                                            spin_limit);
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
int64_t sort_tile() { return kSortTile; }

// Enqueues the passes.  Expects: b->d_kbuf[0] holds the unsorted codes and
// b->d_hist[0 .. n_morton_passes) the code histograms; the scene-pass
// histograms are already in place.  Leaves the sorted pairs in
// (b->d_keys, b->d_perm).
int sort_enqueue(flg_ctx ctx, flg_bvh b) {
  const int64_t n = b->n_tri;
  if (n <= 0) return FLG_OK;
  uint32_t *hist = b->d_hist;
  uint32_t *off = b->d_hist + (size_t)b->n_passes * kRadix;
  int64_t scene_stride = 0;
  if (b->d_tile_start) {
    // Segmented: the bucket starts are per scene ([scene][pass][digit], from
    // k_scan_seg).
    off = b->d_shist + 4 * kRadix * (size_t)b->n_scenes;
    scene_stride = 4 * kRadix;
  } else {
    k_scan_hist<<<b->n_passes, kRadix, 0, ctx->stream>>>(hist, off);
    FLG_LAUNCH_CHECK(ctx, "k_scan_hist");
  }
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
    launch_pass(ctx->stream, grid, p == 0, scene_pass, in_k, in_v, out_k, out_v, n, shift, b->d_tri_off, b->n_scenes,
                off + (size_t)p * kRadix, b->d_tile_start, scene_stride, lb, b->d_tile_ctr + p, ctx->d_err,
                ctx->spin_limit);
    FLG_LAUNCH_CHECK(ctx, "k_onesweep");
    stage_mark(ctx, ctx->stream, scene_pass ? "sort_scene_pass" : "sort_pass");
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
    launch_pass(st, (unsigned)tiles, p == 0, false, keys[p & 1], vals[p & 1], keys[(p + 1) & 1], vals[(p + 1) & 1], n,
                8 * p, nullptr, 1, off + (size_t)p * kRadix, nullptr, 0, lb, tile_ctr + p, ctx->d_err,
                ctx->spin_limit);
    FLG_LAUNCH_CHECK(ctx, "k_onesweep");
    stage_mark(ctx, st, "ray_sort_pass");
  }
  return FLG_OK;
}

}  // namespace flg
