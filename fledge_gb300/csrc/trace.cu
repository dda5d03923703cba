// trace.cu — closest-hit and any-hit ray traversal (RadixBVHBuilder::
// intersect / recursiveIntersect, radix_bvh.cpp:26-30,202-245, with the
// watertight Pluecker test of intersector.hpp:63-101).
//
// Layouts: BVH2 nodes carry both children's boxes (one 64-byte record per
// visit); wide nodes (4 or 8 children) store their child boxes as structure
// of arrays inside a 112/224-byte record read with 16-byte loads; triangles
// are gathered in sorted (leaf) order, 48 bytes each.
//
// Kernels:
//   k_trace_bvh2        one ray per thread over BVH2, leaf triangles tested
//                       directly as the reference does (no leaf box test)
//   k_trace_wide        one ray per thread over 4/8-wide nodes, children
//                       visited nearest first (sorting network on t|ref keys)
//   k_trace_persistent  persistent warps that refill idle lanes from a global
//                       ray counter (work stealing across scenes of a batch)
//   k_trace_retry       rays whose short stack overflowed, with a deep stack
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace flg {

struct RaySoA {
  const float *ox, *oy, *oz, *dx, *dy, *dz, *tmin, *tmax;
  float tmin_c, tmax_c;
};

struct Out {
  int32_t *prim;
  float *t, *u, *v;
  uint8_t *occ;
};

struct Scratch {
  int64_t *ovf;
  uint32_t *ovf_count;
  int64_t ovf_cap;
  unsigned long long *work;
  uint32_t *err;
};

constexpr int kRetryStack = 256;

__device__ __forceinline__ void load_ray(const RaySoA &R, int64_t i, float3 &o, float3 &d, float3 &inv,
                                         float &tmin, float &tmax) {
  o = make_float3(__ldg(R.ox + i), __ldg(R.oy + i), __ldg(R.oz + i));
  d = make_float3(__ldg(R.dx + i), __ldg(R.dy + i), __ldg(R.dz + i));
  inv = make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
  tmin = R.tmin ? __ldg(R.tmin + i) : R.tmin_c;
  tmax = R.tmax ? __ldg(R.tmax + i) : R.tmax_c;
}

__device__ __forceinline__ int32_t scene_root(const int32_t *__restrict__ roots, const int64_t *__restrict__ ray_off,
                                              int n_scenes, int64_t i) {
  int s = ray_off ? find_segment(ray_off, n_scenes, i) : 0;
  return __ldg(roots + s);
}

// The same for a lane whose rays only grow (persistent kernels take them
// from one counter): `sc` holds the scene of the lane's previous ray (-1:
// none yet); one search, then a forward walk.
__device__ __forceinline__ int32_t scene_root_walk(const int32_t *__restrict__ roots,
                                                   const int64_t *__restrict__ ray_off, int n_scenes, int64_t i,
                                                   int &sc) {
  if (!ray_off) return __ldg(roots);
  if (sc < 0) {
    sc = find_segment(ray_off, n_scenes, i);
  } else {
    while (sc < n_scenes - 1 && __ldg(ray_off + sc + 1) <= i) ++sc;
  }
  return __ldg(roots + sc);
}

// Tests sorted triangle g; updates the closest hit.  Returns true on accept.
// MT selects the live renderer's Moller-Trumbore test and its strict
// t < tMax rule instead of the watertight Pluecker test.
template <bool MT = false>
__device__ __forceinline__ bool test_tri(const TriRec *__restrict__ tris, int64_t g, const float3 &o,
                                         const float3 &d, float tmin, float &best, bool &have, int32_t &prim) {
  const float4 *p = (const float4 *)(tris + g);
  float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  float t;
  const float3 pa = make_float3(a.x, a.y, a.z), pb = make_float3(b.x, b.y, b.z), pc = make_float3(c.x, c.y, c.z);
  if (MT) {
    if (!moller_t(pa, pb, pc, o, d, t)) return false;
    if (!(t >= tmin && t < best)) return false;
  } else {
    if (!pluecker_t(pa, pb, pc, o, d, t)) return false;
    if (!accept_closest(t, tmin, best, have)) return false;
  }
  best = t;
  have = true;
  prim = (int32_t)g;  // sorted position; write_result maps it to the original id
  return true;
}

// Any-hit variant: accepts t in [tmin, tmax] ([tmin, tmax) with MT).
template <bool MT = false>
__device__ __forceinline__ bool test_tri_any(const TriRec *__restrict__ tris, int64_t g, const float3 &o,
                                             const float3 &d, float tmin, float tmax) {
  const float4 *p = (const float4 *)(tris + g);
  float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  float t;
  const float3 pa = make_float3(a.x, a.y, a.z), pb = make_float3(b.x, b.y, b.z), pc = make_float3(c.x, c.y, c.z);
  if (MT) return moller_t(pa, pb, pc, o, d, t) && t >= tmin && t < tmax;
  if (!pluecker_t(pa, pb, pc, o, d, t)) return false;
  return t >= tmin && !(t > tmax);
}

__device__ __forceinline__ uint64_t stack_key(float t, int32_t ref) {
  return ((uint64_t)(__float_as_uint(t) & 0x7FFFFFFFu) << 32) | (uint32_t)ref;
}

// Writes one ray's result.  For closest hit, `prim` holds the sorted
// position of the winning triangle: its record gives the original id and the
// vertices for the float-float refinement of t, u, v.  The traversal keeps
// only t; the fp32 barycentrics (pluecker) are formed here, for the winner,
// and replaced by the refined ones unless the refinement finds den == 0.
// Result of a finished ray.  Closest hits store the sorted position of the
// triangle and the fp32 t; k_trace_finish turns them into the original id
// and the refined t, u, v afterwards.  Refining here cost several hundred
// instructions per ray, run whenever a ray retired, i.e. with few lanes of
// the warp active: about a fifth of the traversal kernel's issue slots.
__device__ __forceinline__ void write_result(const Out &O, int64_t i, bool any, bool have, int32_t prim,
                                             float best, float tmax) {
  if (any) {
    O.occ[i] = have ? 1 : 0;
  } else {
    O.prim[i] = have ? prim : -1;
    O.t[i] = have ? best : tmax;
    if (!have) {
      O.u[i] = 0.0f;
      O.v[i] = 0.0f;
    }
  }
}

// Hit values of every closest hit, one ray per thread after the traversal
// (same ray floats, same triangle record, same arithmetic as in the loop):
// barycentrics from the Pluecker quantities, then t, u, v recomputed in
// float-float and rounded once (refine_tuv); the sorted position becomes
// the caller's triangle id.
__global__ void __launch_bounds__(256, 4)
    k_trace_finish(RaySoA R, int64_t n, Out O, const TriRec *__restrict__ tris) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = O.prim[i];
    if (g < 0) continue;
    const float3 o = make_float3(__ldg(R.ox + i), __ldg(R.oy + i), __ldg(R.oz + i));
    const float3 d = make_float3(__ldg(R.dx + i), __ldg(R.dy + i), __ldg(R.dz + i));
    const float4 *p = (const float4 *)(tris + g);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    const float3 pa = make_float3(a.x, a.y, a.z), pb = make_float3(b.x, b.y, b.z), pc = make_float3(c.x, c.y, c.z);
    float best = O.t[i], u = 0.0f, v = 0.0f;
    if (!refine_tuv(pa, pb, pc, o, d, best, u, v)) {
      // N.D == 0: the fp32 barycentrics of the test stand (t stays the test's)
      float tf;
      pluecker(pa, pb, pc, o, d, tf, u, v);
    }
    O.prim[i] = __float_as_int(a.w);
    O.t[i] = best;
    O.u[i] = u;
    O.v[i] = v;
  }
}

__device__ __forceinline__ void record_overflow(const Scratch &S, int64_t ray) {
  uint32_t k = atomicAdd(S.ovf_count, 1u);
  if (k < S.ovf_cap) S.ovf[k] = ray;
  else atomicOr(S.err, kErrStack);
}

// ----------------------------------------------------------------------------
// BVH2 traversal (reference-faithful leaf handling).
// ----------------------------------------------------------------------------
template <bool ANY, int STACK, bool MT = false>
__device__ __forceinline__ bool trace_bvh2(const Node2 *__restrict__ nodes, const TriRec *__restrict__ tris,
                                           int32_t root, const float3 &o, const float3 &d, const float3 &inv,
                                           float tmin, float tmax, bool &have, int32_t &prim, float &best) {
  best = tmax;
  have = false;
  prim = -1;
  if (root == INT32_MIN) return true;
  if (root < 0) {
    if (ANY) have = test_tri_any<MT>(tris, ~(int64_t)root, o, d, tmin, tmax);
    else test_tri<MT>(tris, ~(int64_t)root, o, d, tmin, best, have, prim);
    return true;
  }
  uint64_t stk[STACK];
  int sp = 0;
  int32_t cur = root;
  const float miss = __int_as_float(0x7fffffff);  // NaN: never <= a limit
  while (true) {
    const float4 *np = (const float4 *)(nodes + cur);
    const float4 A = __ldg(np), B = __ldg(np + 1), C = __ldg(np + 2);
    const int4 Dd = __ldg((const int4 *)(np + 3));
    const int32_t c0 = Dd.x, c1 = Dd.y;
    if (c0 < 0) {
      if (ANY) {
        if (test_tri_any<MT>(tris, ~(int64_t)c0, o, d, tmin, tmax)) { have = true; return true; }
      } else {
        test_tri<MT>(tris, ~(int64_t)c0, o, d, tmin, best, have, prim);
      }
    }
    if (c1 < 0) {
      if (ANY) {
        if (test_tri_any<MT>(tris, ~(int64_t)c1, o, d, tmin, tmax)) { have = true; return true; }
      } else {
        test_tri<MT>(tris, ~(int64_t)c1, o, d, tmin, best, have, prim);
      }
    }
    const float lim = ANY ? tmax : best;
    float t0 = c0 >= 0 ? slab_tnear(A.x, A.y, A.z, A.w, C.x, C.y, o, inv) : miss;
    float t1 = c1 >= 0 ? slab_tnear(B.x, B.y, B.z, B.w, C.z, C.w, o, inv) : miss;
    const bool h0 = c0 >= 0 && t0 <= lim, h1 = c1 >= 0 && t1 <= lim;
    if (h0 && h1) {
      if (sp >= STACK) return false;
      const bool swap = t1 < t0;
      stk[sp++] = swap ? stack_key(t0, c0) : stack_key(t1, c1);
      cur = swap ? c1 : c0;
      continue;
    }
    if (h0) { cur = c0; continue; }
    if (h1) { cur = c1; continue; }
    bool found = false;
    while (sp > 0) {
      uint64_t e = stk[--sp];
      if (__uint_as_float((uint32_t)(e >> 32)) > (ANY ? tmax : best)) continue;
      cur = (int32_t)(uint32_t)e;
      found = true;
      break;
    }
    if (!found) return true;
  }
}

template <bool ANY, bool MT = false>
__global__ void __launch_bounds__(256)
    k_trace_bvh2(const Node2 *__restrict__ nodes, const TriRec *__restrict__ tris, const int32_t *__restrict__ roots,
                 const int64_t *__restrict__ ray_off, int n_scenes, RaySoA R, int64_t n, Out O, Scratch S) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 o, d, inv;
  float tmin, tmax;
  load_ray(R, i, o, d, inv, tmin, tmax);
  const int32_t root = scene_root(roots, ray_off, n_scenes, i);
  bool have;
  int32_t prim;
  float best;
  if (!trace_bvh2<ANY, 64, MT>(nodes, tris, root, o, d, inv, tmin, tmax, have, prim, best)) {
    record_overflow(S, i);
    return;
  }
  write_result(O, i, ANY, have, prim, best, tmax);
}

// ----------------------------------------------------------------------------
// Wide traversal as a resumable state machine (one node or leaf range per
// step) so the persistent kernel can swap rays between steps.
// ----------------------------------------------------------------------------
// Child keys for the nearest-first order: the bits of tnear (non-negative,
// so integer order is float order) with the child's slot in the low
// log2(W) bits.  Dropping those mantissa bits only rounds tnear down, which
// keeps the stack's culling test (entry tnear > best) conservative.
__device__ __forceinline__ void cas(uint32_t &a, uint32_t &b) {
  const uint32_t lo = min(a, b), hi = max(a, b);
  a = lo;
  b = hi;
}

template <int W>
__device__ __forceinline__ void sort_keys(uint32_t (&k)[W]) {
  if constexpr (W == 4) {
    cas(k[0], k[1]); cas(k[2], k[3]); cas(k[0], k[2]); cas(k[1], k[3]); cas(k[1], k[2]);
  } else {
    cas(k[0], k[1]); cas(k[2], k[3]); cas(k[4], k[5]); cas(k[6], k[7]);
    cas(k[0], k[2]); cas(k[1], k[3]); cas(k[4], k[6]); cas(k[5], k[7]);
    cas(k[1], k[2]); cas(k[5], k[6]);
    cas(k[0], k[4]); cas(k[1], k[5]); cas(k[2], k[6]); cas(k[3], k[7]);
    cas(k[2], k[4]); cas(k[3], k[5]);
    cas(k[1], k[2]); cas(k[3], k[4]); cas(k[5], k[6]);
  }
}

// The child ref a sorted key names (selects, no dynamic register index).
template <int W>
__device__ __forceinline__ int32_t key_ref(uint32_t key, const int32_t (&ref)[W]) {
  if constexpr (W == 4) {
    const int32_t a = (key & 1u) ? ref[1] : ref[0];
    const int32_t b = (key & 1u) ? ref[3] : ref[2];
    return (key & 2u) ? b : a;
  } else {
    const uint32_t slot = key & (uint32_t)(W - 1);
    int32_t r = ref[0];
#pragma unroll
    for (int m = 1; m < W; ++m) r = slot == (uint32_t)m ? ref[m] : r;
    return r;
  }
}

// Stack entry (tnear rounded down | ref) of a sorted key.
template <int W>
__device__ __forceinline__ uint64_t key_entry(uint32_t key, const int32_t (&ref)[W]) {
  return ((uint64_t)(key & ~(uint32_t)(W - 1)) << 32) | (uint32_t)key_ref<W>(key, ref);
}

// Tests the W children of a wide node (7 / 14 16-byte loads) with the
// reference's slab test (BoundIntersect, intersector.hpp:103-120).  The
// near and far plane arrays of each axis are picked by the sign of the
// ray's inverse direction when they are loaded, so the per-child swap of
// slab1 disappears; the products are the same roundings, so tnear and the
// hit decision equal slab_tnear's (a NaN slab, 0 * inf, constrains nothing
// in both).  Returns the number of children hit with tnear <= lim; their
// keys are in key[] (misses are ~0), the child refs in ref[] — loaded only
// when a child is hit (the kernel is bound by L1 throughput; skipping that
// 16-byte load on visits without hits gave +2.5 %).  Empty slots need no
// test of their ref: they hold +inf boxes, which no ray enters.
template <int W>
__device__ __forceinline__ int visit_node(const NodeW<W> *__restrict__ node, const float3 &o, const float3 &inv,
                                          float lim, uint32_t (&key)[W], int32_t (&ref)[W]) {
  constexpr int Q = W / 4;  // float4s per child array
  const float4 *np = (const float4 *)node;
  // Float4 offsets of the near arrays: lo (sign 0) or hi (sign 1) per axis.
  const int nx = (int)(__float_as_uint(inv.x) >> 31) * Q;
  const int ny = 2 * Q + (int)(__float_as_uint(inv.y) >> 31) * Q;
  const int nz = 4 * Q + (int)(__float_as_uint(inv.z) >> 31) * Q;
  float pn[3][W], pf[3][W];
#pragma unroll
  for (int h = 0; h < Q; ++h) {
    const float4 a = __ldg(np + nx + h), b = __ldg(np + (nx ^ Q) + h);
    const float4 c = __ldg(np + ny + h), e = __ldg(np + (ny ^ Q) + h);
    const float4 f = __ldg(np + nz + h), g = __ldg(np + (nz ^ Q) + h);
    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
    const float cv[4] = {c.x, c.y, c.z, c.w}, ev[4] = {e.x, e.y, e.z, e.w};
    const float fv[4] = {f.x, f.y, f.z, f.w}, gv[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      pn[0][4 * h + k] = av[k]; pf[0][4 * h + k] = bv[k];
      pn[1][4 * h + k] = cv[k]; pf[1][4 * h + k] = ev[k];
      pn[2][4 * h + k] = fv[k]; pf[2][4 * h + k] = gv[k];
    }
  }
  const float t1c = fminf(lim, 3.402823466e+38f);
  int nh = 0;
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const float tnx = (pn[0][k] - o.x) * inv.x, tfx = (pf[0][k] - o.x) * inv.x;
    const float tny = (pn[1][k] - o.y) * inv.y, tfy = (pf[1][k] - o.y) * inv.y;
    const float tnz = (pn[2][k] - o.z) * inv.z, tfz = (pf[2][k] - o.z) * inv.z;
    const float t0 = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
    const float t1 = fminf(fminf(tfx, tfy), fminf(tfz, t1c));
    const bool ok = t0 <= t1;  // empty slots hold +inf boxes, which no ray enters
    key[k] = ok ? ((__float_as_uint(t0) & 0x7FFFFFFFu & ~(uint32_t)(W - 1)) | (uint32_t)k) : ~0u;
    nh += ok ? 1 : 0;
  }
  if (nh > 0) {
#pragma unroll
    for (int h = 0; h < Q; ++h) {
      const int4 r = __ldg((const int4 *)np + 6 * Q + h);
      ref[4 * h] = r.x; ref[4 * h + 1] = r.y; ref[4 * h + 2] = r.z; ref[4 * h + 3] = r.w;
    }
  }
  return nh;
}

template <int W, bool ANY, int STACK>
struct Tracer {
  float3 o, d, inv;
  float tmin, tmax, best;
  int32_t cur, prim;
  int sp;
  bool have, overflow;
  uint64_t stk[STACK];

  __device__ __forceinline__ void start(int32_t root) {
    best = tmax;
    have = false;
    overflow = false;
    prim = -1;
    sp = 0;
    cur = root;
  }

  __device__ __forceinline__ bool pop() {
    const float lim = ANY ? tmax : best;
    while (sp > 0) {
      uint64_t e = stk[--sp];
      if (__uint_as_float((uint32_t)(e >> 32)) > lim) continue;
      cur = (int32_t)(uint32_t)e;
      return true;
    }
    return false;
  }

  // Returns true when the ray is finished.
  __device__ __forceinline__ bool step(const NodeW<W> *__restrict__ nodes, const TriRec *__restrict__ tris) {
    if (cur == kEmptyChild || cur == INT32_MIN) return true;
    if (cur >= 0) {
      uint32_t key[W];
      int32_t ref[W];
      const int nh = visit_node<W>(nodes + cur, o, inv, ANY ? tmax : best, key, ref);
      if (nh == 0) return !pop();
      sort_keys<W>(key);
      if (sp + nh - 1 > STACK) {
        overflow = true;
        return true;
      }
#pragma unroll
      for (int k = W - 1; k >= 1; --k)
        if (k < nh) stk[sp++] = key_entry<W>(key[k], ref);
      cur = key_ref<W>(key[0], ref);
      return false;
    }
    const int32_t enc = ~cur;
    const int64_t first = (int64_t)((uint32_t)enc >> 3);
    const int count = (enc & 7) + 1;
    for (int j = 0; j < count; ++j) {
      if (ANY) {
        if (test_tri_any(tris, first + j, o, d, tmin, tmax)) {
          have = true;
          return true;
        }
      } else {
        test_tri(tris, first + j, o, d, tmin, best, have, prim);
      }
    }
    return !pop();
  }
};

template <int W, bool ANY, int STACK>
__global__ void __launch_bounds__(256)
    k_trace_wide(const NodeW<W> *__restrict__ nodes, const TriRec *__restrict__ tris, const int32_t *__restrict__ roots,
                 const int64_t *__restrict__ ray_off, int n_scenes, RaySoA R, int64_t n, Out O, Scratch S) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Tracer<W, ANY, STACK> tr;
  load_ray(R, i, tr.o, tr.d, tr.inv, tr.tmin, tr.tmax);
  tr.start(scene_root(roots, ray_off, n_scenes, i));
  while (!tr.step(nodes, tris)) {
  }
  if (tr.overflow) record_overflow(S, i);
  else write_result(O, i, ANY, tr.have, tr.prim, tr.best, tr.tmax);
}

template <int W, bool ANY, int STACK>
__global__ void __launch_bounds__(256)
    k_trace_persistent(const NodeW<W> *__restrict__ nodes, const TriRec *__restrict__ tris,
                       const int32_t *__restrict__ roots, const int64_t *__restrict__ ray_off, int n_scenes, RaySoA R,
                       int64_t n, Out O, Scratch S, int refill) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt = (1u << lane) - 1u;
  Tracer<W, ANY, STACK> tr;
  bool active = false, exhausted = false;
  int64_t ray = -1;
  int scene = -1;
  while (true) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !active);
    const int nidle = __popc(idle);
    if (!exhausted && nidle >= refill) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(S.work, (unsigned long long)nidle);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (!active) {
        const int64_t my = (int64_t)base + __popc(idle & lt);
        if (my < n) {
          ray = my;
          load_ray(R, ray, tr.o, tr.d, tr.inv, tr.tmin, tr.tmax);
          tr.start(scene_root_walk(roots, ray_off, n_scenes, ray, scene));
          active = true;
        }
      }
      if ((int64_t)base + nidle >= n) exhausted = true;
    }
    if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
      if (exhausted) break;
      continue;
    }
    if (active && tr.step(nodes, tris)) {
      if (tr.overflow) record_overflow(S, ray);
      else write_result(O, ray, ANY, tr.have, tr.prim, tr.best, tr.tmax);
      active = false;
    }
  }
}

template <int W, bool ANY, bool MT = false>
__global__ void __launch_bounds__(128)
    k_trace_retry(const NodeW<(W == 2 ? 4 : W)> *__restrict__ nodes, const Node2 *__restrict__ nodes2,
                  const TriRec *__restrict__ tris,
                  const int32_t *__restrict__ roots, const int64_t *__restrict__ ray_off, int n_scenes, RaySoA R, Out O,
                  Scratch S) {
  const uint32_t cnt = min((int64_t)*S.ovf_count, S.ovf_cap);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int64_t i = S.ovf[j];
    float3 o, d, inv;
    float tmin, tmax;
    load_ray(R, i, o, d, inv, tmin, tmax);
    const int32_t root = scene_root(roots, ray_off, n_scenes, i);
    if (W == 2) {
      bool have;
      int32_t prim;
      float best;
      if (!trace_bvh2<ANY, kRetryStack, MT>(nodes2, tris, root, o, d, inv, tmin, tmax, have, prim, best)) {
        atomicOr(S.err, kErrStack);
        continue;
      }
      write_result(O, i, ANY, have, prim, best, tmax);
    } else {
      Tracer<(W == 2 ? 4 : W), ANY, kRetryStack> tr;
      tr.o = o; tr.d = d; tr.inv = inv; tr.tmin = tmin; tr.tmax = tmax;
      tr.start(root);
      while (!tr.step(nodes, tris)) {
      }
      if (tr.overflow) atomicOr(S.err, kErrStack);
      else write_result(O, i, ANY, tr.have, tr.prim, tr.best, tr.tmax);
    }
  }
}

// ----------------------------------------------------------------------------
// Host side.
// ----------------------------------------------------------------------------

// ----------------------------------------------------------------------------
// Ray sort (flg_trace_opts.ray_sort = 1): rays of a single-scene trace are
// reordered by a 30-bit key — direction octant (3 bits) above a 27-bit Morton
// code of the origin in the scene box enlarged by its extent on every side —
// traced in that order, and their hits written back in the caller's order.
// Neighbouring lanes then start in the same region heading the same way.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_ray_keys(RaySoA R, int64_t n, const float *__restrict__ box, uint32_t *__restrict__ keys,
               uint32_t *__restrict__ hist) {
  __shared__ uint32_t s_hist[4][256];
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
  __syncthreads();
  float lo[3], sc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float e = box[3 + k] - box[k];
    lo[k] = box[k] - e;
    sc[k] = e > 0.0f ? 1.0f / (3.0f * e) : 0.0f;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float o[3] = {__ldg(R.ox + i), __ldg(R.oy + i), __ldg(R.oz + i)};
    const float d[3] = {__ldg(R.dx + i), __ldg(R.dy + i), __ldg(R.dz + i)};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float u = fminf(fmaxf((o[k] - lo[k]) * sc[k], 0.0f), 1.0f);
      q[k] = min((uint32_t)(u * 512.0f), 511u);  // NaN origins land in cell 0
    }
    const uint32_t oct = (d[0] < 0.0f ? 1u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 4u : 0u);
    const uint32_t key = (oct << 27) | (left_shift3(q[2]) << 2) | (left_shift3(q[1]) << 1) | left_shift3(q[0]);
    keys[i] = key;
#pragma unroll
    for (int p = 0; p < 4; ++p) atomicAdd(&s_hist[p][(key >> (8 * p)) & 0xFFu], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
    const uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

// Sorted position j takes ray perm[j].
__global__ void k_ray_gather(RaySoA R, int64_t n, const uint32_t *__restrict__ perm, float *__restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm[j];
    if (i < 0 || i >= n) continue;  // only a timed-out sort leaves such slots (error word set)
    out[j] = __ldg(R.ox + i);
    out[n + j] = __ldg(R.oy + i);
    out[2 * n + j] = __ldg(R.oz + i);
    out[3 * n + j] = __ldg(R.dx + i);
    out[4 * n + j] = __ldg(R.dy + i);
    out[5 * n + j] = __ldg(R.dz + i);
    out[6 * n + j] = R.tmin ? __ldg(R.tmin + i) : R.tmin_c;
    out[7 * n + j] = R.tmax ? __ldg(R.tmax + i) : R.tmax_c;
  }
}

// Hits of sorted position j go back to ray perm[j].
__global__ void k_ray_scatter(int64_t n, const uint32_t *__restrict__ perm, const int32_t *__restrict__ prim,
                              const float *__restrict__ t, const float *__restrict__ u, const float *__restrict__ v,
                              const uint8_t *__restrict__ occ, Out O) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm[j];
    if (i < 0 || i >= n) continue;
    if (occ) {
      O.occ[i] = occ[j];
    } else {
      O.prim[i] = prim[j];
      O.t[i] = t[j];
      O.u[i] = u[j];
      O.v[i] = v[j];
    }
  }
}

static int ensure_trace_scratch(flg_ctx ctx) {
  if (ctx->d_ovf) return FLG_OK;
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "first trace allocates; not allowed during capture");
  ctx->ovf_cap = 1 << 20;
  // Two sets (index 0: default stream, 1: staging second stream).
  FLG_CUDA(ctx, cudaMalloc((void **)&ctx->d_ovf, sizeof(int64_t) * ctx->ovf_cap * 2));
  FLG_CUDA(ctx, cudaMalloc((void **)&ctx->d_ovf_count, sizeof(uint32_t) * 2));
  FLG_CUDA(ctx, cudaMalloc((void **)&ctx->d_work, sizeof(unsigned long long) * 2));
  return FLG_OK;
}

static Scratch scratch_for(flg_ctx ctx, int set) {
  return Scratch{ctx->d_ovf + set * ctx->ovf_cap, ctx->d_ovf_count + set, ctx->ovf_cap, ctx->d_work + set,
                 ctx->d_err};
}

static int check_rays(flg_ctx ctx, const flg_rays *r, int64_t n) {
  if (!r) return set_error(ctx, FLG_ERR_ARG, "rays is NULL");
  if (n < 0) return set_error(ctx, FLG_ERR_ARG, "n < 0");
  if (n > 0 && (!r->ox || !r->oy || !r->oz || !r->dx || !r->dy || !r->dz))
    return set_error(ctx, FLG_ERR_ARG, "ray origin/direction pointer is NULL");
  return FLG_OK;
}

// ----------------------------------------------------------------------------
// Persistent while-while traversal with speculative leaf postponing (Aila &
// Laine, "Understanding the efficiency of ray traversal on GPUs", HPG 2009),
// on wide nodes.  Each lane walks inner nodes; a lane that reaches a leaf
// parks it (up to two) and keeps walking inner nodes until all but
// kLeafWait lanes of the warp hold a parked leaf (or have no inner node
// left); then the warp tests the parked leaves together.  Node and leaf code
// thus run with most lanes active, instead of the two branches diverging at
// every step.  Measured on config 3 (32 scenes): waiting for every lane kept
// only 37 % of the lanes at a node per node iteration; two parked leaves and
// kLeafWait = 4 give 21 % more rays/s.  Finished lanes are refilled from the
// global ray counter once `refill` of them are idle.
// ----------------------------------------------------------------------------
constexpr int kLeafWait = 4;
// Shared-memory stack entries per lane (a power of two; 32 KB per 256-thread
// CTA).  16 measured 3.7 % faster than a local-memory stack, 8 gave 2 %.
constexpr int kStackTop = 16;

template <int W, bool ANY, int STACK>
__global__ void __launch_bounds__(256, 4)
    k_trace_ww(const NodeW<W> *__restrict__ nodes, const TriRec *__restrict__ tris, const int32_t *__restrict__ roots,
               const int64_t *__restrict__ ray_off, int n_scenes, RaySoA R, int64_t n, Out O, Scratch S, int refill) {
  constexpr int32_t kNone = kEmptyChild;  // "no node" / "no parked leaf"
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt = (1u << lane) - 1u;
  float3 o = make_float3(0.f, 0.f, 0.f), d = o, inv = o;
  float tmin = 0.f, tmax = 0.f, best = 0.f;
  int32_t prim = -1, cur = kNone, leaf = kNone, leaf2 = kNone;
  int sp = 0, scene = -1;
  bool have = false, active = false, overflow = false, exhausted = false;
  int64_t ray = -1;
  // Two-level stack: the top kStackTop entries of every lane live in shared
  // memory (a ring indexed by sp, laid out [slot][thread] so that a warp's
  // accesses fall in distinct banks); deeper entries spill to the per-thread
  // local array.  Most rays never go below the shared part, so pops no longer
  // wait on local-memory misses (57 % of the local-stack loads missed L1).
  uint64_t stk[STACK];
  constexpr int KS = kStackTop;
  __shared__ uint64_t s_stk[KS][256];
  const int tid = threadIdx.x;
  auto push = [&](uint64_t e) {
    if (sp >= KS) stk[sp - KS] = s_stk[sp & (KS - 1)][tid];
    s_stk[sp & (KS - 1)][tid] = e;
    ++sp;
  };

  auto pop = [&]() -> int32_t {
    const float lim = ANY ? tmax : best;
    while (sp > 0) {
      --sp;
      const uint64_t e = s_stk[sp & (KS - 1)][tid];
      if (sp >= KS) s_stk[sp & (KS - 1)][tid] = stk[sp - KS];
      if (__uint_as_float((uint32_t)(e >> 32)) > lim) continue;
      return (int32_t)(uint32_t)e;
    }
    return kNone;
  };

  while (true) {
    // Retire finished rays.
    if (active && cur == kNone && leaf == kNone && leaf2 == kNone) {
      if (overflow) record_overflow(S, ray);
      else write_result(O, ray, ANY, have, prim, best, tmax);
      active = false;
    }
    // Refill idle lanes.
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !active);
    const int nidle = __popc(idle);
    if (!exhausted && nidle >= refill) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(S.work, (unsigned long long)nidle);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (!active) {
        const int64_t my = (int64_t)base + __popc(idle & lt);
        if (my < n) {
          ray = my;
          load_ray(R, ray, o, d, inv, tmin, tmax);
          best = tmax;
          have = false;
          overflow = false;
          prim = -1;
          sp = 0;
          leaf = kNone;
          leaf2 = kNone;
          cur = scene_root_walk(roots, ray_off, n_scenes, ray, scene);
          if (cur == INT32_MIN) cur = kNone;
          active = true;
        }
      }
      if ((int64_t)base + nidle >= n) exhausted = true;
    }
    if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
      if (exhausted) break;
      continue;
    }

    // Inner nodes, parking the first two leaves found.
    while (true) {
      if (active && cur < 0) {
        if (leaf == kNone) {
          leaf = cur;
          cur = pop();
        } else if (leaf2 == kNone) {
          leaf2 = cur;
          cur = pop();
        }
      }
      const bool at_node = active && cur >= 0 && cur != kNone;
      if (!__any_sync(0xFFFFFFFFu, at_node)) break;
      if (at_node) {
        uint32_t key[W];
        int32_t ref[W];
        const int nh = visit_node<W>(nodes + cur, o, inv, ANY ? tmax : best, key, ref);
        if (nh == 0) {
          cur = pop();
        } else {
          sort_keys<W>(key);
          if (sp + nh - 1 > STACK + KS) {
            overflow = true;
            cur = kNone;
            leaf = kNone;
            leaf2 = kNone;
          } else {
#pragma unroll
            for (int k = W - 1; k >= 1; --k)
              if (k < nh) push(key_entry<W>(key[k], ref));
            cur = key_ref<W>(key[0], ref);
          }
        }
      }
      // Leave once at most kLeafWait active lanes are still looking for
      // their first leaf: waiting for the last few cost more idle node
      // iterations than the leaf tests they would have joined.
      const bool ready = !active || leaf != kNone || cur == kNone || (cur < 0 && leaf != kNone);
      if (__popc(__ballot_sync(0xFFFFFFFFu, !ready)) <= kLeafWait) break;
    }

    // Test the (up to two) parked leaves together.
    for (int q = 0; q < 2; ++q) {
      const int32_t lf = q == 0 ? leaf : leaf2;
      if (active && lf != kNone && !(ANY && have)) {
        const int32_t enc = ~lf;
        const int64_t first = (int64_t)((uint32_t)enc >> 3);
        const int count = (enc & 7) + 1;
        for (int j = 0; j < count; ++j) {
          if (ANY) {
            if (test_tri_any(tris, first + j, o, d, tmin, tmax)) {
              have = true;
              cur = kNone;
              break;
            }
          } else {
            test_tri(tris, first + j, o, d, tmin, best, have, prim);
          }
        }
      }
    }
    leaf = kNone;
    leaf2 = kNone;
  }
}

template <int W, bool ANY>
static void launch_wide(flg_ctx ctx, cudaStream_t st, flg_bvh b, const RaySoA &R, int64_t n, const Out &O,
                        const Scratch &S, const int64_t *ray_off, int n_scenes, const flg_trace_opts &op) {
  const NodeW<W> *nodes = (const NodeW<W> *)b->d_wide;
  const int threads = op.block_threads;
  if (op.persistent == 2) {
    int per_sm = 0;
    if (op.stack_depth <= 32)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_ww<W, ANY, 32>, threads, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_ww<W, ANY, 64>, threads, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t g = std::min<int64_t>((int64_t)per_sm * ctx->num_sms, ceil_div(n, threads));
    if (g < 1) g = 1;
    const int refill = std::max(1, std::min(32, op.refill_lanes));
    if (op.stack_depth <= 32)
      k_trace_ww<W, ANY, 32><<<(unsigned)g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off, n_scenes, R,
                                                              n, O, S, refill);
    else
      k_trace_ww<W, ANY, 64><<<(unsigned)g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off, n_scenes, R,
                                                              n, O, S, refill);
  } else if (op.persistent) {
    int per_sm = 0;
    if (op.stack_depth <= 32)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_persistent<W, ANY, 32>, threads, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_persistent<W, ANY, 64>, threads, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t want = ceil_div(n, threads);
    int64_t g = std::min<int64_t>((int64_t)per_sm * ctx->num_sms, want);
    if (g < 1) g = 1;
    const int refill = std::max(1, std::min(32, op.refill_lanes));
    if (op.stack_depth <= 32)
      k_trace_persistent<W, ANY, 32><<<(unsigned)g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off,
                                                                      n_scenes, R, n, O, S, refill);
    else
      k_trace_persistent<W, ANY, 64><<<(unsigned)g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off,
                                                                      n_scenes, R, n, O, S, refill);
  } else {
    const unsigned g = (unsigned)ceil_div(n, threads);
    if (op.stack_depth <= 32)
      k_trace_wide<W, ANY, 32><<<g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off, n_scenes, R, n, O,
                                                      S);
    else
      k_trace_wide<W, ANY, 64><<<g, threads, 0, st>>>(nodes, b->d_tris, b->d_wide_root, ray_off, n_scenes, R, n, O,
                                                      S);
  }
}

// Enqueues one traversal of n rays on stream st with scratch set `set`.
// Closest hits: the hit-value pass after every traversal kernel of a call.
static int finish_enqueue(flg_ctx ctx, cudaStream_t st, const RaySoA &R, int64_t n, const Out &O, flg_bvh b,
                          bool any) {
  if (any || n <= 0) return FLG_OK;
  k_trace_finish<<<grid_for(n, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(R, n, O, b->d_tris);
  FLG_LAUNCH_CHECK(ctx, "k_trace_finish");
  stage_mark(ctx, st, "trace_finish");
  return FLG_OK;
}

int trace_enqueue(flg_ctx ctx, cudaStream_t st, int set, flg_bvh b, const flg_rays *rays, int64_t n,
                  const flg_trace_opts *opts, const int64_t *ray_off_dev, int n_scenes, flg_hits *hits,
                  uint8_t *occ) {
  flg_trace_opts op{};
  if (opts) op = *opts;
  if (op.stack_depth == 0) op.stack_depth = 64;
  if (op.block_threads == 0) op.block_threads = 256;
  if (op.refill_lanes == 0) op.refill_lanes = 16;
  if (op.stack_depth != 32 && op.stack_depth != 64) return set_error(ctx, FLG_ERR_ARG, "stack_depth must be 32 or 64");
  if (op.block_threads != 64 && op.block_threads != 128 && op.block_threads != 256)
    return set_error(ctx, FLG_ERR_ARG, "block_threads must be 64, 128 or 256");
  if (op.ray_sort != 0 && op.ray_sort != 1) return set_error(ctx, FLG_ERR_ARG, "ray_sort must be 0 or 1");
  if (op.ray_sort && (ray_off_dev || n_scenes != 1))
    return set_error(ctx, FLG_ERR_UNSUPPORTED, "ray_sort applies to single-scene traces");
  if (op.ray_sort && n > ((int64_t)1 << 28)) return set_error(ctx, FLG_ERR_UNSUPPORTED, "ray_sort: at most 2^28 rays");
  if (op.tri_test != 0 && op.tri_test != 1) return set_error(ctx, FLG_ERR_ARG, "tri_test must be 0 or 1");
  int rc = ensure_trace_scratch(ctx);
  if (rc) return rc;
  if (n == 0) return FLG_OK;
  RaySoA R{rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmin, rays->tmax,
           rays->tmin_const, rays->tmax_const};
  if (op.ray_sort) {
    // Scratch: keys and indices (2 x 2), digit counts and offsets, look-back,
    // tile counters, the sorted rays (8 arrays) and their hits (4 arrays).
    const int64_t tiles = sort_tiles(n);
    const size_t w = (size_t)n * 4;
    const size_t need = 4 * w + 2 * 4 * 256 * 4 + (size_t)4 * tiles * 256 * 4 + 64 + 8 * w + 4 * w + 16 * 256;
    if (ctx->rs_bytes < need) {
      if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "ray-sort scratch grows; not allowed during capture");
      cudaFree(ctx->rs_buf);
      ctx->rs_buf = nullptr;
      ctx->rs_bytes = 0;
      FLG_CUDA(ctx, cudaMalloc(&ctx->rs_buf, need));
      ctx->rs_bytes = need;
    }
    char *bp = (char *)ctx->rs_buf;
    auto take = [&](size_t bytes) {
      char *p = bp;
      bp += (bytes + 255) & ~(size_t)255;
      return (void *)p;
    };
    uint32_t *keys[2] = {(uint32_t *)take(w), (uint32_t *)take(w)};
    uint32_t *vals[2] = {(uint32_t *)take(w), (uint32_t *)take(w)};
    uint32_t *hist = (uint32_t *)take(2 * 4 * 256 * 4);
    uint32_t *lookback = (uint32_t *)take((size_t)4 * tiles * 256 * 4);
    uint32_t *tile_ctr = (uint32_t *)take(64);
    float *sr = (float *)take(8 * w);
    float *sh = (float *)take(4 * w);
    if (bp > (char *)ctx->rs_buf + need) return set_error(ctx, FLG_ERR_STATE, "ray-sort buffer layout");
    FLG_CUDA(ctx, cudaMemsetAsync(hist, 0, sizeof(uint32_t) * 4 * 256, st));
    const unsigned g = grid_for(n, 256, (int64_t)ctx->num_sms * 8);
    k_ray_keys<<<g, 256, 0, st>>>(R, n, b->d_scene_box, keys[0], hist);
    FLG_LAUNCH_CHECK(ctx, "k_ray_keys");
    rc = sort_pairs_enqueue(ctx, st, n, 4, keys, vals, hist, lookback, tile_ctr);
    if (rc) return rc;
    const uint32_t *perm = vals[0];  // 4 passes: the result is back in buffer 0
    k_ray_gather<<<g, 256, 0, st>>>(R, n, perm, sr);
    FLG_LAUNCH_CHECK(ctx, "k_ray_gather");
    flg_rays sorted{sr, sr + n, sr + 2 * n, sr + 3 * n, sr + 4 * n, sr + 5 * n, sr + 6 * n, sr + 7 * n, 0.0f, 0.0f};
    flg_trace_opts op2 = op;
    op2.ray_sort = 0;
    uint8_t *socc = occ ? (uint8_t *)sh : nullptr;
    flg_hits shits{(int32_t *)sh, sh + n, sh + 2 * n, sh + 3 * n};
    rc = trace_enqueue(ctx, st, set, b, &sorted, n, &op2, nullptr, 1, occ ? nullptr : &shits, socc);
    if (rc) return rc;
    Out O{hits ? hits->prim : nullptr, hits ? hits->t : nullptr, hits ? hits->u : nullptr,
          hits ? hits->v : nullptr, occ};
    k_ray_scatter<<<g, 256, 0, st>>>(n, perm, (const int32_t *)sh, sh + n, sh + 2 * n, sh + 3 * n, socc, O);
    FLG_LAUNCH_CHECK(ctx, "k_ray_scatter");
    return FLG_OK;
  }
  Out O{hits ? hits->prim : nullptr, hits ? hits->t : nullptr, hits ? hits->u : nullptr,
        hits ? hits->v : nullptr, occ};
  Scratch S = scratch_for(ctx, set);
  stage_mark(ctx, st, "start");
  FLG_CUDA(ctx, cudaMemsetAsync(S.ovf_count, 0, sizeof(uint32_t), st));
  FLG_CUDA(ctx, cudaMemsetAsync(S.work, 0, sizeof(unsigned long long), st));
  const bool any = occ != nullptr;
  if (op.tri_test == 1) {
    // The live renderer's Moller-Trumbore test: one ray per thread over the
    // BVH2 layout (kept by every handle), overflow retried with a deep stack.
    const unsigned g = (unsigned)ceil_div(n, 256);
    if (any)
      k_trace_bvh2<true, true><<<g, 256, 0, st>>>(b->d_nodes2, b->d_tris, b->d_root, ray_off_dev, n_scenes, R, n, O,
                                                  S);
    else
      k_trace_bvh2<false, true><<<g, 256, 0, st>>>(b->d_nodes2, b->d_tris, b->d_root, ray_off_dev, n_scenes, R, n, O,
                                                   S);
    FLG_LAUNCH_CHECK(ctx, "trace kernel");
    stage_mark(ctx, st, "trace");
    const unsigned rg = (unsigned)ctx->num_sms;
    if (any)
      k_trace_retry<2, true, true><<<rg, 128, 0, st>>>(nullptr, b->d_nodes2, b->d_tris, b->d_root, ray_off_dev,
                                                       n_scenes, R, O, S);
    else
      k_trace_retry<2, false, true><<<rg, 128, 0, st>>>(nullptr, b->d_nodes2, b->d_tris, b->d_root, ray_off_dev,
                                                        n_scenes, R, O, S);
    FLG_LAUNCH_CHECK(ctx, "trace retry kernel");
    stage_mark(ctx, st, "trace_retry");
    return finish_enqueue(ctx, st, R, n, O, b, any);
  }
  if (b->width == 2) {
    const unsigned g = (unsigned)ceil_div(n, 256);
    if (any)
      k_trace_bvh2<true><<<g, 256, 0, st>>>(b->d_nodes2, b->d_tris, b->d_root, ray_off_dev, n_scenes, R, n, O, S);
    else
      k_trace_bvh2<false><<<g, 256, 0, st>>>(b->d_nodes2, b->d_tris, b->d_root, ray_off_dev, n_scenes, R, n, O, S);
  } else if (b->width == 4) {
    if (any) launch_wide<4, true>(ctx, st, b, R, n, O, S, ray_off_dev, n_scenes, op);
    else launch_wide<4, false>(ctx, st, b, R, n, O, S, ray_off_dev, n_scenes, op);
  } else {
    if (any) launch_wide<8, true>(ctx, st, b, R, n, O, S, ray_off_dev, n_scenes, op);
    else launch_wide<8, false>(ctx, st, b, R, n, O, S, ray_off_dev, n_scenes, op);
  }
  FLG_LAUNCH_CHECK(ctx, "trace kernel");
  stage_mark(ctx, st, "trace");
  const unsigned rg = (unsigned)ctx->num_sms;
  const void *wide = b->d_wide;
  const int32_t *roots = b->width == 2 ? b->d_root : b->d_wide_root;
#define FLG_RETRY(WW)                                                                                       \
  if (any)                                                                                                  \
    k_trace_retry<WW, true><<<rg, 128, 0, st>>>((const NodeW<(WW == 2 ? 4 : WW)> *)wide, b->d_nodes2,       \
                                                b->d_tris, roots, ray_off_dev, n_scenes, R, O, S);          \
  else                                                                                                      \
    k_trace_retry<WW, false><<<rg, 128, 0, st>>>((const NodeW<(WW == 2 ? 4 : WW)> *)wide, b->d_nodes2,      \
                                                 b->d_tris, roots, ray_off_dev, n_scenes, R, O, S);
  if (b->width == 2) {
    FLG_RETRY(2)
  } else if (b->width == 4) {
    FLG_RETRY(4)
  } else {
    FLG_RETRY(8)
  }
#undef FLG_RETRY
  FLG_LAUNCH_CHECK(ctx, "trace retry kernel");
  stage_mark(ctx, st, "trace_retry");
  return finish_enqueue(ctx, st, R, n, O, b, any);
}

}  // namespace flg

using namespace flg;

FLG_API int flg_trace_closest(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n,
                              const flg_trace_opts *opts, flg_hits *out) {
  if (!ctx || !bvh || !out) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (n > 0 && (!out->prim || !out->t || !out->u || !out->v))
    return set_error(ctx, FLG_ERR_ARG, "hit output pointer is NULL");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle: use flg_trace_closest_batched");
  return trace_enqueue(ctx, ctx->stream, 0, bvh, rays, n, opts, nullptr, 1, out, nullptr);
}

FLG_API int flg_trace_any(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, const flg_trace_opts *opts,
                          uint8_t *occluded) {
  if (!ctx || !bvh) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (n > 0 && !occluded) return set_error(ctx, FLG_ERR_ARG, "occluded is NULL");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle: use flg_trace_closest_batched");
  return trace_enqueue(ctx, ctx->stream, 0, bvh, rays, n, opts, nullptr, 1, nullptr, occluded);
}

FLG_API int flg_trace_closest_batched(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays,
                                      const int64_t *ray_offsets_host, const flg_trace_opts *opts,
                                      flg_hits *out) {
  if (!ctx || !bvh || !out || !ray_offsets_host)
    return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  const int ns = bvh->n_scenes;
  if (ray_offsets_host[0] != 0) return set_error(ctx, FLG_ERR_ARG, "ray_offsets[0] must be 0");
  for (int s = 0; s < ns; ++s)
    if (ray_offsets_host[s + 1] < ray_offsets_host[s])
      return set_error(ctx, FLG_ERR_ARG, "ray_offsets must be non-decreasing");
  const int64_t n = ray_offsets_host[ns];
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (n > 0 && (!out->prim || !out->t || !out->u || !out->v))
    return set_error(ctx, FLG_ERR_ARG, "hit output pointer is NULL");
  // Device copy of the offsets, refreshed only when they change (so a
  // captured graph replays without a host copy).
  std::vector<int64_t> &cached = ctx->ray_off_h;
  bool same = ctx->d_ray_off && ctx->ray_off_cap >= ns + 1 && cached.size() == (size_t)(ns + 1) &&
              std::equal(cached.begin(), cached.end(), ray_offsets_host);
  if (!same) {
    if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "new ray offsets inside a capture; call once before");
    if (ctx->ray_off_cap < ns + 1) {
      cudaFree(ctx->d_ray_off);
      FLG_CUDA(ctx, cudaMalloc((void **)&ctx->d_ray_off, sizeof(int64_t) * (ns + 1)));
      ctx->ray_off_cap = ns + 1;
    }
    // Stream-ordered: earlier traces on this stream read the old offsets
    // first.  From pageable memory the source is staged before the call
    // returns, and the host does not wait for the stream's earlier work.
    FLG_CUDA(ctx, cudaMemcpyAsync(ctx->d_ray_off, ray_offsets_host, sizeof(int64_t) * (ns + 1),
                                  cudaMemcpyHostToDevice, ctx->stream));
    cached.assign(ray_offsets_host, ray_offsets_host + ns + 1);
  }
  return trace_enqueue(ctx, ctx->stream, 0, bvh, rays, n, opts, ctx->d_ray_off, ns, out, nullptr);
}

// Host-buffer entry point: chunks of rays are staged through two device
// buffers.  Every copy runs on the copy stream, in the order H0 H1 D0 H2 D1
// H3 ... (Hi: chunk i's rays in, Di: its hits out, once its trace on the
// context's stream is done), so copies overlap the traces but never each
// other: a host-to-device and a device-to-host copy that run at once each
// drop to about a third of their bandwidth alone.
FLG_API int flg_trace_closest_host(flg_ctx ctx, flg_bvh bvh, const flg_rays *rh, int64_t n,
                                   const flg_trace_opts *opts, flg_hits *oh) {
  if (!ctx || !bvh || !oh) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  int rc = check_rays(ctx, rh, n);
  if (rc) return rc;
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "host staging cannot be captured");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle");
  if (n > 0 && (!oh->prim || !oh->t || !oh->u || !oh->v))
    return set_error(ctx, FLG_ERR_ARG, "hit output pointer is NULL");
  if ((rc = ensure_trace_scratch(ctx))) return rc;
  const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 22);
  if (chunk == 0) return FLG_OK;
  // Per buffer: 8 ray arrays + 4 hit arrays, 4 bytes each.
  const size_t per_buf = (size_t)chunk * 12 * sizeof(float);
  if (ctx->stage_bytes < 2 * per_buf) {
    cudaFree(ctx->stage);
    ctx->stage = nullptr;
    ctx->stage_bytes = 0;
    FLG_CUDA(ctx, cudaMalloc(&ctx->stage, 2 * per_buf));
    ctx->stage_bytes = 2 * per_buf;
  }
  cudaStream_t cs = ctx->stream, cp = ctx->copy_stream;
  cudaEvent_t *in_done = ctx->ev, *traced = ctx->ev + 2;  // per buffer
  // The copy stream must not start before earlier work on the context's stream.
  FLG_CUDA(ctx, cudaEventRecord(traced[0], cs));
  FLG_CUDA(ctx, cudaStreamWaitEvent(cp, traced[0], 0));
  const int64_t n_chunks = (n + chunk - 1) / chunk;
  auto buffers = [&](int k, float *(&arr)[12]) {
    float *base = (float *)((char *)ctx->stage + k * per_buf);
    for (int a = 0; a < 12; ++a) arr[a] = base + (size_t)a * chunk;
  };
  auto copy_in = [&](int64_t ci) -> int {
    const int k = (int)(ci & 1);
    const int64_t c0 = ci * chunk, m = std::min(chunk, n - c0);
    float *arr[12];
    buffers(k, arr);
    const float *src[8] = {rh->ox, rh->oy, rh->oz, rh->dx, rh->dy, rh->dz, rh->tmin, rh->tmax};
    for (int a = 0; a < 8; ++a)
      if (src[a]) FLG_CUDA(ctx, cudaMemcpyAsync(arr[a], src[a] + c0, sizeof(float) * m, cudaMemcpyHostToDevice, cp));
    FLG_CUDA(ctx, cudaEventRecord(in_done[k], cp));
    return FLG_OK;
  };
  if ((rc = copy_in(0))) return rc;
  if (n_chunks > 1 && (rc = copy_in(1))) return rc;
  for (int64_t ci = 0; ci < n_chunks; ++ci) {
    const int k = (int)(ci & 1);
    const int64_t c0 = ci * chunk, m = std::min(chunk, n - c0);
    float *arr[12];
    buffers(k, arr);
    flg_rays dr{arr[0], arr[1], arr[2], arr[3], arr[4], arr[5], rh->tmin ? arr[6] : nullptr,
                rh->tmax ? arr[7] : nullptr, rh->tmin_const, rh->tmax_const};
    flg_hits dh{(int32_t *)arr[8], arr[9], arr[10], arr[11]};
    flg_trace_opts op{};
    if (opts) op = *opts;
    op.persistent = 0;
    FLG_CUDA(ctx, cudaStreamWaitEvent(cs, in_done[k], 0));
    rc = trace_enqueue(ctx, cs, k, bvh, &dr, m, &op, nullptr, 1, &dh, nullptr);
    if (rc) return rc;
    FLG_CUDA(ctx, cudaEventRecord(traced[k], cs));
    FLG_CUDA(ctx, cudaStreamWaitEvent(cp, traced[k], 0));
    FLG_CUDA(ctx, cudaMemcpyAsync(oh->prim + c0, dh.prim, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, cp));
    FLG_CUDA(ctx, cudaMemcpyAsync(oh->t + c0, dh.t, sizeof(float) * m, cudaMemcpyDeviceToHost, cp));
    FLG_CUDA(ctx, cudaMemcpyAsync(oh->u + c0, dh.u, sizeof(float) * m, cudaMemcpyDeviceToHost, cp));
    FLG_CUDA(ctx, cudaMemcpyAsync(oh->v + c0, dh.v, sizeof(float) * m, cudaMemcpyDeviceToHost, cp));
    // this buffer's next rays: after its hits are out (same stream)
    if (ci + 2 < n_chunks && (rc = copy_in(ci + 2))) return rc;
  }
  FLG_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
  FLG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return flg_ctx_sync(ctx);
}

namespace flg {

// Staged search of the traversal configuration on a given workload (node
// width and leaf size, then the kernel, then the block size; single-scene
// handles also try the ray-sort key).  Every trial is one untimed launch and
// `reps` launches timed one by one with events; the trial's time is their
// median.  Leaves the handle at the fastest layout.
struct Tuner {
  flg_ctx ctx;
  flg_bvh bvh;
  const flg_rays *rays;
  int64_t n;
  const int64_t *ray_off;
  int n_scenes, reps;
  flg_hits h;
  std::vector<cudaEvent_t> ev;
  std::string rec = "{\"trials\": [";
  bool first = true;
  float best_ms = 1e30f;
  flg_trace_opts best{};
  int best_w = 4, best_leaf = 1;

  int trial(int w, int leaf, const flg_trace_opts &op, const char *stage) {
    int rc = trace_enqueue(ctx, ctx->stream, 0, bvh, rays, n, &op, ray_off, n_scenes, &h, nullptr);
    if (rc) return rc;
    for (int r = 0; r < reps; ++r) {
      FLG_CUDA(ctx, cudaEventRecord(ev[2 * r], ctx->stream));
      rc = trace_enqueue(ctx, ctx->stream, 0, bvh, rays, n, &op, ray_off, n_scenes, &h, nullptr);
      if (rc) return rc;
      FLG_CUDA(ctx, cudaEventRecord(ev[2 * r + 1], ctx->stream));
    }
    FLG_CUDA(ctx, cudaEventSynchronize(ev[2 * reps - 1]));
    std::vector<float> ms(reps);
    for (int r = 0; r < reps; ++r) FLG_CUDA(ctx, cudaEventElapsedTime(&ms[r], ev[2 * r], ev[2 * r + 1]));
    std::sort(ms.begin(), ms.end());
    const float med = reps % 2 ? ms[reps / 2] : 0.5f * (ms[reps / 2 - 1] + ms[reps / 2]);
    char line[384];
    snprintf(line, sizeof(line),
             "%s{\"stage\": \"%s\", \"node_width\": %d, \"leaf_size\": %d, \"stack_depth\": %d, \"persistent\": %d, "
             "\"refill_lanes\": %d, \"block_threads\": %d, \"ray_sort\": %d, \"ms\": %.5f, \"ms_min\": %.5f, "
             "\"ms_max\": %.5f, \"mrays_s\": %.2f}",
             first ? "" : ", ", stage, w, leaf, op.stack_depth, op.persistent, op.refill_lanes, op.block_threads,
             op.ray_sort, med, ms.front(), ms.back(), n / (med * 1e3));
    first = false;
    rec += line;
    if (med < best_ms) {
      best_ms = med;
      best = op;
      best_w = w;
      best_leaf = leaf;
    }
    return FLG_OK;
  }

  static flg_trace_opts kernel_opts(int w, int pers, int refill, int stack, int threads) {
    flg_trace_opts op{};
    op.stack_depth = stack;
    op.persistent = w == 2 ? 0 : pers;
    op.refill_lanes = refill;
    op.block_threads = threads;
    return op;
  }

  int run() {
    int rc;
    // 1. layout, with the default kernel of each width
    for (int w : {2, 4, 8}) {
      for (int leaf : {1, 2, 3, 4}) {
        if (w == 2 && leaf > 1) continue;
        rc = flg_bvh_set_width(ctx, bvh, w, leaf);
        if (rc) return rc;
        rc = trial(w, leaf, kernel_opts(w, 2, 8, 64, 256), "layout");
        if (rc) return rc;
      }
    }
    const int w = best_w, leaf = best_leaf;
    rc = flg_bvh_set_width(ctx, bvh, w, leaf);
    if (rc) return rc;
    // 2. kernel on that layout
    if (w > 2) {
      for (int pers : {0, 1, 2})
        for (int refill : {4, 8, 16})
          for (int stack : {32, 64}) {
            if (pers == 0 && refill != 8) continue;
            if (pers == 2 && refill == 8 && stack == 64) continue;  // tried in stage 1
            rc = trial(w, leaf, kernel_opts(w, pers, refill, stack, 256), "kernel");
            if (rc) return rc;
          }
    } else {
      rc = trial(w, leaf, kernel_opts(w, 0, 8, 32, 256), "kernel");
      if (rc) return rc;
    }
    // 3. block size
    {
      flg_trace_opts op = best;
      op.block_threads = 128;
      rc = trial(w, leaf, op, "block");
      if (rc) return rc;
    }
    // 4. ray-sort key (single-scene traces): pays when neighbouring rays are
    // scattered, costs a sort and two gathers when they are not
    if (!ray_off && n_scenes == 1 && n <= ((int64_t)1 << 28)) {
      flg_trace_opts op = best;
      op.ray_sort = 1;
      rc = trial(w, leaf, op, "ray_sort");
      if (rc) return rc;
    }
    char tail[384];
    snprintf(tail, sizeof(tail),
             "], \"reps\": %d, \"rays\": %lld, \"scenes\": %d, \"best\": {\"node_width\": %d, \"leaf_size\": %d, "
             "\"stack_depth\": %d, \"persistent\": %d, \"refill_lanes\": %d, \"block_threads\": %d, \"ray_sort\": %d, "
             "\"ms\": %.5f, \"mrays_s\": %.2f}}",
             reps, (long long)n, n_scenes, best_w, best_leaf, best.stack_depth, best.persistent, best.refill_lanes,
             best.block_threads, best.ray_sort, best_ms, n / (best_ms * 1e3));
    rec += tail;
    return FLG_OK;
  }
};

static int autotune(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, const int64_t *ray_off,
                    int n_scenes, int reps, flg_trace_opts *best, int32_t *best_width, int32_t *best_leaf,
                    char *json, size_t json_len) {
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "autotuning cannot be captured");
  if (reps < 1 || reps > 64) return set_error(ctx, FLG_ERR_ARG, "reps must be in [1, 64]");
  if (n <= 0) return set_error(ctx, FLG_ERR_ARG, "autotuning needs rays");
  void *buf = nullptr;
  FLG_CUDA(ctx, cudaMalloc(&buf, sizeof(float) * 4 * (size_t)n));
  Tuner T{ctx, bvh, rays, n, ray_off, n_scenes, reps,
          flg_hits{(int32_t *)buf, (float *)buf + n, (float *)buf + 2 * n, (float *)buf + 3 * n}};
  T.ev.assign(2 * reps, nullptr);
  int rc = FLG_OK;
  for (auto &e : T.ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      rc = set_error(ctx, FLG_ERR_CUDA, "cudaEventCreate failed");
      break;
    }
  if (!rc) rc = T.run();
  for (auto &e : T.ev)
    if (e) cudaEventDestroy(e);
  cudaFree(buf);
  if (rc) return rc;
  *best = T.best;
  if (best_width) *best_width = T.best_w;
  if (best_leaf) *best_leaf = T.best_leaf;
  if (json && json_len) {
    if (T.rec.size() + 1 > json_len)
      return set_error(ctx, FLG_ERR_ARG, "json buffer too small (%zu bytes needed)", T.rec.size() + 1);
    std::memcpy(json, T.rec.c_str(), T.rec.size() + 1);
  }
  return flg_ctx_sync(ctx);
}

}  // namespace flg

FLG_API int flg_autotune_trace(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, flg_trace_opts *best,
                               int32_t *best_width, char *json, size_t json_len) {
  if (!ctx || !bvh || !best) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle: use flg_autotune_trace_batched");
  return autotune(ctx, bvh, rays, n, nullptr, 1, 5, best, best_width, nullptr, json, json_len);
}

FLG_API int flg_autotune_trace_batched(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays,
                                       const int64_t *ray_offsets_host, int32_t reps, flg_trace_opts *best,
                                       int32_t *best_width, int32_t *best_leaf, char *json, size_t json_len) {
  if (!ctx || !bvh || !best || !ray_offsets_host)
    return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  const int ns = bvh->n_scenes;
  if (ray_offsets_host[0] != 0) return set_error(ctx, FLG_ERR_ARG, "ray_offsets[0] must be 0");
  for (int s = 0; s < ns; ++s)
    if (ray_offsets_host[s + 1] < ray_offsets_host[s])
      return set_error(ctx, FLG_ERR_ARG, "ray_offsets must be non-decreasing");
  const int64_t n = ray_offsets_host[ns];
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "autotuning cannot be captured");
  if (ctx->ray_off_cap < ns + 1) {
    cudaFree(ctx->d_ray_off);
    ctx->d_ray_off = nullptr;
    ctx->ray_off_cap = 0;
    FLG_CUDA(ctx, cudaMalloc((void **)&ctx->d_ray_off, sizeof(int64_t) * (ns + 1)));
    ctx->ray_off_cap = ns + 1;
  }
  FLG_CUDA(ctx, cudaMemcpy(ctx->d_ray_off, ray_offsets_host, sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice));
  ctx->ray_off_h.assign(ray_offsets_host, ray_offsets_host + ns + 1);
  return autotune(ctx, bvh, rays, n, ctx->d_ray_off, ns, reps, best, best_width, best_leaf, json, json_len);
}

// ---------------------------------------------------------------------------
// Closest hit that allocates nothing.
//
// flg_trace_closest takes its traversal scratch (the list of rays whose short
// stack overflowed, plus two counters) from the context and allocates it with
// cudaMalloc on the context's first trace.  Some callers cannot allocate at
// that moment: a renderer recording its frame loop into a CUDA graph (an
// allocation inside a stream capture is refused), an application whose
// device memory is handed out once, up front, by its own arena (as the
// reference's Resource arena owns every allocation, src/resource.hpp:45-120),
// or a latency-critical loop in which a cudaMalloc would synchronise the
// device.  This entry point runs the same traversal kernels with the scratch
// in a fixed file-scope device array instead.
//
// The array holds the overflow list for at most kNoAllocMaxRays rays (8 MB
// plus 256 bytes of counters) and stays resident on every GPU that loads the
// library until the process exits.  All calls share it: calls that overlap
// on the GPU (concurrent streams or contexts) race on it and must not be
// issued.  Its counters are cleared at the start of every call.
// ---------------------------------------------------------------------------
constexpr int64_t kNoAllocMaxRays = int64_t(1) << 20;
// words: [0] overflow count (low 32 bits), [1] work counter, [2, 32) unused,
// [32, 32 + kNoAllocMaxRays) overflow list of ray indices
static __device__ __align__(256) unsigned long long g_noalloc_scratch[32 + kNoAllocMaxRays];

static std::mutex g_noalloc_mu;
static unsigned long long *g_noalloc_ptr[64] = {};

// Device address of the scratch array on ctx's device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device with that device current, and cached.  The lookup may load
// the library's device code, which a stream capture does not allow: a first
// call on a device inside a capture is refused, as allocating calls are.
static int noalloc_scratch(flg_ctx ctx, unsigned long long **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (ctx->device < 0 || ctx->device >= 64) return set_error(ctx, FLG_ERR_UNSUPPORTED, "device index >= 64");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!g_noalloc_ptr[ctx->device] &&
      (ctx->capturing || (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)))
    return set_error(ctx, FLG_ERR_STATE,
                     "the first flg_trace_closest_noalloc on a device looks up its scratch; not allowed during capture");
  if (!g_noalloc_ptr[ctx->device]) {
    int prev = 0;
    FLG_CUDA(ctx, cudaGetDevice(&prev));
    FLG_CUDA(ctx, cudaSetDevice(ctx->device));
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    cudaError_t e2 = cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaSetDevice");
    g_noalloc_ptr[ctx->device] = (unsigned long long *)p;
  }
  *out = g_noalloc_ptr[ctx->device];
  return FLG_OK;
}

FLG_API int flg_trace_closest_noalloc(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, flg_hits *out) {
  if (!ctx || !bvh || !out) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  int rc = check_rays(ctx, rays, n);
  if (rc) return rc;
  if (n > kNoAllocMaxRays)
    return set_error(ctx, FLG_ERR_ARG, "flg_trace_closest_noalloc: n = %lld exceeds its maximum of %lld rays",
                     (long long)n, (long long)kNoAllocMaxRays);
  if (n > 0 && (!out->prim || !out->t || !out->u || !out->v))
    return set_error(ctx, FLG_ERR_ARG, "hit output pointer is NULL");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle: use flg_trace_closest_batched");
  unsigned long long *s = nullptr;
  if ((rc = noalloc_scratch(ctx, &s))) return rc;
  if (n == 0) return FLG_OK;
  cudaStream_t st = ctx->stream;
  // Clear the shared counters left by the previous call.
  FLG_CUDA(ctx, cudaMemsetAsync(s, 0, 2 * sizeof(unsigned long long), st));
  Scratch S{(int64_t *)(s + 32), (uint32_t *)s, kNoAllocMaxRays, s + 1, ctx->d_err};
  RaySoA R{rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmin, rays->tmax,
           rays->tmin_const, rays->tmax_const};
  Out O{out->prim, out->t, out->u, out->v, nullptr};
  const unsigned g = (unsigned)ceil_div(n, 256);
  const unsigned rg = (unsigned)ctx->num_sms;
  if (bvh->width == 2) {
    k_trace_bvh2<false><<<g, 256, 0, st>>>(bvh->d_nodes2, bvh->d_tris, bvh->d_root, nullptr, 1, R, n, O, S);
    FLG_LAUNCH_CHECK(ctx, "k_trace_bvh2");
    k_trace_retry<2, false><<<rg, 128, 0, st>>>(nullptr, bvh->d_nodes2, bvh->d_tris, bvh->d_root, nullptr, 1, R, O, S);
  } else if (bvh->width == 4) {
    k_trace_wide<4, false, 64><<<g, 256, 0, st>>>((const NodeW<4> *)bvh->d_wide, bvh->d_tris, bvh->d_wide_root,
                                                  nullptr, 1, R, n, O, S);
    FLG_LAUNCH_CHECK(ctx, "k_trace_wide");
    k_trace_retry<4, false><<<rg, 128, 0, st>>>((const NodeW<4> *)bvh->d_wide, bvh->d_nodes2, bvh->d_tris,
                                                bvh->d_wide_root, nullptr, 1, R, O, S);
  } else {
    k_trace_wide<8, false, 64><<<g, 256, 0, st>>>((const NodeW<8> *)bvh->d_wide, bvh->d_tris, bvh->d_wide_root,
                                                  nullptr, 1, R, n, O, S);
    FLG_LAUNCH_CHECK(ctx, "k_trace_wide");
    k_trace_retry<8, false><<<rg, 128, 0, st>>>((const NodeW<8> *)bvh->d_wide, bvh->d_nodes2, bvh->d_tris,
                                                bvh->d_wide_root, nullptr, 1, R, O, S);
  }
  FLG_LAUNCH_CHECK(ctx, "k_trace_retry");
  return finish_enqueue(ctx, st, R, n, O, bvh, false);
}
