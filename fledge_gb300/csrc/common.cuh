// common.cuh — device-side building blocks shared by the kernels of libflg:
// Philox streams, the deterministic logarithm, the Morton spread, the slab
// test and the watertight Pluecker triangle test.
//
// Bit-exactness: every .cu file of the library is compiled with -fmad=false,
// so no multiply-add is contracted implicitly and each fp32 expression below
// rounds exactly as written (the order of the reference expressions).  Where
// a kernel wants a fused multiply-add it calls fmaf() explicitly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace flg {

// Free-flight loops stop after this many steps (degenerate or NaN rays would
// otherwise never leave the medium).
constexpr int kMaxTrackSteps = 1 << 20;

// Device error word bits (ctx->d_err); read back by flg_ctx_sync.
enum : uint32_t {
  kErrTimeout = 1u,  // a bounded spin-wait gave up
  kErrStack = 2u,    // traversal stack overflow after the deep retry
  kErrQueue = 4u,    // a work queue overflowed its reservation
};

// --------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// --------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ float u01(uint32_t x) {
  return __uint2float_rn(x >> 8) * (1.0f / 16777216.0f);
}

// Per-ray stream: draw k of ray r under seed s is word (k & 3) of
// philox({k >> 2, r_lo, r_hi, 0x7e5}, {s_lo, s_hi}).
struct RayStream {
  uint32_t k0, k1, rlo, rhi, k, cached;
  uint4 block;
  __device__ __forceinline__ void init(uint64_t seed, uint64_t ray, uint32_t start) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    rlo = (uint32_t)ray;
    rhi = (uint32_t)(ray >> 32);
    k = start;
    cached = 0xFFFFFFFFu;
  }
  __device__ __forceinline__ float next() {
    uint32_t b = k >> 2;
    if (b != cached) {
      block = philox4x32_10(make_uint4(b, rlo, rhi, 0x7e5u), k0, k1);
      cached = b;
    }
    uint32_t w = k & 3u;
    ++k;
    uint32_t x = w == 0 ? block.x : w == 1 ? block.y : w == 2 ? block.z : block.w;
    return u01(x);
  }
};

// --------------------------------------------------------------------------
// Natural logarithm for free-path sampling, identical on host and device:
//   x = m 2^e, m in [sqrt(1/2), sqrt(2)),  s = (m-1)/(m+1),
//   ln x = e ln2 + 2 (s + s^3/3 + s^5/5 + s^7/7 + s^9/9)
// (the atanh series), evaluated with plain IEEE operations.  Valid for
// normal positive x; the samplers call it on 1-u in [2^-24, 1].
// --------------------------------------------------------------------------
__device__ __forceinline__ float flg_logf(float x) {
  uint32_t b = __float_as_uint(x);
  int e = (int)(b >> 23) - 127;
  uint32_t mb = (b & 0x007FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  float m = __uint_as_float(mb);
  float s = __fdiv_rn(m - 1.0f, m + 1.0f);
  float z = s * s;
  float p = 0.11111111f;
  p = p * z;
  p = p + 0.14285715f;
  p = p * z;
  p = p + 0.2f;
  p = p * z;
  p = p + 0.33333334f;
  p = p * z;
  float sp = s * p;
  float lnm = s + sp;
  lnm = lnm + lnm;
  float fe = (float)e;
  float hi = fe * 0.693145752f;
  float lo = fe * 1.42860677e-06f;
  return hi + (lnm + lo);
}

// --------------------------------------------------------------------------
// Morton spread (LeftShift3, experimental_utils.hpp:33-40).
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t left_shift3(uint32_t x) {
  if (x == (1u << 10)) --x;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

// float -> uint32 of the normalised coordinate; truncation as the implicit
// conversion in EncodeMorton3 (experimental_utils.hpp:42-45); non-positive and
// NaN (zero-extent axis) map to 0.
__device__ __forceinline__ uint32_t to_u32(float v) {
  return (v > 0.0f) ? __float2uint_rz(v) : 0u;
}

struct Box {
  float lo[3], hi[3];
};

// --------------------------------------------------------------------------
// Slab test (BoundIntersect, intersector.hpp:103-120): t0 starts at 0 and t1
// at FLT_MAX; a NaN slab (0 * inf) leaves the interval unchanged, as the
// reference's compare-and-swap does.  Returns tnear, or NaN on a miss (so
// that `t <= limit` is false on a miss even when the limit is +inf).
// --------------------------------------------------------------------------
__device__ __forceinline__ float slab1(float lo, float hi, float o, float inv, float &t0, float &t1) {
  float tn = (lo - o) * inv;
  float tf = (hi - o) * inv;
  bool s = tn > tf;
  float a = s ? tf : tn;
  float b = s ? tn : tf;
  t0 = fmaxf(a, t0);
  t1 = fminf(b, t1);
  return 0.0f;
}

__device__ __forceinline__ float slab_tnear(float lox, float hix, float loy, float hiy, float loz,
                                            float hiz, const float3 &o, const float3 &inv) {
  float t0 = 0.0f, t1 = 3.402823466e+38f;
  slab1(lox, hix, o.x, inv.x, t0, t1);
  slab1(loy, hiy, o.y, inv.y, t0, t1);
  slab1(loz, hiz, o.z, inv.z, t0, t1);
  return t0 > t1 ? __int_as_float(0x7fffffff) : t0;
}

// --------------------------------------------------------------------------
// Watertight Pluecker test (PlueckerTriangleIntersect, intersector.hpp:
// 63-101) with the normal left unnormalised: t = dot(v0,N)/dot(N,D) (the
// factor 2 of Twice() cancels exactly), u = U/(U+V+W), v = V/(U+V+W).
// Returns false on a miss; otherwise t (not yet range-checked), u, v.
// --------------------------------------------------------------------------
__device__ __forceinline__ float3 f3sub(float3 a, float3 b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 f3add(float3 a, float3 b) {
  return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float f3dot(float3 a, float3 b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float3 f3cross(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Hit test and t only; U, V and U+V+W are returned for the barycentrics.
__device__ __forceinline__ bool pluecker_core(float3 a, float3 b, float3 c, float3 O, float3 D, float &t, float &U,
                                              float &V, float &UVW) {
  float3 v0 = f3sub(a, O), v1 = f3sub(b, O), v2 = f3sub(c, O);
  float3 e0 = f3sub(v2, v0), e1 = f3sub(v0, v1), e2 = f3sub(v1, v2);
  U = f3dot(f3cross(e0, f3add(v2, v0)), D);
  V = f3dot(f3cross(e1, f3add(v0, v1)), D);
  float W = f3dot(f3cross(e2, f3add(v1, v2)), D);
  UVW = U + V + W;
  float eps = 1.1920928955078125e-07f * fabsf(UVW);
  bool valid = fminf(U, fminf(V, W)) >= -eps || fmaxf(U, fmaxf(V, W)) <= eps;
  if (!valid) return false;
  // StableTriangleNormal (intersector.hpp:45-60)
  float ab_x = e0.z * e1.y, ab_y = e0.x * e1.z, ab_z = e0.y * e1.x;
  float bc_x = e1.z * e2.y, bc_y = e1.x * e2.z, bc_z = e1.y * e2.x;
  float3 N;
  N.x = fabsf(ab_x) < fabsf(bc_x) ? e0.y * e1.z - ab_x : e1.y * e2.z - bc_x;
  N.y = fabsf(ab_y) < fabsf(bc_y) ? e0.z * e1.x - ab_y : e1.z * e2.x - bc_y;
  N.z = fabsf(ab_z) < fabsf(bc_z) ? e0.x * e1.y - ab_z : e1.x * e2.y - bc_z;
  float den = f3dot(N, D);
  float T = f3dot(v0, N);
  float tt = __fdiv_rn(T, den);
  if (!(0.0f <= tt)) return false;
  if (!(den != 0.0f)) return false;
  t = tt;
  return true;
}

// Triangle::intersect of the live renderer (shape.cpp:100-148): Moller-
// Trumbore, not watertight; zero-area triangles never hit (area() == 0);
// accepts 0 < t, the caller applies t < tMax.  Same operation order as the
// reference (its Dot/Cross/Norm, vector.h:364-404).
__device__ __forceinline__ bool moller_t(float3 p0, float3 p1, float3 p2, float3 O, float3 D, float &t) {
  const float3 e1 = f3sub(p1, p0), e2 = f3sub(p2, p0);
  const float3 n = f3cross(e1, e2);
  if (sqrtf(f3dot(n, n)) / 2.0f == 0.0f) return false;
  const float3 p = f3cross(D, e2);
  const float d = f3dot(e1, p);
  const float inv_det = __frcp_rn(d);
  if (d == 0.0f) return false;
  const float3 tv = f3sub(O, p0);
  const float u = f3dot(tv, p) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const float3 q = f3cross(tv, e1);
  const float v = f3dot(D, q) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  const float tn = f3dot(e2, q) * inv_det;
  if (!(tn > 0.0f)) return false;
  t = tn;
  return true;
}

// The traversal's test: t only (the closest hit's barycentrics are formed
// once, for the winner).
__device__ __forceinline__ bool pluecker_t(float3 a, float3 b, float3 c, float3 O, float3 D, float &t) {
  float U, V, UVW;
  return pluecker_core(a, b, c, O, D, t, U, V, UVW);
}

__device__ __forceinline__ bool pluecker(float3 a, float3 b, float3 c, float3 O, float3 D, float &t,
                                         float &u, float &v) {
  float U, V, UVW;
  if (!pluecker_core(a, b, c, O, D, t, U, V, UVW)) return false;
  if (UVW != 0.0f) {
    u = __fdiv_rn(U, UVW);
    v = __fdiv_rn(V, UVW);
  } else {
    u = 0.0f;
    v = 0.0f;
  }
  return true;
}

// --------------------------------------------------------------------------
// Float-float ("double-word") arithmetic on the FP32 pipe: a value is an
// unevaluated sum hi + lo of two floats (error-free transforms of Knuth and
// Dekker; multiplication with FMA, as analysed by Joldes, Muller and Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic", 2017).  About 44 significant bits.  GB300's FP64 rate is far
// too low for a per-ray step, so the refinement below uses this instead.
// --------------------------------------------------------------------------
struct dfl {
  float hi, lo;
};
__device__ __forceinline__ dfl two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
  dfl s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
  dfl v = fast_two_sum(s.hi, s.lo + t.hi);
  return fast_two_sum(v.hi, t.lo + v.lo);
}
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, dfl{-y.hi, -y.lo}); }
__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
  float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl df_mulf(dfl x, float y) {
  float p = x.hi * y;
  float e = fmaf(x.hi, y, -p);
  e = fmaf(x.lo, y, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl df_div(dfl x, dfl y) {
  float q1 = x.hi / y.hi;
  dfl r = df_sub(x, df_mulf(y, q1));
  float q2 = r.hi / y.hi;
  return fast_two_sum(q1, q2);
}

// Hit values of the selected triangle recomputed in float-float and rounded
// once to fp32: t = (v0.N)/(N.D) with N = e0 x e1, and the barycentrics of
// the Pluecker test, u = U/S and v = V/S with S = U+V+W = 2 N.D, through
// the identities U = 2 e0.(v0 x D) and V = 2 e1.(v0 x D) (the vertex sums of
// U and V are 2 v0 + e0 and 2 v0 - e1), so u = e0.w / N.D and v = e1.w / N.D
// with one float-float cross product w = v0 x D.  The fp32 test decides
// hit/miss and which triangle is closest; this makes the reported t, u, v
// accurate to about an ulp even for grazing rays, where the fp32 quotients
// lose digits.  Edges are formed exactly (e0 = c - a, e1 = a - b as
// float-float).  Returns false, leaving the inputs unchanged, when N.D is
// zero.
__device__ __forceinline__ bool refine_tuv(float3 a, float3 b, float3 c, float3 O, float3 D, float &t, float &u,
                                           float &v) {
  const dfl e0x = two_sum(c.x, -a.x), e0y = two_sum(c.y, -a.y), e0z = two_sum(c.z, -a.z);
  const dfl e1x = two_sum(a.x, -b.x), e1y = two_sum(a.y, -b.y), e1z = two_sum(a.z, -b.z);
  const dfl v0x = two_sum(a.x, -O.x), v0y = two_sum(a.y, -O.y), v0z = two_sum(a.z, -O.z);
  // w = v0 x D
  const dfl wx = df_sub(df_mulf(v0y, D.z), df_mulf(v0z, D.y));
  const dfl wy = df_sub(df_mulf(v0z, D.x), df_mulf(v0x, D.z));
  const dfl wz = df_sub(df_mulf(v0x, D.y), df_mulf(v0y, D.x));
  // N = e0 x e1
  const dfl Nx = df_sub(df_mul(e0y, e1z), df_mul(e0z, e1y));
  const dfl Ny = df_sub(df_mul(e0z, e1x), df_mul(e0x, e1z));
  const dfl Nz = df_sub(df_mul(e0x, e1y), df_mul(e0y, e1x));
  const dfl den = df_add(df_add(df_mulf(Nx, D.x), df_mulf(Ny, D.y)), df_mulf(Nz, D.z));
  if (den.hi == 0.0f) return false;
  const dfl num = df_add(df_add(df_mul(v0x, Nx), df_mul(v0y, Ny)), df_mul(v0z, Nz));
  const dfl U = df_add(df_add(df_mul(e0x, wx), df_mul(e0y, wy)), df_mul(e0z, wz));
  const dfl V = df_add(df_add(df_mul(e1x, wx), df_mul(e1y, wy)), df_mul(e1z, wz));
  const dfl tt = df_div(num, den), uu = df_div(U, den), vv = df_div(V, den);
  t = tt.hi + tt.lo;
  u = uu.hi + uu.lo;
  v = vv.hi + vv.lo;
  return true;
}

// Accept a candidate t for closest hit: tmin <= t, and t < best (or t == best
// when nothing has been accepted yet, so that t == tmax counts as in the
// reference's `thit > tfar` rejection).
__device__ __forceinline__ bool accept_closest(float t, float tmin, float best, bool have) {
  return t >= tmin && (t < best || (!have && t == best));
}

// --------------------------------------------------------------------------
// Bounded spin on a global word (mbarrier-free waits of the look-back and the
// work queues).  Returns false when the limit was reached.
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *(const volatile uint32_t *)p;
}

// Waits until (*p & mask) != 0 and returns the word; after `limit` polls
// (with a short back-off) sets kErrTimeout in *err and returns 0.
__device__ __forceinline__ uint32_t wait_flag(const uint32_t *p, uint32_t mask, uint32_t limit,
                                              uint32_t *err) {
  for (uint32_t spins = 0;; ++spins) {
    uint32_t s = ld_volatile(p);
    if (s & mask) return s;
    if (spins >= limit) {
      atomicOr(err, kErrTimeout);
      return 0u;
    }
    if (spins > 64) __nanosleep(64);
  }
}

// Binary search: largest s with off[s] <= x (off ascending, off[0] = 0).
__device__ __forceinline__ int find_segment(const int64_t *off, int n_seg, int64_t x) {
  int lo = 0, hi = n_seg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// find_segment over 32-bit offsets.
__device__ __forceinline__ int find_segment32(const int32_t *off, int n_seg, int32_t x) {
  int lo = 0, hi = n_seg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Vertices of triangle t of a soup (idx NULL) or an indexed mesh.
__device__ __forceinline__ void tri_verts(const float *__restrict__ pos, const int32_t *__restrict__ idx,
                                          int64_t t, float3 &a, float3 &b, float3 &c) {
  int64_t i0, i1, i2;
  if (idx) {
    i0 = idx[3 * t];
    i1 = idx[3 * t + 1];
    i2 = idx[3 * t + 2];
  } else {
    i0 = 3 * t;
    i1 = 3 * t + 1;
    i2 = 3 * t + 2;
  }
  a = make_float3(pos[3 * i0], pos[3 * i0 + 1], pos[3 * i0 + 2]);
  b = make_float3(pos[3 * i1], pos[3 * i1 + 1], pos[3 * i1 + 2]);
  c = make_float3(pos[3 * i2], pos[3 * i2 + 1], pos[3 * i2 + 2]);
}

// BVHBuilderBase::Triangle::getBound (base_bvh.hpp:90-102): std::min/max
// order; fminf/fmaxf agree on finite input up to the sign of zero.
__device__ __forceinline__ void tri_box(float3 a, float3 b, float3 c, float *lo, float *hi) {
  lo[0] = fminf(fminf(a.x, b.x), c.x);
  lo[1] = fminf(fminf(a.y, b.y), c.y);
  lo[2] = fminf(fminf(a.z, b.z), c.z);
  hi[0] = fmaxf(fmaxf(a.x, b.x), c.x);
  hi[1] = fmaxf(fmaxf(a.y, b.y), c.y);
  hi[2] = fmaxf(fmaxf(a.z, b.z), c.z);
}

}  // namespace flg
