// oracle.cpp — CPU restatement of fledge's acceleration-structure and
// participating-media hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library in
// fledge_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline legs load it.  The product path never calls into it.
//
// Every function cites the reference source it restates (paths are relative
// to the fledge project root).  The reference itself cannot be compiled here:
// radix_bvh.cpp / base_bvh.hpp need TBB and Embree headers, volume.cpp needs
// OpenVDB and debug.hpp needs fmt, none of which exist on this machine.
// Parity status:
//   * Morton codes, sorted order, Karras topology, refit bounds, Pluecker
//     hit/miss and closest-hit selection: restated line by line; pinned only
//     by the reference's own property tests (watertight mesh, two accelerators
//     agree exactly) because the reference ships no golden vectors.
//   * OpenVDB trilinear sampling and world transform: PARITY UNPINNED (the
//     dense vertex-centred lattice below is this project's definition).
//   * Embree / TBB: PARITY UNPINNED (absent); the TBB sort is unstable, the
//     defined tie order is (code, original index).
//
// Arithmetic modes.  Compiled with -ffp-contract=off so that no multiply-add
// is fused; every fp32 expression is evaluated exactly in the order written,
// which is the order of the reference expressions (Dot = (x0*y0 + x1*y1) +
// x2*y2, Cross as in common/vector.h:399-404).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif
#include <parallel/algorithm>

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace {

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11).  The reference draws with std::mt19937
// (rng.hpp:21-34); the hot path fixes per-ray counter-based streams instead so
// that the adjoint can replay them.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

inline U4 philox(U4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Free-flight loops stop after this many steps (same cap as the GPU kernels).
constexpr int kMaxTrackSteps = 1 << 20;

// Per-ray stream: draw k of ray r under seed s is word (k & 3) of
// philox({k >> 2, r_lo, r_hi, 0x7e5}, {s_lo, s_hi}).
struct RayStream {
  uint32_t k0, k1, rlo, rhi;
  uint32_t k = 0;
  U4 block{};
  uint32_t cached = 0xFFFFFFFFu;
  float next() {
    uint32_t b = k >> 2;
    if (b != cached) {
      block = philox(U4{b, rlo, rhi, 0x7e5u}, k0, k1);
      cached = b;
    }
    uint32_t w = k & 3;
    ++k;
    uint32_t x = w == 0 ? block.x : w == 1 ? block.y : w == 2 ? block.z : block.w;
    return u01(x);
  }
};

// ---------------------------------------------------------------------------
// Natural logarithm used by the free-path sampler.  The reference calls
// std::log (volume.cpp:187,226); libm and the GPU's logf do not round alike,
// so both sides use this restatement of the textbook reduction
//   x = m * 2^e,  m in [sqrt(1/2), sqrt(2)),
//   ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + s^7/7 + s^9/9),  s=(m-1)/(m+1)
// evaluated with plain IEEE fp32 operations, giving bit-identical step
// lengths on host and device.
// ---------------------------------------------------------------------------
inline float flg_logf(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  int e = (int)(b >> 23) - 127;
  uint32_t mb = (b & 0x007FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) {  // m > sqrt(2)
    mb -= 0x00800000u;
    e += 1;
  }
  float m;
  std::memcpy(&m, &mb, 4);
  float s = (m - 1.0f) / (m + 1.0f);
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

// ---------------------------------------------------------------------------
// Bounds (experimental/base_bvh.hpp:53-60, 90-102).
// ---------------------------------------------------------------------------
struct Bound {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void merge(const Bound &o) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], o.lo[k]);
      hi[k] = std::max(hi[k], o.hi[k]);
    }
  }
};

struct Mesh {
  const float *pos;
  const int32_t *idx;  // nullptr: triangle soup, vertex k of tri i = 3i+k
  int64_t n_tri;
  const float *v(int64_t tri, int k) const {
    int64_t vi = idx ? (int64_t)idx[3 * tri + k] : 3 * tri + k;
    return pos + 3 * vi;
  }
  Bound bound(int64_t tri) const {
    // BVHBuilderBase::Triangle::getBound (base_bvh.hpp:90-102)
    const float *p0 = v(tri, 0), *p1 = v(tri, 1), *p2 = v(tri, 2);
    Bound b;
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = std::min(std::min(p0[k], p1[k]), p2[k]);
      b.hi[k] = std::max(std::max(p0[k], p1[k]), p2[k]);
    }
    return b;
  }
};

// experimental_utils.hpp:33-40 (LeftShift3) and :42-45 (EncodeMorton3)
inline uint32_t left_shift3(uint32_t x) {
  if (x == (1u << 10)) --x;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

// float -> uint32 conversion of the normalised coordinate (the implicit
// conversion at experimental_utils.hpp:43-44).  A zero-extent axis divides 0
// by 0 in the reference (undefined conversion); here it is defined as 0.
inline uint32_t to_u32(float v) {
  if (!(v > 0.0f)) return 0u;
  return (uint32_t)v;
}

// radix_bvh.cpp:63-73 (prestage Morton loop)
inline uint32_t morton_of(const Bound &tb, const Bound &scene) {
  float e[3], n[3];
  for (int k = 0; k < 3; ++k) {
    e[k] = scene.hi[k] - scene.lo[k];
    float c = (tb.lo[k] + tb.hi[k]) / 2.0f;
    n[k] = e[k] == 0.0f ? 0.0f : (c - scene.lo[k]) / e[k];
    n[k] = n[k] * 1024.0f;
  }
  return (left_shift3(to_u32(n[2])) << 2) | (left_shift3(to_u32(n[1])) << 1) |
         left_shift3(to_u32(n[0]));
}

// experimental_utils.hpp:27-31: pow(2, ceil(log2(n))) for n >= 1
inline int next2pow(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

struct Karras {
  const uint32_t *code;
  int n;
  // radix_bvh.hpp:68-74
  inline int delta(int i, int j) const {
    if (j < 0 || j >= n) return -1;
    if (code[i] == code[j]) return __builtin_clz((uint32_t)(i ^ j)) + 32;
    return __builtin_clz(code[i] ^ code[j]);
  }
};

// ---------------------------------------------------------------------------
// Pluecker ray/triangle test (experimental/intersector.hpp:45-101).
// Mode REF: the reference formula; the normal is normalised in double with
//   the Euclidean norm.  The reference's StableNormalize (common/vector.h:
//   495-503) adds z instead of z*z; mode DEFECT restates that literally, which
//   yields a NaN normal (and a miss) whenever x*x + y*y + 2z < 0.
// Mode DEV: the same test with the normal left unnormalised; this is the
//   arithmetic the GPU kernels use (the factor 2 of Twice() cancels exactly).
// u = U/(U+V+W), v = V/(U+V+W) (Embree's barycentric convention; the reference
// computes U, V, W but returns no barycentrics).
// ---------------------------------------------------------------------------
enum { MODE_REF = 0, MODE_DEFECT = 1, MODE_DEV = 2, MODE_MT = 3 };

struct V3 { float x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 ld3(const float *p) { return {p[0], p[1], p[2]}; }

// intersector.hpp:45-60
inline V3 stable_triangle_normal(V3 a, V3 b, V3 c) {
  float ab_x = a.z * b.y, ab_y = a.x * b.z, ab_z = a.y * b.x;
  float bc_x = b.z * c.y, bc_y = b.x * c.z, bc_z = b.y * c.x;
  V3 cab = {a.y * b.z - ab_x, a.z * b.x - ab_y, a.x * b.y - ab_z};
  V3 cbc = {b.y * c.z - bc_x, b.z * c.x - bc_y, b.x * c.y - bc_z};
  return {std::fabs(ab_x) < std::fabs(bc_x) ? cab.x : cbc.x,
          std::fabs(ab_y) < std::fabs(bc_y) ? cab.y : cbc.y,
          std::fabs(ab_z) < std::fabs(bc_z) ? cab.z : cbc.z};
}

struct Hit { float t, u, v; };

// Triangle::intersect of the live renderer (shape.cpp:100-148): Moller-
// Trumbore, not watertight; degenerate (zero-area) triangles never hit;
// accepts 0 < t (the caller applies t < tMax).
inline bool moller(V3 p0, V3 p1, V3 p2, V3 O, V3 D, Hit *h) {
  const V3 e1 = sub(p1, p0), e2 = sub(p2, p0);
  const V3 n = cross(e1, e2);
  if (std::sqrt(dot(n, n)) / 2.0f == 0.0f) return false;  // area() == 0
  const V3 p = cross(D, e2);
  const float d = dot(e1, p);
  const float inv_det = 1.0f / d;
  if (d == 0.0f) return false;
  const V3 t = sub(O, p0);
  const float u = dot(t, p) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const V3 q = cross(t, e1);
  const float v = dot(D, q) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  const float tn = dot(e2, q) * inv_det;
  if (!(tn > 0.0f)) return false;
  h->t = tn;
  h->u = u;
  h->v = v;
  return true;
}

inline bool pluecker(V3 a, V3 b, V3 c, V3 O, V3 D, int mode, Hit *h, V3 *ng_out = nullptr) {
  if (mode == MODE_MT) return moller(a, b, c, O, D, h);
  V3 v0 = sub(a, O), v1 = sub(b, O), v2 = sub(c, O);
  V3 e0 = sub(v2, v0), e1 = sub(v0, v1), e2 = sub(v1, v2);
  float U = dot(cross(e0, add(v2, v0)), D);
  float V = dot(cross(e1, add(v0, v1)), D);
  float W = dot(cross(e2, add(v1, v2)), D);
  float UVW = U + V + W;
  float eps = FLT_EPSILON * std::fabs(UVW);
  bool valid = std::min(U, std::min(V, W)) >= -eps || std::max(U, std::max(V, W)) <= eps;
  if (!valid) return false;
  V3 Ng = stable_triangle_normal(e0, e1, e2);
  if (mode != MODE_DEV) {
    double x = Ng.x, y = Ng.y, z = Ng.z;
    double sq = mode == MODE_DEFECT ? x * x + y * y + z + z : x * x + y * y + z * z;
    double r = std::sqrt(sq);
    Ng = {(float)(x / r), (float)(y / r), (float)(z / r)};
  }
  float den = dot(Ng, D);
  den = den + den;
  float T = dot(v0, Ng);
  T = T + T;
  float t = T / den;
  if (!(0.0f <= t)) return false;
  if (!(den != 0.0f)) return false;
  h->t = t;
  h->u = UVW != 0.0f ? U / UVW : 0.0f;
  h->v = UVW != 0.0f ? V / UVW : 0.0f;
  if (ng_out) *ng_out = Ng;  // the normal the reference stores in BVHRayHit::hit_ng
  return true;
}

// Same test in double precision end to end (the FP64 oracle for t, u, v).
inline bool pluecker64(const float *fa, const float *fb, const float *fc, const double *O,
                       const double *D, double *t, double *u, double *v) {
  double a[3], b[3], c[3], v0[3], v1[3], v2[3], e0[3], e1[3], e2[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = fa[k]; b[k] = fb[k]; c[k] = fc[k];
    v0[k] = a[k] - O[k]; v1[k] = b[k] - O[k]; v2[k] = c[k] - O[k];
  }
  for (int k = 0; k < 3; ++k) {
    e0[k] = v2[k] - v0[k]; e1[k] = v0[k] - v1[k]; e2[k] = v1[k] - v2[k];
  }
  auto crs = [](const double *p, const double *q, double *r) {
    r[0] = p[1] * q[2] - p[2] * q[1];
    r[1] = p[2] * q[0] - p[0] * q[2];
    r[2] = p[0] * q[1] - p[1] * q[0];
  };
  auto dt = [](const double *p, const double *q) { return p[0] * q[0] + p[1] * q[1] + p[2] * q[2]; };
  double s0[3], s1[3], s2[3], cr[3];
  for (int k = 0; k < 3; ++k) { s0[k] = v2[k] + v0[k]; s1[k] = v0[k] + v1[k]; s2[k] = v1[k] + v2[k]; }
  crs(e0, s0, cr); double U = dt(cr, D);
  crs(e1, s1, cr); double V = dt(cr, D);
  crs(e2, s2, cr); double W = dt(cr, D);
  double S = U + V + W;
  double N[3];
  crs(e0, e1, N);
  double den = dt(N, D);
  if (den == 0.0 || S == 0.0) return false;
  *t = dt(v0, N) / den;
  *u = U / S;
  *v = V / S;
  return true;
}

// Float-float arithmetic (error-free transforms: Knuth/Dekker two-sum, FMA
// two-product; Joldes, Muller, Popescu 2017).  std::fmaf is correctly rounded,
// as is the GPU's fmaf, so these routines give the same bits on both sides.
struct Dfl { float hi, lo; };
inline Dfl two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline Dfl fast_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
inline Dfl df_add(Dfl x, Dfl y) {
  Dfl s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
  Dfl v = fast_two_sum(s.hi, s.lo + t.hi);
  return fast_two_sum(v.hi, t.lo + v.lo);
}
inline Dfl df_sub(Dfl x, Dfl y) { return df_add(x, Dfl{-y.hi, -y.lo}); }
inline Dfl df_mul(Dfl x, Dfl y) {
  float p = x.hi * y.hi;
  float e = std::fmaf(x.hi, y.hi, -p);
  e = std::fmaf(x.hi, y.lo, e);
  e = std::fmaf(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}
inline Dfl df_mulf(Dfl x, float y) {
  float p = x.hi * y;
  float e = std::fmaf(x.hi, y, -p);
  e = std::fmaf(x.lo, y, e);
  return fast_two_sum(p, e);
}
inline Dfl df_div(Dfl x, Dfl y) {
  float q1 = x.hi / y.hi;
  Dfl r = df_sub(x, df_mulf(y, q1));
  float q2 = r.hi / y.hi;
  return fast_two_sum(q1, q2);
}

// Reported hit values of the GPU path: the selected triangle's Pluecker t,
// u, v recomputed in float-float and rounded once: t = (v0.N)/(N.D),
// N = e0 x e1; u = U/S, v = V/S, S = 2 N.D, through U = 2 e0.(v0 x D) and
// V = 2 e1.(v0 x D), i.e. u = e0.w / N.D, v = e1.w / N.D, w = v0 x D.
inline void refine_tuv(const float *a, const float *b, const float *c, const float *O, const float *D, float &t,
                       float &u, float &v) {
  Dfl e0[3], e1[3], v0[3], w[3], N[3];
  for (int k = 0; k < 3; ++k) {
    e0[k] = two_sum(c[k], -a[k]);
    e1[k] = two_sum(a[k], -b[k]);
    v0[k] = two_sum(a[k], -O[k]);
  }
  w[0] = df_sub(df_mulf(v0[1], D[2]), df_mulf(v0[2], D[1]));
  w[1] = df_sub(df_mulf(v0[2], D[0]), df_mulf(v0[0], D[2]));
  w[2] = df_sub(df_mulf(v0[0], D[1]), df_mulf(v0[1], D[0]));
  N[0] = df_sub(df_mul(e0[1], e1[2]), df_mul(e0[2], e1[1]));
  N[1] = df_sub(df_mul(e0[2], e1[0]), df_mul(e0[0], e1[2]));
  N[2] = df_sub(df_mul(e0[0], e1[1]), df_mul(e0[1], e1[0]));
  Dfl den = df_add(df_add(df_mulf(N[0], D[0]), df_mulf(N[1], D[1])), df_mulf(N[2], D[2]));
  if (den.hi == 0.0f) return;
  auto dot = [](const Dfl *x, const Dfl *y) {
    return df_add(df_add(df_mul(x[0], y[0]), df_mul(x[1], y[1])), df_mul(x[2], y[2]));
  };
  Dfl num = dot(v0, N), U = dot(e0, w), V = dot(e1, w);
  Dfl tt = df_div(num, den), uu = df_div(U, den), vv = df_div(V, den);
  t = tt.hi + tt.lo;
  u = uu.hi + uu.lo;
  v = vv.hi + vv.lo;
}

// BoundIntersect (intersector.hpp:103-120): t0 starts at 0, t1 at FLT_MAX.
inline bool bound_intersect(const float *lo, const float *hi, const float *o, const float *inv,
                            float *tnear) {
  float t0 = 0.0f, t1 = FLT_MAX;
  for (int i = 0; i < 3; ++i) {
    float tn = (lo[i] - o[i]) * inv[i];
    float tf = (hi[i] - o[i]) * inv[i];
    if (tn > tf) std::swap(tn, tf);
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
    if (t0 > t1) return false;
  }
  *tnear = t0;
  return true;
}

struct Tree {
  int64_t n;
  const int32_t *perm;      // sorted position -> original triangle
  const int32_t *split;     // n-1
  const uint8_t *leaf;      // n-1: bit0 left child is a leaf, bit1 right child
  const float *nb;          // 6*(n-1): node bound lo xyz hi xyz
};

struct RayIn {
  float o[3], d[3], inv[3], tmin, tmax;
};

struct Best {
  float tfar;
  int32_t prim;
  float u, v;
};

// radix_bvh.cpp:202-245 (recursiveIntersect), extended with tmin, prim id and
// barycentrics.  Leaves are tested left then right; a hit is kept unless
// thit > tfar, so an equal-t hit found later replaces the earlier one.
void recursive_intersect(const Tree &T, const Mesh &M, int node, const RayIn &r, int mode, Best &b) {
  float tnear;
  const float *nb = T.nb + 6 * (int64_t)node;
  if (!bound_intersect(nb, nb + 3, r.o, r.inv, &tnear)) return;
  if (b.tfar < tnear) return;
  int s = T.split[node];
  uint8_t lf = T.leaf[node];
  V3 O = ld3(r.o), D = ld3(r.d);
  for (int side = 0; side < 2; ++side) {
    if (!(lf & (1 << side))) continue;
    int tri = T.perm[s + side];
    Hit h;
    if (!pluecker(ld3(M.v(tri, 0)), ld3(M.v(tri, 1)), ld3(M.v(tri, 2)), O, D, mode, &h)) continue;
    if (h.t > b.tfar) continue;
    if (mode == MODE_MT && !(h.t < b.tfar)) continue;  // the live renderer rejects t >= tMax
    if (h.t < r.tmin) continue;
    b.tfar = h.t;
    b.prim = tri;
    b.u = h.u;
    b.v = h.v;
  }
  if (!(lf & 1)) recursive_intersect(T, M, s, r, mode, b);
  if (!(lf & 2)) recursive_intersect(T, M, s + 1, r, mode, b);
}

// Any-hit: the reference has no IntersectP (shadow rays use closest-hit,
// integrator.cpp:29-37); this terminates at the first accepted hit in
// [tmin, tmax] using the same node and triangle tests.
bool recursive_occluded(const Tree &T, const Mesh &M, int node, const RayIn &r, int mode) {
  float tnear;
  const float *nb = T.nb + 6 * (int64_t)node;
  if (!bound_intersect(nb, nb + 3, r.o, r.inv, &tnear)) return false;
  if (r.tmax < tnear) return false;
  int s = T.split[node];
  uint8_t lf = T.leaf[node];
  V3 O = ld3(r.o), D = ld3(r.d);
  for (int side = 0; side < 2; ++side) {
    if (!(lf & (1 << side))) continue;
    int tri = T.perm[s + side];
    Hit h;
    if (!pluecker(ld3(M.v(tri, 0)), ld3(M.v(tri, 1)), ld3(M.v(tri, 2)), O, D, mode, &h)) continue;
    if (h.t > r.tmax || h.t < r.tmin || (mode == MODE_MT && !(h.t < r.tmax))) continue;
    return true;
  }
  if (!(lf & 1) && recursive_occluded(T, M, s, r, mode)) return true;
  if (!(lf & 2) && recursive_occluded(T, M, s + 1, r, mode)) return true;
  return false;
}

inline RayIn make_ray(const float *rays, int64_t i, int64_t n) {
  // rays: SoA of 8 arrays of n floats: ox oy oz dx dy dz tmin tmax
  RayIn r;
  for (int k = 0; k < 3; ++k) {
    r.o[k] = rays[k * n + i];
    r.d[k] = rays[(3 + k) * n + i];
    r.inv[k] = 1.0f / r.d[k];
  }
  r.tmin = rays[6 * n + i];
  r.tmax = rays[7 * n + i];
  return r;
}

// ---------------------------------------------------------------------------
// Dense density grid (restatement of OpenVDBVolume's sampling, volume.cpp:
// 33-70, 94): a vertex-centred lattice of nx*ny*nz samples spanning the box,
// x fastest; trilinear interpolation; lattice points outside the grid read
// the background value 0.
// ---------------------------------------------------------------------------
struct Grid {
  const float *rho;
  int nx, ny, nz;
  float lo[3], hi[3], scale[3];
  float sigma_s, sigma_a, sigma_t, g;
  float maxd, inv_maxd, rr;

  inline float at(int x, int y, int z) const {
    if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.0f;
    return rho[((int64_t)z * ny + y) * nx + x];
  }
  // Returns the density; fills the corner base and fractions for the adjoint.
  inline float sample(const float *p, int *base, float *f) const {
    float gx = (p[0] - lo[0]) * scale[0];
    float gy = (p[1] - lo[1]) * scale[1];
    float gz = (p[2] - lo[2]) * scale[2];
    float fx0 = std::floor(gx), fy0 = std::floor(gy), fz0 = std::floor(gz);
    int x = (int)fx0, y = (int)fy0, z = (int)fz0;
    float fx = gx - fx0, fy = gy - fy0, fz = gz - fz0;
    base[0] = x; base[1] = y; base[2] = z;
    f[0] = fx; f[1] = fy; f[2] = fz;
    auto lerp = [](float a, float b, float w) { return a + (b - a) * w; };
    float c00 = lerp(at(x, y, z), at(x + 1, y, z), fx);
    float c10 = lerp(at(x, y + 1, z), at(x + 1, y + 1, z), fx);
    float c01 = lerp(at(x, y, z + 1), at(x + 1, y, z + 1), fx);
    float c11 = lerp(at(x, y + 1, z + 1), at(x + 1, y + 1, z + 1), fx);
    float c0 = lerp(c00, c10, fy);
    float c1 = lerp(c01, c11, fy);
    return lerp(c0, c1, fz);
  }
  inline double at64(int x, int y, int z, const double *r64, int64_t pv = -1, double pd = 0.0) const {
    if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.0;
    const int64_t v = ((int64_t)z * ny + y) * nx + x;
    const double r = r64 ? r64[v] : (double)rho[v];
    return v == pv ? r + pd : r;
  }
};

// AABB::intersect_pbrt (common/aabb.h:38-59), t1 starting at the ray's tMax.
inline bool box_intersect_pbrt(const Grid &G, const float *o, const float *d, float tmax,
                               float *t0o, float *t1o) {
  float t0 = 0.0f, t1 = tmax;
  for (int i = 0; i < 3; ++i) {
    float inv = 1.0f / d[i];
    float tn = (G.lo[i] - o[i]) * inv;
    float tf = (G.hi[i] - o[i]) * inv;
    if (tn > tf) std::swap(tn, tf);
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
    if (t0 > t1) return false;
  }
  *t0o = t0;
  *t1o = t1;
  return true;
}

struct TrState {  // state after the last Russian-roulette survival
  float t;
  uint32_t k;
  float c;
};

// OpenVDBVolume::tr (volume.cpp:75-107): ratio tracking with Russian roulette.
float ratio_track(const Grid &G, const float *o, const float *d, float tmax, RayStream &rs,
                  TrState *ck) {
  float t_min, t_max;
  if (ck) *ck = TrState{0.0f, 0u, 1.0f};
  if (!box_intersect_pbrt(G, o, d, tmax, &t_min, &t_max)) return 1.0f;
  float tr = 1.0f, t = std::max(t_min, 0.0f);
  t_max = std::min(t_max, tmax);
  float max_mu = G.sigma_t * G.maxd;
  if (ck) *ck = TrState{t, rs.k, tr};
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = rs.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    float pos[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
    int base[3];
    float f[3];
    float density = G.sample(pos, base, f);
    tr *= 1.0f - std::max(0.0f, density * G.inv_maxd);
    if (tr < G.rr) {
      float q = std::max(0.05f, 1.0f - tr);
      if (rs.next() < q) return 0.0f;
      tr /= 1.0f - q;
      if (ck) *ck = TrState{t, rs.k, tr};
    }
  }
  return tr;
}

// Same estimator in double precision (the FP64 oracle); the random draws are
// the same uniforms.  rho64 (optional) overrides the grid values.
double ratio_track64(const Grid &G, const double *rho64, const float *o, const float *d, float tmax,
                     RayStream &rs, int *n_rr, int64_t pv = -1, double pd = 0.0) {
  double t0 = 0.0, t1 = tmax;
  for (int i = 0; i < 3; ++i) {
    double inv = 1.0 / (double)d[i];
    double tn = ((double)G.lo[i] - o[i]) * inv;
    double tf = ((double)G.hi[i] - o[i]) * inv;
    if (tn > tf) std::swap(tn, tf);
    t0 = std::max(tn, t0);
    t1 = std::min(tf, t1);
    if (t0 > t1) return 1.0;
  }
  double tr = 1.0, t = std::max(t0, 0.0), t_max = std::min(t1, (double)tmax);
  double max_mu = (double)G.sigma_t * (double)G.maxd;
  double inv_maxd = 1.0 / (double)G.maxd;
  double sc[3];
  for (int k = 0; k < 3; ++k) sc[k] = (double)(G.nx * (k == 0) + G.ny * (k == 1) + G.nz * (k == 2) - 1) / ((double)G.hi[k] - G.lo[k]);
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    double u = rs.next();
    t += -std::log(1.0 - u) / max_mu;
    if (t >= t_max) break;
    double g[3];
    for (int k = 0; k < 3; ++k) g[k] = ((double)o[k] + (double)d[k] * t - G.lo[k]) * sc[k];
    int x = (int)std::floor(g[0]), y = (int)std::floor(g[1]), z = (int)std::floor(g[2]);
    double fx = g[0] - x, fy = g[1] - y, fz = g[2] - z;
    double den = 0.0;
    for (int c = 0; c < 8; ++c) {
      int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
      double w = (cx ? fx : 1.0 - fx) * (cy ? fy : 1.0 - fy) * (cz ? fz : 1.0 - fz);
      den += w * G.at64(x + cx, y + cy, z + cz, rho64, pv, pd);
    }
    tr *= 1.0 - std::max(0.0, den * inv_maxd);
    if (tr < (double)G.rr) {
      double q = std::max(0.05, 1.0 - tr);
      if (n_rr) ++*n_rr;
      if (rs.next() < q) return 0.0;
      tr /= 1.0 - q;
    }
  }
  return tr;
}

inline RayStream stream_for(uint64_t seed, int64_t ray) {
  RayStream rs;
  rs.k0 = (uint32_t)seed;
  rs.k1 = (uint32_t)(seed >> 32);
  rs.rlo = (uint32_t)ray;
  rs.rhi = (uint32_t)((uint64_t)ray >> 32);
  return rs;
}

}  // namespace

// ===========================================================================
// C ABI of the oracle (loaded with ctypes by tests/ and bench.py).
// ===========================================================================

ORC_API int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

ORC_API void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

ORC_API void orc_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  U4 r = philox(U4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

ORC_API void orc_logf(const float *x, float *y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = flg_logf(x[i]);
}

ORC_API void orc_stream_uniforms(uint64_t seed, int64_t ray, int32_t n, float *out) {
  RayStream rs = stream_for(seed, ray);
  for (int i = 0; i < n; ++i) out[i] = rs.next();
}

// prestage bounds reduce (radix_bvh.cpp:49-60): union of triangle AABBs.
ORC_API void orc_scene_bound(const float *pos, const int32_t *idx, int64_t n_tri, float *out6) {
  Mesh M{pos, idx, n_tri};
  Bound b;
#pragma omp parallel
  {
    Bound local;
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n_tri; ++i) local.merge(M.bound(i));
#pragma omp critical
    b.merge(local);
  }
  for (int k = 0; k < 3; ++k) {
    out6[k] = b.lo[k];
    out6[3 + k] = b.hi[k];
  }
}

// prestage Morton loop (radix_bvh.cpp:63-73).
ORC_API void orc_morton(const float *pos, const int32_t *idx, int64_t n_tri, const float *bound6,
                        uint32_t *codes) {
  Mesh M{pos, idx, n_tri};
  Bound s;
  for (int k = 0; k < 3; ++k) {
    s.lo[k] = bound6[k];
    s.hi[k] = bound6[3 + k];
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n_tri; ++i) codes[i] = morton_of(M.bound(i), s);
}

// Sort (radix_bvh.cpp:77-81) in the defined stable (code, index) order.
ORC_API void orc_sort(const uint32_t *codes, int64_t n, uint32_t *sorted, int32_t *perm) {
  std::vector<int32_t> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = (int32_t)i;
  std::stable_sort(p.begin(), p.end(), [&](int32_t a, int32_t b) { return codes[a] < codes[b]; });
  for (int64_t i = 0; i < n; ++i) {
    perm[i] = p[i];
    sorted[i] = codes[p[i]];
  }
}

// Karras node pass (radix_bvh.cpp:118-161).  parent: n-1 internal parents
// (root keeps 0, as zero-initialised nodes do), leaf_parent: n.
ORC_API void orc_karras(const uint32_t *sorted, int64_t n64, int32_t *split, uint8_t *leaf,
                        int32_t *range_j, int32_t *parent, int32_t *leaf_parent) {
  int n = (int)n64;
  Karras K{sorted, n};
  if (n >= 1) std::memset(parent, 0, sizeof(int32_t) * (size_t)std::max(n - 1, 0));
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n - 1; ++i) {
    int dd = K.delta(i, i + 1) - K.delta(i, i - 1);
    int d = dd == 0 ? 0 : (dd > 0 ? 1 : -1);
    int delta_min = K.delta(i, i - d);
    int l_max = 2;
    while (K.delta(i, i + l_max * d) > delta_min) l_max <<= 1;
    int l = 0;
    for (int t = l_max / 2; t >= 1; t >>= 1)
      if (K.delta(i, i + (l + t) * d) > delta_min) l += t;
    int j = i + l * d;
    int delta_node = K.delta(i, j);
    int s = 0;
    for (int t = next2pow(l); t >= 1; t >>= 1)
      if (K.delta(i, i + (s + t) * d) > delta_node) s += t;
    int sp = i + s * d + std::min(d, 0);
    uint8_t lf = 0;
    if (std::min(i, j) == sp) lf |= 1;
    if (std::max(i, j) == sp + 1) lf |= 2;
    split[i] = sp;
    leaf[i] = lf;
    range_j[i] = j;
    if (lf & 1) leaf_parent[sp] = i; else parent[sp] = i;
    if (lf & 2) leaf_parent[sp + 1] = i; else parent[sp + 1] = i;
  }
  if (n == 1) leaf_parent[0] = -1;
}

// Bottom-up refit (radix_bvh.cpp:163-199): one climber per leaf; the first
// arrival at a node stops, the second merges the sibling bound and climbs on.
// The reference's relaxed __sync_fetch_and_add is given acquire/release order
// here so the sibling's bound is visible to the second arrival.
ORC_API void orc_refit(const float *pos, const int32_t *idx, int64_t n64, const int32_t *perm,
                       const int32_t *split, const uint8_t *leaf, const int32_t *parent,
                       const int32_t *leaf_parent, float *nb) {
  int n = (int)n64;
  if (n < 2) return;
  Mesh M{pos, idx, n64};
  std::vector<std::atomic<int>> flag(n - 1);
  for (auto &f : flag) f.store(0, std::memory_order_relaxed);
  std::vector<Bound> bound(n - 1);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    int cur = leaf_parent[i];
    int prev = i;
    Bound sub = M.bound(perm[i]);
    while (true) {
      // The first arrival stops; its bound is re-read from the tree (leaf) or
      // from bound[] (internal, published before its flag increment).
      int pf = flag[cur].fetch_add(1, std::memory_order_acq_rel);
      if (pf == 0) break;
      int sp = split[cur];
      uint8_t lf = leaf[cur];
      Bound other;
      if (prev == sp) {  // arrived from the left child (radix_bvh.cpp:177)
        other = (lf & 2) ? M.bound(perm[sp + 1]) : bound[sp + 1];
      } else {
        other = (lf & 1) ? M.bound(perm[sp]) : bound[sp];
      }
      Bound nbd;
      nbd.merge(other);
      nbd.merge(sub);
      bound[cur] = nbd;
      std::atomic_thread_fence(std::memory_order_release);
      sub = nbd;
      if (cur == 0) break;
      prev = cur;
      cur = parent[cur];
    }
  }
  for (int i = 0; i < n - 1; ++i)
    for (int k = 0; k < 3; ++k) {
      nb[6 * i + k] = bound[i].lo[k];
      nb[6 * i + 3 + k] = bound[i].hi[k];
    }
}

// Binned-SAH build: BasicBVHBuilder::recursiveBuilder with
// EBVHPartitionMethod::ESAH at every node (src/experimental/base_bvh.cpp:33-173),
// written out as a tree in the Karras arrays' form:
//   * leaf when n <= 8 or depth >= 26 (:44); otherwise 16 buckets of the
//     centroids (a + b + c) / 3 (base_bvh.hpp:86-87) along axis depth % 3
//     (:53, :113-114), costs 1/8 + (SA_L n_L + SA_R n_R) / SA for the splits
//     after buckets 1..14 (:138-152, SA as base_bvh.hpp:58-63, the 1/8 added
//     in double), the first minimum taken, a split only below the leaf cost n
//     (:154-165);
//   * bucket indices outside [0, 15] are clamped, NaN to 0 (the reference
//     indexes out of bounds there), and the partition is stable (std::partition
//     leaves the order unspecified);
//   * a leaf of k > 1 triangles is stored as a balanced binary subtree (left
//     part k / 2); internal nodes are numbered as Karras numbers them (root 0,
//     a left child by its last position, a right child by its first).
namespace {
struct SahRec {
  Bound b;
  float c[3];
  int32_t orig;
};

inline float sah_area(const Bound &b) {
  float ex = b.hi[0] - b.lo[0], ey = b.hi[1] - b.lo[1], ez = b.hi[2] - b.lo[2];
  return 2 * (ex * ey + ex * ez + ey * ez);
}

inline int sah_bucket(float c, float lo, float hi) {
  float f = std::floor(((c - lo) / (hi - lo)) * 16);
  return f >= 0.0f ? (f < 16.0f ? (int)f : 15) : 0;
}

struct SahOut {
  std::vector<SahRec> r;
  int32_t *split;
  uint8_t *leaf;
  int32_t *range_j, *parent, *leaf_parent;
  float *nb;

  Bound range_bound(int64_t f, int64_t cnt) const {
    Bound b;
    for (int64_t i = f; i < f + cnt; ++i) b.merge(r[i].b);
    return b;
  }

  void node(int64_t f, int64_t cnt, int depth, bool sah, int64_t slot) {
    const Bound B = range_bound(f, cnt);
    int64_t h = -1;
    Bound lb, rb;
    if (sah && !(cnt <= 8 || depth >= 26)) {
      const int dim = depth % 3;
      Bound bb[16], pre[16], suf[16];
      int64_t bn[16] = {0}, pn[16], sn[16];
      for (int64_t i = f; i < f + cnt; ++i) {
        int b = sah_bucket(r[i].c[dim], B.lo[dim], B.hi[dim]);
        bb[b].merge(r[i].b);
        ++bn[b];
      }
      pre[0] = bb[0];
      pn[0] = bn[0];
      for (int i = 1; i < 16; ++i) {
        pre[i] = pre[i - 1];
        pre[i].merge(bb[i]);
        pn[i] = pn[i - 1] + bn[i];
      }
      suf[15] = bb[15];
      sn[15] = bn[15];
      for (int i = 14; i >= 0; --i) {
        suf[i] = suf[i + 1];
        suf[i].merge(bb[i]);
        sn[i] = sn[i + 1] + bn[i];
      }
      float min_cost = FLT_MAX;
      int min_i = 0;
      for (int i = 1; i < 15; ++i) {
        float q = (sah_area(pre[i]) * (float)pn[i] + sah_area(suf[i + 1]) * (float)sn[i + 1]) / sah_area(B);
        float cost = (float)(1.0 / 8 + (double)q);
        if (cost < min_cost) {
          min_cost = cost;
          min_i = i;
        }
      }
      if (min_cost < (float)cnt) {
        std::stable_partition(r.begin() + f, r.begin() + f + cnt, [&](const SahRec &t) {
          return sah_bucket(t.c[dim], B.lo[dim], B.hi[dim]) <= min_i;
        });
        h = pn[min_i];
        lb = pre[min_i];
        rb = suf[min_i + 1];
      }
    }
    const bool child_sah = sah && h >= 0;
    if (h < 0) {
      h = cnt / 2;
      lb = range_bound(f, h);
      rb = range_bound(f + h, cnt - h);
    }
    const int64_t last = f + cnt - 1, m = f + h;
    split[slot] = (int32_t)(m - 1);
    leaf[slot] = (uint8_t)((h == 1 ? 1 : 0) | (cnt - h == 1 ? 2 : 0));
    range_j[slot] = (int32_t)(slot == f ? last : f);
    for (int k = 0; k < 3; ++k) {
      nb[6 * slot + k] = std::min(lb.lo[k], rb.lo[k]);
      nb[6 * slot + 3 + k] = std::max(lb.hi[k], rb.hi[k]);
    }
    if (h == 1) leaf_parent[f] = (int32_t)slot; else parent[m - 1] = (int32_t)slot;
    if (cnt - h == 1) leaf_parent[m] = (int32_t)slot; else parent[m] = (int32_t)slot;
    if (h >= 2) node(f, h, depth + 1, child_sah, m - 1);
    if (cnt - h >= 2) node(m, cnt - h, depth + 1, child_sah, m);
  }
};
}  // namespace

ORC_API void orc_build_sah(const float *pos, const int32_t *idx, int64_t n, int32_t *perm, int32_t *split,
                           uint8_t *leaf, int32_t *range_j, int32_t *parent, int32_t *leaf_parent, float *nb) {
  Mesh M{pos, idx, n};
  SahOut S;
  S.r.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const float *a = M.v(i, 0), *b = M.v(i, 1), *c = M.v(i, 2);
    S.r[i].b = M.bound(i);
    for (int k = 0; k < 3; ++k) S.r[i].c[k] = (a[k] + b[k] + c[k]) / 3;
    S.r[i].orig = (int32_t)i;
  }
  S.split = split;
  S.leaf = leaf;
  S.range_j = range_j;
  S.parent = parent;
  S.leaf_parent = leaf_parent;
  S.nb = nb;
  if (n >= 2) {
    parent[0] = 0;
    S.node(0, n, 0, true, 0);
  } else if (n == 1) {
    leaf_parent[0] = -1;
  }
  for (int64_t i = 0; i < n; ++i) perm[i] = S.r[i].orig;
}

// ---------------------------------------------------------------------------
// Treelet restructuring of the LBVH (Karras & Aila, "Fast Parallel
// Construction of High-Quality Bounding Volume Hierarchies", HPG 2013; no
// counterpart in the reference, whose quality builder is the binned SAH of
// base_bvh.cpp:33-173).  `rounds` bottom-up passes; pass r visits every
// internal node after both its children (post order) and, when its subtree
// holds at least 7 << r triangles, rebuilds the treelet of its 7 largest
// descendants (repeatedly opening the treelet leaf of largest surface area,
// first in list order on ties; the opened node's left child takes its place
// and its right child is appended) into the topology of least SAH cost
//   C(S) = Ci A(S) + min over splits {P, S \ P} of C(P) + C(S \ P),
// P holding the lowest member of S, splits enumerated from S - 1 downwards,
// the first minimum kept; a treelet leaf costs its subtree's SAH cost
// (a triangle Ct A).  A = dx dy + dy dz + dz dx (half the surface area),
// Ci = 1.2, Ct = 1.  The treelet's internal nodes are reused in pre-order.
// Afterwards the leaves are renumbered in depth-first order and the internal
// nodes take Karras' numbering (root 0, a left child its last position, a
// right child its first), so the result has the Karras arrays' form: perm,
// split, leaf flags, range end, parents, node bounds.
// ---------------------------------------------------------------------------
namespace {
constexpr float kTlCi = 1.2f, kTlCt = 1.0f;
constexpr int kTreelet = 7;

inline float tl_area(const Bound &b) {
  const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}
inline Bound tl_union(const Bound &a, const Bound &b) {
  Bound r;
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = std::min(a.lo[k], b.lo[k]);
    r.hi[k] = std::max(a.hi[k], b.hi[k]);
  }
  return r;
}

struct Treelets {
  int64_t n;
  // internal nodes 0 .. n-2 (the LBVH's slots); refs >= 0 internal, < 0 ~leaf
  std::vector<int32_t> left, right, parent, nleaf;  // parent of the root: -1
  std::vector<int32_t> leaf_par;                    // per leaf (old sorted position)
  std::vector<Bound> box;
  std::vector<float> cost;
  std::vector<Bound> lbox;  // per leaf: triangle box
  Bound bx(int32_t r) const { return r >= 0 ? box[r] : lbox[~r]; }
  float cs(int32_t r) const { return r >= 0 ? cost[r] : kTlCt * tl_area(lbox[~r]); }
  int32_t nl(int32_t r) const { return r >= 0 ? nleaf[r] : 1; }
  void set_parent(int32_t r, int32_t p) {
    if (r >= 0) parent[r] = p; else leaf_par[~r] = p;
  }

  void finish(int32_t x) {  // box, cost and count from the children
    const int32_t l = left[x], r = right[x];
    box[x] = tl_union(bx(l), bx(r));
    cost[x] = kTlCi * tl_area(box[x]) + (cs(l) + cs(r));
    nleaf[x] = nl(l) + nl(r);
  }

  void restructure(int32_t R) {
    int32_t L[kTreelet], I[kTreelet - 1];
    int nL = 2, nI = 1;
    L[0] = left[R];
    L[1] = right[R];
    I[0] = R;
    while (nL < kTreelet) {
      int best = -1;
      float ba = -1.0f;
      for (int k = 0; k < nL; ++k)
        if (L[k] >= 0) {
          const float a = tl_area(box[L[k]]);
          if (a > ba) {
            ba = a;
            best = k;
          }
        }
      if (best < 0) return;
      const int32_t x = L[best];
      I[nI++] = x;
      L[best] = left[x];
      L[nL++] = right[x];
    }
    constexpr int kFull = (1 << kTreelet) - 1;
    float c[kFull + 1], a[kFull + 1];
    int part[kFull + 1];
    Bound sb[kFull + 1];
    for (int S = 1; S <= kFull; ++S) {
      const int low = S & -S;
      const int li = __builtin_ctz((unsigned)low);
      sb[S] = S == low ? bx(L[li]) : tl_union(sb[S ^ low], bx(L[li]));
      a[S] = tl_area(sb[S]);
      if (S == low) {
        c[S] = cs(L[li]);
        part[S] = 0;
        continue;
      }
      float best = FLT_MAX;
      int bp = 0;
      for (int P = (S - 1) & S; P > 0; P = (P - 1) & S) {
        if (!(P & low)) continue;
        const float v = c[P] + c[S ^ P];
        if (v < best) {
          best = v;
          bp = P;
        }
      }
      c[S] = kTlCi * a[S] + best;
      part[S] = bp;
    }
    // rebuild: internal nodes of the treelet in pre-order, left before right
    int next = 1;
    struct Item { int S; int32_t node; };
    Item st[kTreelet];
    int sp = 0;
    st[sp++] = Item{kFull, R};
    // pre-order assignment, then box / cost / count bottom-up
    int32_t order[kTreelet - 1];
    int no = 0;
    while (sp) {
      const Item it = st[--sp];
      order[no++] = it.node;
      const int P = part[it.S], Q = it.S ^ P;
      int32_t ch[2];
      const int sub[2] = {P, Q};
      for (int k = 0; k < 2; ++k) {
        if (__builtin_popcount((unsigned)sub[k]) == 1) {
          ch[k] = L[__builtin_ctz((unsigned)sub[k])];
        } else {
          ch[k] = I[next++];
        }
      }
      left[it.node] = ch[0];
      right[it.node] = ch[1];
      set_parent(ch[0], it.node);
      set_parent(ch[1], it.node);
      // right first on the stack so that the left subtree takes the next nodes
      if (__builtin_popcount((unsigned)Q) > 1) st[sp++] = Item{Q, ch[1]};
      if (__builtin_popcount((unsigned)P) > 1) st[sp++] = Item{P, ch[0]};
    }
    for (int k = no - 1; k >= 0; --k) finish(order[k]);
  }

  void pass(int32_t x, int64_t gamma) {  // post order
    if (left[x] >= 0) pass(left[x], gamma);
    if (right[x] >= 0) pass(right[x], gamma);
    finish(x);
    if (nleaf[x] >= gamma) restructure(x);
  }
};
}  // namespace

ORC_API void orc_build_treelet(const float *pos, const int32_t *idx, int64_t n, int32_t rounds, int32_t *perm,
                               int32_t *split, uint8_t *leaf, int32_t *range_j, int32_t *parent,
                               int32_t *leaf_parent, float *nb) {
  Mesh M{pos, idx, n};
  // the LBVH (radix_bvh.cpp:32-200)
  float sb[6];
  orc_scene_bound(pos, idx, n, sb);
  std::vector<uint32_t> codes((size_t)n), sc((size_t)n);
  std::vector<int32_t> p0((size_t)n);
  orc_morton(pos, idx, n, sb, codes.data());
  orc_sort(codes.data(), n, sc.data(), p0.data());
  if (n < 2) {
    for (int64_t i = 0; i < n; ++i) perm[i] = p0[i];
    if (n == 1) leaf_parent[0] = -1;
    return;
  }
  std::vector<int32_t> sp((size_t)n - 1), kp((size_t)n - 1), klp((size_t)n), rj((size_t)n - 1);
  std::vector<uint8_t> lf((size_t)n - 1);
  orc_karras(sc.data(), n, sp.data(), lf.data(), rj.data(), kp.data(), klp.data());
  Treelets T;
  T.n = n;
  T.left.resize(n - 1);
  T.right.resize(n - 1);
  T.parent.resize(n - 1);
  T.nleaf.resize(n - 1);
  T.box.resize(n - 1);
  T.cost.resize(n - 1);
  T.leaf_par.resize(n);
  T.lbox.resize(n);
  for (int64_t i = 0; i < n; ++i) T.lbox[i] = M.bound(p0[i]);
  for (int64_t i = 0; i + 1 < n; ++i) {
    T.left[i] = (lf[i] & 1) ? ~sp[i] : sp[i];
    T.right[i] = (lf[i] & 2) ? ~(sp[i] + 1) : sp[i] + 1;
  }
  for (int64_t i = 0; i + 1 < n; ++i) {
    T.set_parent(T.left[i], (int32_t)i);
    T.set_parent(T.right[i], (int32_t)i);
  }
  T.parent[0] = -1;
  for (int r = 0; r < rounds; ++r) T.pass(0, (int64_t)kTreelet << r);
  if (rounds == 0) {  // boxes, costs and counts of the plain LBVH
    std::vector<int32_t> st{0}, ord;
    while (!st.empty()) {
      const int32_t x = st.back();
      st.pop_back();
      ord.push_back(x);
      if (T.left[x] >= 0) st.push_back(T.left[x]);
      if (T.right[x] >= 0) st.push_back(T.right[x]);
    }
    for (size_t k = ord.size(); k-- > 0;) T.finish(ord[k]);
  }
  // depth-first renumbering and Karras slots
  struct Item { int32_t ref; int64_t first; int32_t pslot; int side; };
  std::vector<Item> st;
  st.push_back(Item{0, 0, -1, -1});
  while (!st.empty()) {
    const Item it = st.back();
    st.pop_back();
    if (it.ref < 0) {
      perm[it.first] = p0[~it.ref];
      leaf_parent[it.first] = it.pslot;
      continue;
    }
    const int32_t x = it.ref;
    const int64_t cnt = T.nleaf[x], last = it.first + cnt - 1;
    const int32_t slot = (int32_t)(it.side < 0 ? 0 : it.side == 0 ? last : it.first);
    if (it.pslot >= 0) parent[slot] = it.pslot; else parent[slot] = 0;
    const int64_t nl = T.nl(T.left[x]);
    split[slot] = (int32_t)(it.first + nl - 1);
    leaf[slot] = (uint8_t)((T.left[x] < 0 ? 1 : 0) | (T.right[x] < 0 ? 2 : 0));
    range_j[slot] = (int32_t)(slot == it.first ? last : it.first);
    for (int k = 0; k < 3; ++k) {
      nb[6 * (int64_t)slot + k] = T.box[x].lo[k];
      nb[6 * (int64_t)slot + 3 + k] = T.box[x].hi[k];
    }
    st.push_back(Item{T.right[x], it.first + nl, slot, 1});
    st.push_back(Item{T.left[x], it.first, slot, 0});
  }
}

// Closest hit over a tree built by the functions above (recursiveIntersect).
// rays: 8 SoA arrays of n floats (ox oy oz dx dy dz tmin tmax).  out: prim
// (-1 = miss), t, u, v.
ORC_API void orc_trace_closest(const float *pos, const int32_t *idx, int64_t n_tri,
                               const int32_t *perm, const int32_t *split, const uint8_t *leaf,
                               const float *nb, const float *rays, int64_t n, int32_t mode,
                               int32_t *prim, float *t, float *u, float *v) {
  Mesh M{pos, idx, n_tri};
  Tree T{n_tri, perm, split, leaf, nb};
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    RayIn r = make_ray(rays, i, n);
    Best b{r.tmax, -1, 0.0f, 0.0f};
    if (n_tri == 1) {
      Hit h;
      if (pluecker(ld3(M.v(0, 0)), ld3(M.v(0, 1)), ld3(M.v(0, 2)), ld3(r.o), ld3(r.d), mode, &h) &&
          !(h.t > b.tfar) && !(mode == MODE_MT && !(h.t < b.tfar)) && !(h.t < r.tmin))
        b = Best{h.t, 0, h.u, h.v};
    } else if (n_tri > 1) {
      recursive_intersect(T, M, 0, r, mode, b);
    }
    if ((mode == MODE_DEV || mode == MODE_MT) && b.prim >= 0) {
      // The GPU reports the selected triangle's t, u, v recomputed in
      // float-float arithmetic and rounded once; same operations here.
      refine_tuv(M.v(b.prim, 0), M.v(b.prim, 1), M.v(b.prim, 2), r.o, r.d, b.tfar, b.u, b.v);
    }
    prim[i] = b.prim;
    t[i] = b.prim >= 0 ? b.tfar : r.tmax;
    u[i] = b.u;
    v[i] = b.v;
  }
}

ORC_API void orc_trace_any(const float *pos, const int32_t *idx, int64_t n_tri, const int32_t *perm,
                           const int32_t *split, const uint8_t *leaf, const float *nb,
                           const float *rays, int64_t n, int32_t mode, uint8_t *occluded) {
  Mesh M{pos, idx, n_tri};
  Tree T{n_tri, perm, split, leaf, nb};
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    RayIn r = make_ray(rays, i, n);
    bool occ = false;
    if (n_tri == 1) {
      Hit h;
      occ = pluecker(ld3(M.v(0, 0)), ld3(M.v(0, 1)), ld3(M.v(0, 2)), ld3(r.o), ld3(r.d), mode, &h) &&
            !(h.t > r.tmax) && !(h.t < r.tmin) && !(mode == MODE_MT && !(h.t < r.tmax));
    } else if (n_tri > 1) {
      occ = recursive_occluded(T, M, 0, r, mode);
    }
    occluded[i] = occ ? 1 : 0;
  }
}

// Single ray/triangle evaluation (tests use it to classify ties): returns 1 on
// a hit and fills t, u, v.
ORC_API int orc_pluecker(const float *a, const float *b, const float *c, const float *o,
                         const float *d, int32_t mode, float *tuv) {
  Hit h;
  if (!pluecker(ld3(a), ld3(b), ld3(c), ld3(o), ld3(d), mode, &h)) return 0;
  tuv[0] = h.t; tuv[1] = h.u; tuv[2] = h.v;
  return 1;
}

// Normal Ng of PlueckerTriangleIntersect (intersector.hpp:88) for ray i and
// original triangle prim[i], as the reference writes it to BVHRayHit::hit_ng
// (radix_bvh.cpp:233); ng[i] = 0 where prim[i] < 0 or the test rejects.
ORC_API void orc_hit_normals(const float *pos, const int32_t *idx, int64_t n_tri, const float *rays,
                             int64_t n, const int32_t *prim, int32_t mode, float *ng) {
  Mesh M{pos, idx, n_tri};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    V3 N{0.0f, 0.0f, 0.0f};
    if (prim[i] >= 0) {
      RayIn r = make_ray(rays, i, n);
      Hit h;
      V3 Nh;
      if (pluecker(ld3(M.v(prim[i], 0)), ld3(M.v(prim[i], 1)), ld3(M.v(prim[i], 2)), ld3(r.o), ld3(r.d), mode,
                   &h, &Nh))
        N = Nh;
    }
    ng[3 * i] = N.x;
    ng[3 * i + 1] = N.y;
    ng[3 * i + 2] = N.z;
  }
}

// FP64 t, u, v of ray i against original triangle prim[i] (the FP64 oracle
// for the GPU's hit values).  ok[i] = 0 where the triangle's plane is parallel.
ORC_API void orc_hit_values64(const float *pos, const int32_t *idx, int64_t n_tri, const float *rays,
                              int64_t n, const int32_t *prim, double *tuv, uint8_t *ok) {
  Mesh M{pos, idx, n_tri};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    ok[i] = 0;
    tuv[3 * i] = tuv[3 * i + 1] = tuv[3 * i + 2] = 0.0;
    if (prim[i] < 0) continue;
    double O[3], D[3];
    for (int k = 0; k < 3; ++k) {
      O[k] = rays[k * n + i];
      D[k] = rays[(3 + k) * n + i];
    }
    double t, u, v;
    if (pluecker64(M.v(prim[i], 0), M.v(prim[i], 1), M.v(prim[i], 2), O, D, &t, &u, &v)) {
      tuv[3 * i] = t; tuv[3 * i + 1] = u; tuv[3 * i + 2] = v;
      ok[i] = 1;
    }
  }
}

// Gradient of (t, u, v) of a fixed hit with respect to the three vertices, in
// FP64: with b = (1-u-v, u, v) and M = [D, -(p1-p0), -(p2-p0)],
// dL/dp_k = b_k * M^{-T} (dL/dt, dL/du, dL/dv).  Accumulates into grad
// (3 floats per vertex, or per soup corner).
ORC_API void orc_hit_adjoint64(const float *pos, const int32_t *idx, int64_t n_tri, int64_t n_vert,
                               const float *rays, int64_t n, const int32_t *prim, const float *g_t,
                               const float *g_u, const float *g_v, double *grad) {
  Mesh M{pos, idx, n_tri};
  (void)n_vert;
  for (int64_t i = 0; i < n; ++i) {
    if (prim[i] < 0) continue;
    double O[3], D[3];
    for (int k = 0; k < 3; ++k) {
      O[k] = rays[k * n + i];
      D[k] = rays[(3 + k) * n + i];
    }
    const float *p[3] = {M.v(prim[i], 0), M.v(prim[i], 1), M.v(prim[i], 2)};
    double t, u, v;
    if (!pluecker64(p[0], p[1], p[2], O, D, &t, &u, &v)) continue;
    double c1[3], c2[3], c3[3];
    for (int k = 0; k < 3; ++k) {
      c1[k] = D[k];
      c2[k] = -((double)p[1][k] - p[0][k]);
      c3[k] = -((double)p[2][k] - p[0][k]);
    }
    auto crs = [](const double *a, const double *b, double *r) {
      r[0] = a[1] * b[2] - a[2] * b[1];
      r[1] = a[2] * b[0] - a[0] * b[2];
      r[2] = a[0] * b[1] - a[1] * b[0];
    };
    double x23[3], x31[3], x12[3];
    crs(c2, c3, x23); crs(c3, c1, x31); crs(c1, c2, x12);
    double det = c1[0] * x23[0] + c1[1] * x23[1] + c1[2] * x23[2];
    if (det == 0.0) continue;
    double w[3];
    for (int k = 0; k < 3; ++k) w[k] = (x23[k] * g_t[i] + x31[k] * g_u[i] + x12[k] * g_v[i]) / det;
    double bc[3] = {1.0 - u - v, u, v};
    for (int c = 0; c < 3; ++c) {
      int64_t vi = idx ? (int64_t)idx[3 * prim[i] + c] : 3 * (int64_t)prim[i] + c;
      for (int k = 0; k < 3; ++k) grad[3 * vi + k] += bc[c] * w[k];
    }
  }
}

// ------------------------------- volumes -----------------------------------

struct OrcMedium {
  float sigma_s, sigma_a, g, rr_threshold, majorant;
};

static Grid make_grid(const float *rho, int nx, int ny, int nz, const float *lo, const float *hi,
                      const OrcMedium *m) {
  Grid G;
  G.rho = rho;
  G.nx = nx; G.ny = ny; G.nz = nz;
  int dims[3] = {nx, ny, nz};
  for (int k = 0; k < 3; ++k) {
    G.lo[k] = lo[k];
    G.hi[k] = hi[k];
    G.scale[k] = (float)(dims[k] - 1) / (hi[k] - lo[k]);
  }
  G.sigma_s = m->sigma_s;
  G.sigma_a = m->sigma_a;
  G.sigma_t = m->sigma_a + m->sigma_s;  // volume.cpp:38
  G.g = m->g;
  G.rr = m->rr_threshold;
  float mx = m->majorant;
  if (!(mx > 0.0f)) {
    mx = 0.0f;
    int64_t nv = (int64_t)nx * ny * nz;
    for (int64_t i = 0; i < nv; ++i) mx = std::max(mx, rho[i]);
  }
  G.maxd = mx;
  G.inv_maxd = (float)(1.0 / (double)mx);  // volume.cpp:55 (double quotient stored as Float)
  return G;
}

ORC_API float orc_grid_majorant(const float *rho, int64_t nv) {
  float mx = 0.0f;
  for (int64_t i = 0; i < nv; ++i) mx = std::max(mx, rho[i]);
  return mx;
}

// Ratio-tracking transmittance (fp32, same arithmetic as the GPU).  ck (may
// be null): 3 arrays of n (t, k as float bits, c) = state after the last
// Russian-roulette survival.
ORC_API void orc_volume_tr(const float *rho, int nx, int ny, int nz, const float *lo, const float *hi,
                           const OrcMedium *m, const float *rays, int64_t n, uint64_t seed,
                           float *T, float *ck_t, uint32_t *ck_k, float *ck_c) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    float tmax = rays[7 * n + i];
    RayStream rs = stream_for(seed, i);
    TrState ck;
    T[i] = ratio_track(G, o, d, tmax, rs, &ck);
    if (ck_t) { ck_t[i] = ck.t; ck_k[i] = ck.k; ck_c[i] = ck.c; }
  }
}

// FP64 ratio tracking; rho64 (nullable) replaces the grid values so that tests
// can take central finite differences.  n_rr (nullable) counts roulette events
// per ray (used to exclude rays whose control flow flips between +h and -h).
ORC_API void orc_volume_tr64(const float *rho, const double *rho64, int nx, int ny, int nz,
                             const float *lo, const float *hi, const OrcMedium *m, const float *rays,
                             int64_t n, uint64_t seed, double *T, int32_t *n_rr) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    RayStream rs = stream_for(seed, i);
    int nr = 0;
    T[i] = ratio_track64(G, rho64, o, d, rays[7 * n + i], rs, &nr);
    if (n_rr) n_rr[i] = nr;
  }
}

// FP64 ratio tracking of a subset of rays: ray j of the arrays is ray
// ray_ids[j] of the full set (its Philox stream), and grid value `vox` (-1:
// none) is raised by `delta` in double precision.  For central finite
// differences on large grids without copying them.
ORC_API void orc_volume_tr64_sub(const float *rho, int nx, int ny, int nz, const float *lo, const float *hi,
                                 const OrcMedium *m, const float *rays, int64_t n, const int64_t *ray_ids,
                                 uint64_t seed, int64_t vox, double delta, double *T, int32_t *n_rr) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    RayStream rs = stream_for(seed, ray_ids[i]);
    int nr = 0;
    T[i] = ratio_track64(G, nullptr, o, d, rays[7 * n + i], rs, &nr, vox, delta);
    if (n_rr) n_rr[i] = nr;
  }
}

// Adjoint of ratio tracking with respect to the grid, fp32 forward arithmetic
// (identical to the GPU's) and FP64 accumulation:
//   T = c * prod_{i in last segment} (1 - d_i / rho_max),
//   dT/drho_v = sum_i -T / (1 - d_i/rho_max) * w_iv / rho_max,
// with the majorant held constant (steps do not move with the grid) and the
// roulette rescale 1/(1-q) = 1/T contributing nothing (T is reset to ~1).
namespace {
// One ray's adjoint: replays its stream from the last roulette checkpoint and
// calls emit(flat voxel index, dL/drho contribution) for every lattice point
// of every step after it.
template <typename Emit>
void tr_adjoint_ray(const Grid &G, const float *o, const float *d, float tmax, uint64_t seed, int64_t ray,
                    float dL, Emit &&emit) {
  RayStream rs = stream_for(seed, ray);
  TrState ck;
  float Tf = ratio_track(G, o, d, tmax, rs, &ck);
  if (Tf == 0.0f || dL == 0.0f) return;
  float t_min, t_max;
  if (!box_intersect_pbrt(G, o, d, tmax, &t_min, &t_max)) return;
  t_max = std::min(t_max, tmax);
  float max_mu = G.sigma_t * G.maxd;
  RayStream r2 = stream_for(seed, ray);
  r2.k = ck.k;
  float t = ck.t;
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = r2.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    float pos[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
    int b[3];
    float f[3];
    float den = G.sample(pos, b, f);
    float x = den * G.inv_maxd;
    if (!(x > 0.0f)) continue;
    double fac = 1.0 - (double)x;
    double coef = -(double)dL * (double)Tf * (double)G.inv_maxd / fac;
    for (int c = 0; c < 8; ++c) {
      int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
      int X = b[0] + cx, Y = b[1] + cy, Z = b[2] + cz;
      if (X < 0 || Y < 0 || Z < 0 || X >= G.nx || Y >= G.ny || Z >= G.nz) continue;
      double w = (cx ? (double)f[0] : 1.0 - f[0]) * (cy ? (double)f[1] : 1.0 - f[1]) *
                 (cz ? (double)f[2] : 1.0 - f[2]);
      emit(((int64_t)Z * G.ny + Y) * G.nx + X, coef * w);
    }
  }
}
}  // namespace

ORC_API void orc_volume_tr_adjoint(const float *rho, int nx, int ny, int nz, const float *lo,
                                   const float *hi, const OrcMedium *m, const float *rays, int64_t n,
                                   uint64_t seed, const float *dLdT, double *grad) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    tr_adjoint_ray(G, o, d, rays[7 * n + i], seed, i, dLdT[i], [&](int64_t v, double g) { grad[v] += g; });
  }
}

// Per-ray contributions to dT/drho at one voxel (flat index vox), dL/dT = 1,
// for a subset of rays: ray j of the arrays is ray ray_ids[j] of the full set
// (its Philox stream).  out: n doubles.
ORC_API void orc_volume_tr_adjoint_vox(const float *rho, int nx, int ny, int nz, const float *lo,
                                       const float *hi, const OrcMedium *m, const float *rays, int64_t n,
                                       const int64_t *ray_ids, uint64_t seed, int64_t vox, double *out) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    double acc = 0.0;
    tr_adjoint_ray(G, o, d, rays[7 * n + i], seed, ray_ids[i], 1.0f, [&](int64_t v, double g) {
      if (v == vox) acc += g;
    });
    out[i] = acc;
  }
}

// Delta tracking (OpenVDBVolume::sample, volume.cpp:109-148).  Outputs
// success (0/1), collision position and the returned weight sigma_s/sigma_t
// (1 when no collision).
ORC_API void orc_volume_sample(const float *rho, int nx, int ny, int nz, const float *lo,
                               const float *hi, const OrcMedium *m, const float *rays, int64_t n,
                               uint64_t seed, uint8_t *success, float *p, float *weight) {
  Grid G = make_grid(rho, nx, ny, nz, lo, hi, m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; ++i) {
    float o[3] = {rays[i], rays[n + i], rays[2 * n + i]};
    float d[3] = {rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]};
    float tmax = rays[7 * n + i];
    RayStream rs = stream_for(seed, i);
    success[i] = 0;
    weight[i] = 1.0f;
    p[3 * i] = p[3 * i + 1] = p[3 * i + 2] = 0.0f;
    float t_min, t_max;
    if (!box_intersect_pbrt(G, o, d, tmax, &t_min, &t_max)) continue;
    float t = std::max(t_min, 0.0f);
    float max_mu = G.sigma_t * G.maxd;
    t_max = std::min(t_max, tmax);
    for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
      float u = rs.next();
      t += -flg_logf(1.0f - u) / max_mu;
      if (t >= t_max) break;
      float pos[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
      int b[3];
      float f[3];
      float density = G.sample(pos, b, f);
      float p_s = G.sigma_s * density / max_mu;
      float p_a = G.sigma_a * density / max_mu;
      float p_n = 1.0f - p_s - p_a;
      if (rs.next() > p_n) {
        success[i] = 1;
        p[3 * i] = pos[0]; p[3 * i + 1] = pos[1]; p[3 * i + 2] = pos[2];
        weight[i] = G.sigma_s / G.sigma_t;
        break;
      }
    }
  }
}

// Henyey-Greenstein phase function value (math_utils.h:103-107) — used by the
// delta-tracking caller; exposed for tests.
ORC_API float orc_hg_p(const float *wi, const float *wo, float g) {
  float cos_theta = wi[0] * wo[0] + wi[1] * wo[1] + wi[2] * wo[2];
  float denom = 1.0f + g * g + 2.0f * g * cos_theta;
  return (1.0f - g * g) / (denom * std::sqrt(denom)) * 0.07957747154594766788f;
}

// ------------------------ reference-performance mode ------------------------
// Build timed the way the reference runs it: parallel bounds reduce, parallel
// Morton, parallel sort of 32-byte records (the RadixTriangle layout,
// radix_bvh.hpp:35-37), parallel Karras and atomic refit.  Returns the node
// count; outputs are the same arrays as the step-by-step functions.
namespace {
struct Rec32 {
  const int32_t *v;
  const void *mesh;
  uint32_t code, parent;
};
}  // namespace

ORC_API int64_t orc_build(const float *pos, const int32_t *idx, int64_t n_tri, uint32_t *sorted,
                          int32_t *perm, int32_t *split, uint8_t *leaf, int32_t *range_j,
                          int32_t *parent, int32_t *leaf_parent, float *nb) {
  if (n_tri <= 0) return 0;
  float b6[6];
  orc_scene_bound(pos, idx, n_tri, b6);
  std::vector<uint32_t> codes(n_tri);
  orc_morton(pos, idx, n_tri, b6, codes.data());
  std::vector<Rec32> rec(n_tri);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n_tri; ++i) rec[i] = Rec32{idx ? idx + 3 * i : nullptr, (const void *)(intptr_t)i, codes[i], 0};
  __gnu_parallel::stable_sort(rec.begin(), rec.end(),
                              [](const Rec32 &a, const Rec32 &b) { return a.code < b.code; });
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n_tri; ++i) {
    sorted[i] = rec[i].code;
    perm[i] = (int32_t)(intptr_t)rec[i].mesh;
  }
  orc_karras(sorted, n_tri, split, leaf, range_j, parent, leaf_parent);
  orc_refit(pos, idx, n_tri, perm, split, leaf, parent, leaf_parent, nb);
  return n_tri - 1;
}

// ------------------------------ path tracing --------------------------------
// PathIntegrator::Li (integrator.cpp:252-326) with UniformSampleOneLight /
// EstimateDirect (:69-120), the Halton sampler (sampler.h:143-252) and
// eval_pixel's sample order (integrator.cpp:136-159), over the oracle's
// closest-hit (DEV arithmetic, refined hit values) and any-hit traversal.
// Emitters: triangles [light_first, light_first + light_count); a light
// triangle is chosen uniformly and sampled with UniformSampleTriangle
// (math_utils.h:90-93) since the reference's Triangle::sample is TODO.
namespace {

const int kPrimes[64] = {2,   3,   5,   7,   11,  13,  17,  19,  23,  29,  31,  37,  41,  43,  47,  53,
                         59,  61,  67,  71,  73,  79,  83,  89,  97,  101, 103, 107, 109, 113, 127, 131,
                         137, 139, 149, 151, 157, 163, 167, 173, 179, 181, 191, 193, 197, 199, 211, 223,
                         227, 229, 233, 239, 241, 251, 257, 263, 269, 271, 277, 281, 283, 293, 307, 311};

float radical_inverse(int base, uint64_t a) {  // RadicalInverse_ (sampler.h)
  const float inv_base = 1.0f / (float)base;
  uint64_t rev = 0;
  float inv_n = 1.0f;
  while (a) {
    uint64_t next = a / (uint64_t)base;
    uint64_t digit = a - next * (uint64_t)base;
    rev = rev * (uint64_t)base + digit;
    inv_n *= inv_base;
    a = next;
  }
  return (float)rev * inv_n;
}

uint64_t inverse_radical_inverse(int base, uint64_t inverse, int n_digits) {
  uint64_t index = 0;
  for (int i = 0; i < n_digits; ++i) {
    uint64_t digit = inverse % (uint64_t)base;
    inverse /= (uint64_t)base;
    index = index * (uint64_t)base + digit;
  }
  return index;
}

struct HaltonH {
  uint64_t scale[2], stride, inv[2];
  int exp[2];
  HaltonH(int w, int h) {  // HaltonSampler(SPP, {resX, resY}), M_MAX_RESOLUTION 128
    const int res[2] = {w, h};
    for (int i = 0; i < 2; ++i) {
      const int base = i == 0 ? 2 : 3;
      uint64_t sc = 1;
      int e = 0;
      while (sc < (uint64_t)std::min(res[i], 128)) {
        sc *= base;
        ++e;
      }
      scale[i] = sc;
      exp[i] = e;
    }
    stride = scale[0] * scale[1];
    inv[0] = mulinv((int64_t)scale[1], (int64_t)scale[0]);
    inv[1] = mulinv((int64_t)scale[0], (int64_t)scale[1]);
  }
  static void exgcd(int64_t a, int64_t b, int64_t &x, int64_t &y) {  // ExGCD (sampler.h)
    if (b == 0) {
      x = 1;
      y = 0;
      return;
    }
    exgcd(b, a % b, y, x);
    y -= a / b * x;
  }
  static uint64_t mulinv(int64_t a, int64_t b) {
    int64_t x, y;
    exgcd(a, b, x, y);
    int64_t m = x % b;
    return (uint64_t)(m < 0 ? m + b : m);
  }
  uint64_t offset(int x, int y) const {  // getIndexForSample
    if (stride <= 1) return 0;
    uint64_t off = inverse_radical_inverse(2, (uint64_t)(x % 128), exp[0]) * (stride / scale[0]) * inv[0];
    off += inverse_radical_inverse(3, (uint64_t)(y % 128), exp[1]) * (stride / scale[1]) * inv[1];
    return off % stride;
  }
  float sample(uint64_t index, int dim) const {  // sampleDimension + get1D clamp
    float v;
    if (dim == 0) v = radical_inverse(2, index / scale[0]);
    else if (dim == 1) v = radical_inverse(3, index / scale[1]);
    else v = radical_inverse(kPrimes[dim < 64 ? dim : 63], index);
    return std::min(v, 0.99999994f);
  }
};

inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 scale3(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 norm3(V3 a) {
  float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x / l, a.y / l, a.z / l};
}

float offset_axis(float p, float off) {  // OffsetRayOrigin (common/ray.h:64-93)
  int oi = (int)(off * 256.0f);
  int pb;
  std::memcpy(&pb, &p, 4);
  pb += p < 0.0f ? -oi : oi;
  float pi;
  std::memcpy(&pi, &pb, 4);
  return std::fabs(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * off : pi;
}
V3 offset_origin(V3 p, V3 n, V3 d) {
  V3 off = dot(n, d) <= 0.0f ? v3(-n.x, -n.y, -n.z) : n;
  return {offset_axis(p.x, off.x), offset_axis(p.y, off.y), offset_axis(p.z, off.z)};
}

}  // namespace

namespace {

// Delta tracking over [0, tmax] (volume.cpp:109-148); true on a real
// collision, position in p.
bool delta_track(const Grid &G, const float *o, const float *d, float tmax, RayStream &rs, float *p) {
  float t_min, t_max;
  if (!box_intersect_pbrt(G, o, d, tmax, &t_min, &t_max)) return false;
  float t = std::max(t_min, 0.0f);
  const float max_mu = G.sigma_t * G.maxd;
  t_max = std::min(t_max, tmax);
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = rs.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    float pos[3] = {o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t};
    int b[3];
    float f[3];
    float density = G.sample(pos, b, f);
    float p_s = G.sigma_s * density / max_mu;
    float p_a = G.sigma_a * density / max_mu;
    float p_n = 1.0f - p_s - p_a;
    if (rs.next() > p_n) {
      p[0] = pos[0]; p[1] = pos[1]; p[2] = pos[2];
      return true;
    }
  }
  return false;
}

float hg_p(V3 wi, V3 wo, float g) {  // HGP (math_utils.h:103-107)
  const float cos_theta = wi.x * wo.x + wi.y * wo.y + wi.z * wo.z;
  const float denom = 1.0f + g * g + 2.0f * g * cos_theta;
  return (1.0f - g * g) / (denom * std::sqrt(denom)) * 0.07957747154594766788f;
}

V3 hg_sample(V3 wo, float u, float v, float g) {  // HGSampleP (math_utils.h:111-128)
  float cos_theta;
  if (std::fabs(g) < 1e-3f) {
    cos_theta = 1.0f - 2.0f * u;
  } else {
    const float tmp = (1.0f - g * g) / (1.0f + g - 2.0f * g * u);
    cos_theta = -(1.0f + g * g - tmp * tmp) / (2.0f * g);
  }
  const float phi = 2.0f * 3.14159265358979f * v;
  const float sin_theta = std::sqrt(std::max(0.0f, 1.0f - cos_theta * cos_theta));
  V3 v1;
  if (std::fabs(wo.x) > std::fabs(wo.y)) {  // CoordinateSystem (math_utils.h:57-66)
    const float l = std::sqrt(wo.x * wo.x + wo.z * wo.z);
    v1 = v3(-wo.z / l, 0.0f, wo.x / l);
  } else {
    const float l = std::sqrt(wo.y * wo.y + wo.z * wo.z);
    v1 = v3(0.0f, wo.z / l, -wo.y / l);
  }
  const V3 v2 = cross(wo, v1);
  const float a = sin_theta * std::cos(phi), b = sin_theta * std::sin(phi);
  return v3(a * v1.x + b * v2.x + cos_theta * wo.x, a * v1.y + b * v2.y + cos_theta * wo.y,
            a * v1.z + b * v2.z + cos_theta * wo.z);
}

inline uint64_t path_stream_id(int64_t pix, int s, int depth, int purpose) {
  return (uint64_t)pix | ((uint64_t)s << 26) | ((uint64_t)depth << 42) | ((uint64_t)purpose << 50);
}

}  // namespace

// PathIntegrator::Li (integrator.cpp:252-326) per pixel in eval_pixel's sample
// order (:136-159); with a grid (rho != NULL), VolPathIntegrator::Li
// (:407-510) with the medium filling the grid's box: delta tracking over the
// segment up to each surface hit, Henyey-Greenstein scattering, shadow rays
// weighted by ratio tracking (VolEstimateTr, :40-66).
//
// With a medium bounded by a mesh (mm_tri = {first, count} of the boundary
// triangles, mm_coef = sigma_s[3], sigma_a[3], g, density: HVolume attached
// to a mesh, scene.cpp:224-228): boundary hits pass straight through without
// counting as a bounce and set the medium by Entering (interaction.cpp:
// 16-38; a ray leaving a material surface is outside); inside, HVolume::
// sample (volume.cpp:164-190) over the segment; shadow rays follow
// VolEstimateTr (integrator.cpp:40-66) with closest hits through the
// boundaries.  Draws from Philox streams keyed by the path's segment count.
ORC_API void orc_pathtrace(const float *pos, const int32_t *idx, int64_t n_tri, const int32_t *perm,
                           const int32_t *split, const uint8_t *leaf, const float *nb, int32_t light_first,
                           int32_t light_count, const float *le, const float *albedo, const float *eye,
                           const float *target, const float *up, float fov_deg, int32_t width, int32_t height,
                           int32_t spp, int32_t max_depth, int32_t pixel_stride, float *radiance,
                           int64_t *rays, const float *rho, int32_t gnx, int32_t gny, int32_t gnz,
                           const float *glo, const float *ghi, const OrcMedium *gm, uint64_t seed,
                           const int32_t *mm_tri, const float *mm_coef) {
  Mesh M{pos, idx, n_tri};
  Tree T{n_tri, perm, split, leaf, nb};
  HaltonH H(width, height);
  const bool medium = rho != nullptr;
  const bool mm = mm_tri != nullptr;
  const int32_t if_first = mm ? mm_tri[0] : -1, if_count = mm ? mm_tri[1] : 0;
  float m_s[3] = {0, 0, 0}, m_t[3] = {1, 1, 1}, m_g = 0.0f, m_dens = 1.0f;
  if (mm) {
    for (int k = 0; k < 3; ++k) {
      m_s[k] = mm_coef[k];
      m_t[k] = mm_coef[k] + mm_coef[3 + k];
    }
    m_g = mm_coef[6];
    m_dens = mm_coef[7];
  }
  auto iface = [&](int64_t tri) { return tri >= if_first && tri < if_first + if_count; };
  auto closest = [&](V3 o, V3 d, float tmax, Best &b) {  // with the GPU's reported t, u, v
    RayIn r;
    r.o[0] = o.x; r.o[1] = o.y; r.o[2] = o.z;
    r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
    for (int k = 0; k < 3; ++k) r.inv[k] = 1.0f / r.d[k];
    r.tmin = 1e-30f;
    r.tmax = tmax;
    b = Best{tmax, -1, 0.0f, 0.0f};
    recursive_intersect(T, M, 0, r, MODE_DEV, b);
    if (b.prim >= 0) refine_tuv(M.v(b.prim, 0), M.v(b.prim, 1), M.v(b.prim, 2), r.o, r.d, b.tfar, b.u, b.v);
  };
  const float g_phase = mm ? m_g : 0.0f;
  Grid G{};
  if (medium) G = make_grid(rho, gnx, gny, gnz, glo, ghi, gm);
  float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
  auto nrm = [](float *v) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
  };
  nrm(f);
  float r[3] = {up[1] * f[2] - up[2] * f[1], up[2] * f[0] - up[0] * f[2], up[0] * f[1] - up[1] * f[0]};
  nrm(r);
  float u3[3] = {f[1] * r[2] - f[2] * r[1], f[2] * r[0] - f[0] * r[2], f[0] * r[1] - f[1] * r[0]};
  nrm(u3);
  const float fov_ratio = std::tan(3.14159265358979f * fov_deg / 360.0f);
  const float aspect = (float)width / (float)height;
  const float inv_spp = 1.0f / (float)spp;
  const float inv_pi = 1.0f / 3.14159265358979f;
  int64_t n_closest = 0, n_shadow = 0;
  const int64_t npix = (int64_t)width * height;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : n_closest, n_shadow)
  for (int64_t pix = 0; pix < npix; pix += pixel_stride) {
    const int x = (int)(pix % width), y = (int)(pix / width);
    const uint64_t off = H.offset(x, y);
    double acc[3] = {0.0, 0.0, 0.0};
    int cnt_end0 = 0;
    for (int s = 0; s < spp; ++s) {
      float px, py;
      int cnt;
      uint64_t index = off + (uint64_t)(s > 0 ? s - 1 : 0) * H.stride;
      if (s == 0) {
        px = (float)x + 0.5f;
        py = (float)y + 0.5f;
        cnt = 0;
      } else {
        cnt = s == 1 ? cnt_end0 : 0;
        px = (float)x + H.sample(index, cnt);
        py = (float)y + H.sample(index, cnt + 1);
        cnt += 2;
      }
      // Camera::generateRay (camera.h:22-31)
      const float yo = fov_ratio * ((py / (float)height) * 2.0f - 1.0f);
      const float xo = fov_ratio * aspect * ((px / (float)width) * 2.0f - 1.0f);
      V3 O = v3(eye[0], eye[1], eye[2]);
      V3 D = norm3(v3(f[0] + xo * r[0] + yo * u3[0], f[1] + xo * r[1] + yo * u3[1], f[2] + xo * r[2] + yo * u3[2]));
      float beta[3] = {1.0f, 1.0f, 1.0f};
      int bnc = 0, seg = 0;
      bool inmed = false;
      for (int depth = 0;; ++depth) {
        if (mm && depth >= 255) break;
        RayIn ray;
        ray.o[0] = O.x; ray.o[1] = O.y; ray.o[2] = O.z;
        ray.d[0] = D.x; ray.d[1] = D.y; ray.d[2] = D.z;
        for (int k = 0; k < 3; ++k) ray.inv[k] = 1.0f / ray.d[k];
        ray.tmin = 1e-30f;
        ray.tmax = 3.402823466e+38f;
        Best b{ray.tmax, -1, 0.0f, 0.0f};
        recursive_intersect(T, M, 0, ray, MODE_DEV, b);
        ++n_closest;
        if (b.prim >= 0) refine_tuv(M.v(b.prim, 0), M.v(b.prim, 1), M.v(b.prim, 2), ray.o, ray.d, b.tfar, b.u, b.v);
        if (b.prim < 0) break;
        const V3 a = ld3(M.v(b.prim, 0)), bb = ld3(M.v(b.prim, 1)), c = ld3(M.v(b.prim, 2));
        const float w = 1.0f - b.u - b.v;
        const V3 p = v3(w * a.x + b.u * bb.x + b.v * c.x, w * a.y + b.u * bb.y + b.v * c.y,
                        w * a.z + b.u * bb.z + b.v * c.z);
        const V3 ng = norm3(cross(sub(bb, a), sub(c, a)));
        const bool is_light = b.prim >= light_first && b.prim < light_first + light_count;
        const int bounce = mm ? bnc : depth;
        if (bounce == 0 && is_light && dot(ng, v3(-D.x, -D.y, -D.z)) > 0.0f)
          for (int k = 0; k < 3; ++k) acc[k] += (double)(beta[k] * le[k] * inv_spp);
        if (bounce >= max_depth) break;
        const V3 wo = v3(-D.x, -D.y, -D.z);
        bool scatter = false;
        V3 ps = p;
        if (mm && inmed) {
          // HVolume::sample with ray.m_tMax = the hit distance
          RayStream rs = stream_for(seed, (int64_t)path_stream_id(pix, s, seg, 0));
          const int ch = std::min((int)((double)rs.next() * 3.0), 2);
          const float t = -flg_logf(1.0f - rs.next()) / (m_dens * m_t[ch]);
          const float tm = std::min(t, b.tfar);
          float tr[3];
          for (int k = 0; k < 3; ++k) tr[k] = std::exp(-tm * m_dens * m_t[k]);
          if (t < b.tfar) {
            const float pdf = (m_t[0] * tr[0] + m_t[1] * tr[1] + m_t[2] * tr[2]) * 1.0f / 3.0f;
            for (int k = 0; k < 3; ++k) beta[k] = beta[k] * (m_s[k] * tr[k] / pdf);
            ps = v3(ray.o[0] + ray.d[0] * t, ray.o[1] + ray.d[1] * t, ray.o[2] + ray.d[2] * t);
            scatter = true;
          } else {
            const float pdf = (tr[0] + tr[1] + tr[2]) * 1.0f / 3.0f;
            for (int k = 0; k < 3; ++k) beta[k] = beta[k] * (tr[k] / pdf);
          }
        }
        if (mm && !scatter && iface(b.prim)) {  // a material-less boundary: straight on
          O = offset_origin(p, ng, D);
          inmed = dot(D, ng) < 0.0f;
          ++seg;
          continue;
        }
        const bool smed = mm && scatter && inmed;
        ++bnc;
        if (medium) {
          RayStream rs = stream_for(seed, (int64_t)path_stream_id(pix, s, depth, 0));
          float q[3];
          scatter = delta_track(G, ray.o, ray.d, b.tfar, rs, q);
          if (scatter) {
            ps = v3(q[0], q[1], q[2]);
            const float wgt = G.sigma_s / G.sigma_t;
            for (int k = 0; k < 3; ++k) beta[k] = beta[k] * wgt;
          }
        }
        const float ul = H.sample(index, cnt), ua = H.sample(index, cnt + 1), ub = H.sample(index, cnt + 2);
        cnt += 3;
        const int li = std::min((int)(ul * (float)light_count), light_count - 1);
        const float light_pdf = 1.0f / (float)light_count;
        const int64_t lt = light_first + li;
        const V3 la = ld3(M.v(lt, 0)), lb = ld3(M.v(lt, 1)), lc = ld3(M.v(lt, 2));
        const float su0 = std::sqrt(ua);
        const float b0 = 1.0f - su0, b1 = ub * su0, b2 = 1.0f - b0 - b1;
        const V3 lp = v3(b0 * la.x + b1 * lb.x + b2 * lc.x, b0 * la.y + b1 * lb.y + b2 * lc.y,
                         b0 * la.z + b1 * lb.z + b2 * lc.z);
        const V3 lcr = cross(sub(lb, la), sub(lc, la));
        const float area = 0.5f * std::sqrt(dot(lcr, lcr));
        const V3 ln = scale3(lcr, 1.0f / (2.0f * area));
        const V3 toL = sub(lp, ps);
        const float dist = std::sqrt(dot(toL, toL));
        const V3 wi = scale3(toL, 1.0f / dist);
        const float cos_l = -dot(ln, wi);
        if (cos_l > 0.0f && dist > 0.0f) {
          const float pdf = dist * dist / (cos_l * area);
          float fv[3];
          if (scatter) {
            const float ph = hg_p(wi, wo, mm ? g_phase : G.g);
            fv[0] = fv[1] = fv[2] = ph;
          } else {
            const float cos_s = std::fabs(dot(wi, ng));
            for (int k = 0; k < 3; ++k) fv[k] = albedo[k] * inv_pi * cos_s;
          }
          const float kk = inv_spp / (pdf * light_pdf);
          float ct[3];
          for (int k = 0; k < 3; ++k) ct[k] = beta[k] * fv[k] * le[k] * kk;
          if ((ct[0] > 0.0f || ct[1] > 0.0f || ct[2] > 0.0f) && mm) {
            // VolEstimateTr: closest hits through the boundaries
            V3 so = scatter ? ps : offset_origin(p, ng, wi);
            float rem = dist - 1e-4f;
            bool sm = smed;
            for (int step = 0; step < 64; ++step) {
              Best hb;
              closest(so, wi, rem, hb);
              ++n_shadow;
              if (hb.prim < 0) {
                for (int q = 0; q < 3; ++q) acc[q] += (double)ct[q];
                break;
              }
              if (!iface(hb.prim)) break;  // a material surface blocks
              const float t = hb.tfar;
              if (sm)
                for (int q = 0; q < 3; ++q) ct[q] = ct[q] * std::exp(-t * m_dens * m_t[q]);
              const float rem2 = rem - t;
              if (rem2 < 0.0f) {
                for (int q = 0; q < 3; ++q) acc[q] += (double)ct[q];
                break;
              }
              const V3 ia = ld3(M.v(hb.prim, 0)), ib = ld3(M.v(hb.prim, 1)), ic = ld3(M.v(hb.prim, 2));
              const V3 ing = norm3(cross(sub(ib, ia), sub(ic, ia)));
              const V3 ph = v3(so.x + wi.x * t, so.y + wi.y * t, so.z + wi.z * t);
              so = offset_origin(ph, ing, wi);
              sm = dot(wi, ing) < 0.0f;
              rem = rem2;
            }
          } else if (ct[0] > 0.0f || ct[1] > 0.0f || ct[2] > 0.0f) {
            const V3 so = scatter ? ps : offset_origin(p, ng, wi);
            RayIn sr;
            sr.o[0] = so.x; sr.o[1] = so.y; sr.o[2] = so.z;
            sr.d[0] = wi.x; sr.d[1] = wi.y; sr.d[2] = wi.z;
            for (int q = 0; q < 3; ++q) sr.inv[q] = 1.0f / sr.d[q];
            sr.tmin = 1e-30f;
            sr.tmax = dist - 1e-4f;
            ++n_shadow;
            if (!recursive_occluded(T, M, 0, sr, MODE_DEV)) {
              float tr = 1.0f;
              if (medium) {
                RayStream rs = stream_for(seed, (int64_t)path_stream_id(pix, s, depth, 1));
                tr = ratio_track(G, sr.o, sr.d, sr.tmax, rs, nullptr);
              }
              if (tr != 0.0f)
                for (int q = 0; q < 3; ++q) acc[q] += (double)(ct[q] * tr);
            }
          }
        }
        const float u1 = H.sample(index, cnt), u2 = H.sample(index, cnt + 1);
        cnt += 2;
        ++seg;
        if (scatter) {
          D = hg_sample(wo, u1, u2, mm ? g_phase : G.g);
          O = ps;
          continue;  // a medium vertex keeps the medium
        }
        inmed = false;  // a ray leaving a material surface is outside
        V3 bn = std::fabs(ng.x) > std::fabs(ng.z) ? v3(-ng.y, ng.x, 0.0f) : v3(0.0f, -ng.z, ng.y);
        bn = norm3(bn);
        const V3 tg = cross(bn, ng);
        const float woz = dot(wo, ng);
        const float ux = u1 * 2.0f - 1.0f, uy = u2 * 2.0f - 1.0f;
        float dx = 0.0f, dy = 0.0f;
        if (ux != 0.0f || uy != 0.0f) {
          float rr, th;
          if (std::fabs(ux) > std::fabs(uy)) {
            rr = ux;
            th = 0.78539816f * (uy / ux);
          } else {
            rr = uy;
            th = 1.57079633f - 0.78539816f * (ux / uy);
          }
          dx = std::cos(th) * rr;
          dy = std::sin(th) * rr;
        }
        const float dz = std::sqrt(std::max(0.0f, 1.0f - dx * dx - dy * dy));
        const float pdf_b = woz * dz > 0.0f ? std::fabs(dz) * (1.0f / 3.14159265358979f) : 0.0f;
        if (!(pdf_b > 0.0f)) break;
        V3 nd = v3(tg.x * dx + bn.x * dy + ng.x * dz, tg.y * dx + bn.y * dy + ng.y * dz,
                   tg.z * dx + bn.z * dy + ng.z * dz);
        const float fcos = (1.0f / 3.14159265358979f) * std::fabs(dot(nd, ng)) / pdf_b;
        for (int q = 0; q < 3; ++q) beta[q] = beta[q] * albedo[q] * fcos;
        nd = norm3(nd);
        O = offset_origin(p, ng, nd);
        D = nd;
      }
      if (s == 0) cnt_end0 = cnt;
    }
    for (int k = 0; k < 3; ++k) radiance[3 * pix + k] = (float)acc[k];
  }
  rays[0] = n_closest;
  rays[1] = n_shadow;
}
