// pathtrace.cu — wavefront path tracer around the traversal kernels: the
// reference's PathIntegrator::Li (integrator.cpp:252-326) with
// UniformSampleOneLight / EstimateDirect (:69-120), the Halton sampler of
// common/sampler.h:143-252 and the per-pixel sample order of
// ParallelIntegrator::render's eval_pixel (integrator.cpp:136-159), run as
// queues of rays:
//
//   k_pt_camera   camera rays of one sample per pixel into queue A
//   trace         closest hit over queue A (trace.cu)
//   k_pt_shade    emission at the first bounce, next-event estimation (one
//                 shadow ray into the shadow queue), cosine-weighted
//                 Lambertian bounce into queue B; paths that end leave the
//                 queues.  Both queues are compacted with one atomic per
//                 warp (ballot + popc).
//   trace         any hit over the shadow queue; k_pt_shadow adds the
//                 unoccluded contributions to the image
//
// With a medium bounded by a closed mesh (flg_volpath_mesh: the reference's
// HVolume attached to a mesh primitive, scene.cpp:224-228) the boundary
// triangles carry no material: a path that reaches one passes straight
// through (not a bounce) and is inside the medium afterwards if it entered
// (dot(d, ng) < 0) — SInteraction::SpawnRay's rule (interaction.cpp:16-38),
// which also puts every ray leaving a material surface outside any medium.
// Inside, HVolume::sample (volume.cpp:164-190) picks a scattering distance;
// shadow rays follow VolEstimateTr (integrator.cpp:40-66): closest hits in
// turn, a material surface blocks, an interface multiplies HVolume::tr of the
// segment and switches the medium.  Tracking draws come from Philox streams.
//
// Emitters are triangles of the mesh.  The reference cannot sample a
// triangle light (Triangle::sample is TODO, shape.cpp:157-160); here a light
// triangle is chosen uniformly and a point on it by UniformSampleTriangle
// (math_utils.h:90-93), with the area pdf converted to solid angle.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "volume.cuh"

namespace flg {

constexpr int kPtPrimes = 64;
__constant__ int c_primes[kPtPrimes] = {
    2,   3,   5,   7,   11,  13,  17,  19,  23,  29,  31,  37,  41,  43,  47,  53,  59,  61,  67,  71,  73,  79,
    83,  89,  97,  101, 103, 107, 109, 113, 127, 131, 137, 139, 149, 151, 157, 163, 167, 173, 179, 181, 191, 193,
    197, 199, 211, 223, 227, 229, 233, 239, 241, 251, 257, 263, 269, 271, 277, 281, 283, 293, 307, 311};

struct Halton {
  uint64_t scale0, scale1, stride, inv0, inv1;
  int exp0, exp1;
};

// RadicalInverse_ (sampler.h), in fp32 as the reference evaluates it.
__device__ __forceinline__ float radical_inverse(int base, uint64_t a) {
  const float inv_base = 1.0f / (float)base;
  uint64_t rev = 0;
  float inv_n = 1.0f;
  while (a) {
    const uint64_t next = a / (uint64_t)base;
    const uint64_t digit = a - next * (uint64_t)base;
    rev = rev * (uint64_t)base + digit;
    inv_n *= inv_base;
    a = next;
  }
  return (float)rev * inv_n;
}

__device__ __forceinline__ uint64_t inverse_radical_inverse(int base, uint64_t inverse, int n_digits) {
  uint64_t index = 0;
  for (int i = 0; i < n_digits; ++i) {
    const uint64_t digit = inverse % (uint64_t)base;
    inverse /= (uint64_t)base;
    index = index * (uint64_t)base + digit;
  }
  return index;
}

// HaltonSampler::getIndexForSample offset of pixel (x, y) (sampler.h:200-221).
__device__ __forceinline__ uint64_t halton_pixel_offset(const Halton &H, int x, int y) {
  if (H.stride <= 1) return 0;
  const uint64_t pm0 = (uint64_t)(x % 128), pm1 = (uint64_t)(y % 128);
  uint64_t off = inverse_radical_inverse(2, pm0, H.exp0) * (H.stride / H.scale0) * H.inv0;
  off += inverse_radical_inverse(3, pm1, H.exp1) * (H.stride / H.scale1) * H.inv1;
  return off % H.stride;
}

// HaltonSampler::get1D for dimension `dim` of sample `index` (sampler.h:233-244).
__device__ __forceinline__ float halton(const Halton &H, uint64_t index, int dim) {
  float v;
  if (dim == 0) v = radical_inverse(2, index / H.scale0);
  else if (dim == 1) v = radical_inverse(3, index / H.scale1);
  else v = radical_inverse(c_primes[dim < kPtPrimes ? dim : kPtPrimes - 1], index);
  return fminf(v, 0.99999994f);
}

struct PtScene {
  const float *pos;
  const int32_t *idx;
  int32_t light_first, light_count;
  float le[3], albedo[3];
  float eye[3], fwd[3], right[3], up[3];
  float fov_ratio, aspect;
  int width, height, spp, max_depth;
  // Participating medium: 0 none, 1 the grid's medium filling its box,
  // 2 a homogeneous medium bounded by the interface triangles
  // [iface_first, iface_first + iface_count).
  int medium;
  GridDev G;
  float g;
  uint64_t seed;
  int32_t iface_first, iface_count;
  float msig_s[3], msig_t[3], mdens;
};

__device__ __forceinline__ bool pt_iface(const PtScene &S, int64_t tri) {
  return tri >= S.iface_first && tri < S.iface_first + S.iface_count;
}

// HVolume::tr (volume.cpp:159-161) over [0, t]: exp(-t density sigma_t).
__device__ __forceinline__ float3 hvol_tr(const PtScene &S, float t) {
  return make_float3(expf(-t * S.mdens * S.msig_t[0]), expf(-t * S.mdens * S.msig_t[1]),
                     expf(-t * S.mdens * S.msig_t[2]));
}

__device__ __forceinline__ float3 pt_vertex(const PtScene &S, int64_t tri, int k) {
  const int64_t v = S.idx ? (int64_t)S.idx[3 * tri + k] : 3 * tri + k;
  return make_float3(S.pos[3 * v], S.pos[3 * v + 1], S.pos[3 * v + 2]);
}

__device__ __forceinline__ float3 f3scale(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 f3norm(float3 a) {
  const float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
  return make_float3(a.x / l, a.y / l, a.z / l);
}

// OffsetRayOrigin (common/ray.h:64-93).
__device__ __forceinline__ float offset_axis(float p, float off) {
  const int oi = (int)(off * 256.0f);
  const float pi = __int_as_float(__float_as_int(p) + (p < 0.0f ? -oi : oi));
  return fabsf(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * off : pi;
}
__device__ __forceinline__ float3 offset_origin(float3 p, float3 n, float3 dir) {
  const float3 off = f3dot(n, dir) <= 0.0f ? make_float3(-n.x, -n.y, -n.z) : n;
  return make_float3(offset_axis(p.x, off.x), offset_axis(p.y, off.y), offset_axis(p.z, off.z));
}

// Camera::generateRay (common/camera.h:22-31) for continuous pixel (x, y).
__device__ __forceinline__ float3 camera_dir(const PtScene &S, float x, float y) {
  const float yo = S.fov_ratio * ((y / (float)S.height) * 2.0f - 1.0f);
  const float xo = S.fov_ratio * S.aspect * ((x / (float)S.width) * 2.0f - 1.0f);
  return f3norm(make_float3(S.fwd[0] + xo * S.right[0] + yo * S.up[0], S.fwd[1] + xo * S.right[1] + yo * S.up[1],
                            S.fwd[2] + xo * S.right[2] + yo * S.up[2]));
}

// A wavefront carries the paths of K consecutive samples s0 .. s0 + K - 1:
// path p = j * n_pix + pixel is sample s0 + j of that pixel.
struct PtQueues {
  float *rx[2][6];           // ray queues A/B: ox oy oz dx dy dz
  int32_t *path[2];          // queue slot -> path index
  float *sx[7];              // shadow queue: ox oy oz dx dy dz tmax
  float *rsx[6];             // the same segments traced from the far end back: ox oy oz dx dy dz
  float *scontrib;           // 3 per shadow slot
  int32_t *spath;            // path of a shadow slot
  float *beta;               // 3 per path
  float *rad;                // 3 per path: the path's radiance (each path adds to its own, no atomics)
  int32_t *cnt;              // Halton dimensions consumed, per path
  int32_t *cnt_end;          // dimension count at the end of sample 0, per pixel
  int32_t *counts;           // [0] queue B size, [1] shadow size, [2] second shadow queue size
  int32_t n_pix;             // pixels per sample
  // Medium bounded by a mesh: per path the bounce count, the segment count
  // (the key of its tracking streams) and whether it is inside; per shadow
  // slot whether it is inside, and a second shadow queue for the segments
  // past an interface.
  int32_t *bnc, *seg;
  uint8_t *inmed;
  uint8_t *smed[2];
  float *sx2[7];
  float *scontrib2;
  int32_t *spath2;
};

__global__ void k_pt_camera(PtScene S, Halton H, int s0, int n_path, PtQueues Q, int qa) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_path) return;
  const int i = p % Q.n_pix, s = s0 + p / Q.n_pix;
  const int x = i % S.width, y = i / S.width;
  const uint64_t off = halton_pixel_offset(H, x, y);
  float px, py;
  int cnt;
  if (s == 0) {  // eval_pixel's first ray goes through the pixel centre
    px = (float)x + 0.5f;
    py = (float)y + 0.5f;
    cnt = 0;
  } else {
    // sample 1 continues the dimensions left by sample 0; later samples
    // follow HaltonSampler::reset (integrator.cpp:148-156)
    const uint64_t index = off + (uint64_t)(s - 1) * H.stride;
    cnt = s == 1 ? Q.cnt_end[i] : 0;
    px = (float)x + halton(H, index, cnt);
    py = (float)y + halton(H, index, cnt + 1);
    cnt += 2;
  }
  const float3 d = camera_dir(S, px, py);
  Q.rx[qa][0][p] = S.eye[0];
  Q.rx[qa][1][p] = S.eye[1];
  Q.rx[qa][2][p] = S.eye[2];
  Q.rx[qa][3][p] = d.x;
  Q.rx[qa][4][p] = d.y;
  Q.rx[qa][5][p] = d.z;
  Q.path[qa][p] = p;
  Q.beta[3 * p] = Q.beta[3 * p + 1] = Q.beta[3 * p + 2] = 1.0f;
  Q.rad[3 * p] = Q.rad[3 * p + 1] = Q.rad[3 * p + 2] = 0.0f;
  Q.cnt[p] = cnt;
  if (S.medium == 2) {  // camera rays start outside any medium
    Q.bnc[p] = 0;
    Q.seg[p] = 0;
    Q.inmed[p] = 0;
  }
}

// Warp-aggregated slot in a compacted queue.
__device__ __forceinline__ int queue_slot(bool want, int32_t *counter) {
  const unsigned m = __ballot_sync(0xFFFFFFFFu, want);
  if (!m) return -1;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// One path vertex per queued ray (PathIntegrator::Li, integrator.cpp:
// 252-326; with a medium, VolPathIntegrator::Li, :407-510): emission at the
// first bounce; with a medium, delta tracking over [0, t_hit] may move the
// vertex to a scattering point (beta *= sigma_s / sigma_t); next-event
// estimation toward one light triangle (Lambertian or Henyey-Greenstein
// factor; the shadow ray's transmittance is applied in k_pt_shadow); the
// continuation ray (cosine-weighted bounce or HGSampleP).
// 4 CTAs per SM (64 registers, no spills; 74 without the bound): +1.3 % on a
// 1080p / 16-spp render of a 1.3 M-triangle mesh.
__global__ void __launch_bounds__(256, 4)
    k_pt_shade(PtScene S, Halton H, int s0, int depth, int64_t n_in, PtQueues Q, int qa, const int32_t *__restrict__ prim,
               const float *__restrict__ th, const float *__restrict__ uh, const float *__restrict__ vh) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = q < n_in;
  const int qb = qa ^ 1;
  int pid = 0, pix = 0, s = 0, cnt = 0;
  bool cont = false, shadow = false;
  float3 o = make_float3(0.f, 0.f, 0.f), d = o, beta = make_float3(1.f, 1.f, 1.f);
  float3 so = o, sd = o, contrib = o, nd = o, no = o;
  float smax = 0.0f;
  const float inv_spp = 1.0f / (float)S.spp;
  const bool meshmed = S.medium == 2;
  int bnc = depth, sg = depth;     // bounces and segments so far (equal without interfaces)
  bool inmed = false, nmed = false, smed = false;  // inside now / after this vertex / shadow ray start
  if (valid) {
    pid = Q.path[qa][q];
    pix = pid % Q.n_pix;
    s = s0 + pid / Q.n_pix;
    o = make_float3(Q.rx[qa][0][q], Q.rx[qa][1][q], Q.rx[qa][2][q]);
    d = make_float3(Q.rx[qa][3][q], Q.rx[qa][4][q], Q.rx[qa][5][q]);
    beta = make_float3(Q.beta[3 * pid], Q.beta[3 * pid + 1], Q.beta[3 * pid + 2]);
    cnt = Q.cnt[pid];
    if (meshmed) {
      bnc = Q.bnc[pid];
      sg = Q.seg[pid];
      inmed = Q.inmed[pid] != 0;
    }
    const int32_t h = prim[q];
    const int x = pix % S.width, y = pix / S.width;
    const uint64_t off = halton_pixel_offset(H, x, y);
    const uint64_t index = off + (uint64_t)(s > 0 ? s - 1 : 0) * H.stride;
    if (h >= 0) {
      const float3 a = pt_vertex(S, h, 0), b = pt_vertex(S, h, 1), c = pt_vertex(S, h, 2);
      const float u = uh[q], v = vh[q], w = 1.0f - u - v;
      const float3 p = make_float3(w * a.x + u * b.x + v * c.x, w * a.y + u * b.y + v * c.y,
                                   w * a.z + u * b.z + v * c.z);
      const float3 ng = f3norm(f3cross(f3sub(b, a), f3sub(c, a)));
      const bool is_light = h >= S.light_first && h < S.light_first + S.light_count;
      // emission seen directly (bounces == 0); AreaLight::L (light.cpp:76-79)
      if (bnc == 0 && is_light && f3dot(ng, make_float3(-d.x, -d.y, -d.z)) > 0.0f) {
        Q.rad[3 * pid] += beta.x * S.le[0] * inv_spp;
        Q.rad[3 * pid + 1] += beta.y * S.le[1] * inv_spp;
        Q.rad[3 * pid + 2] += beta.z * S.le[2] * inv_spp;
      }
      if (bnc < S.max_depth) {
        const float3 wo = make_float3(-d.x, -d.y, -d.z);
        // Volume::sample over the segment up to the surface (volume.cpp:109-148)
        bool scatter = false;
        float3 ps = p;
        if (S.medium == 1) {
          RayStream rs;
          rs.init(S.seed, path_stream_id(pix, s, depth, 0), 0u);
          scatter = S.G.bidx ? delta_track<true>(S.G, __ldg(S.G.params), o, d, th[q], rs, ps)
                             : delta_track<false>(S.G, __ldg(S.G.params), o, d, th[q], rs, ps);
          if (scatter) {
            const float wgt = S.G.sigma_s / S.G.sigma_t;
            beta = make_float3(beta.x * wgt, beta.y * wgt, beta.z * wgt);
          }
        } else if (meshmed && inmed) {
          // HVolume::sample (volume.cpp:164-190) with ray.m_tMax = t_hit: a
          // channel, then a distance with pdf sigma_t[ch] e^(-sigma_t[ch] t)
          RayStream rs;
          rs.init(S.seed, path_stream_id(pix, s, sg, 0), 0u);
          const int ch = min((int)((double)rs.next() * 3.0), 2);  // get1D() * 3.0 is a double product
          const float t = -flg_logf(1.0f - rs.next()) / (S.mdens * S.msig_t[ch]);
          const float tmax = th[q];
          const float3 tr = hvol_tr(S, fminf(t, tmax));
          if (t < tmax) {
            const float pdf = (S.msig_t[0] * tr.x + S.msig_t[1] * tr.y + S.msig_t[2] * tr.z) * 1.0f / 3.0f;
            beta = make_float3(beta.x * (S.msig_s[0] * tr.x / pdf), beta.y * (S.msig_s[1] * tr.y / pdf),
                               beta.z * (S.msig_s[2] * tr.z / pdf));
            ps = make_float3(o.x + d.x * t, o.y + d.y * t, o.z + d.z * t);
            scatter = true;
          } else {
            const float pdf = (tr.x + tr.y + tr.z) * 1.0f / 3.0f;
            beta = make_float3(beta.x * (tr.x / pdf), beta.y * (tr.y / pdf), beta.z * (tr.z / pdf));
          }
        }
        if (meshmed && !scatter && pt_iface(S, h)) {
          // a material-less boundary: straight on, not a bounce
          no = offset_origin(p, ng, d);
          nd = d;
          nmed = f3dot(d, ng) < 0.0f;
          cont = true;
        } else {
        nmed = meshmed && scatter && inmed;  // a medium vertex keeps the medium; a surface leaves it
        smed = nmed;
        ++bnc;
        // UniformSampleOneLight / EstimateDirect
        const float ul = halton(H, index, cnt);
        const float ua = halton(H, index, cnt + 1), ub = halton(H, index, cnt + 2);
        cnt += 3;
        const int li = min((int)(ul * (float)S.light_count), S.light_count - 1);
        const float light_pdf = 1.0f / (float)S.light_count;
        const int64_t lt = S.light_first + li;
        const float3 la = pt_vertex(S, lt, 0), lb = pt_vertex(S, lt, 1), lc = pt_vertex(S, lt, 2);
        const float su0 = sqrtf(ua);
        const float b0 = 1.0f - su0, b1 = ub * su0, b2 = 1.0f - b0 - b1;
        const float3 lp = make_float3(b0 * la.x + b1 * lb.x + b2 * lc.x, b0 * la.y + b1 * lb.y + b2 * lc.y,
                                      b0 * la.z + b1 * lb.z + b2 * lc.z);
        const float3 lcr = f3cross(f3sub(lb, la), f3sub(lc, la));
        const float area = 0.5f * sqrtf(f3dot(lcr, lcr));
        const float3 ln = f3scale(lcr, 1.0f / (2.0f * area));
        const float3 toL = f3sub(lp, ps);
        const float dist = sqrtf(f3dot(toL, toL));
        const float3 wi = f3scale(toL, 1.0f / dist);
        const float cos_l = -f3dot(ln, wi);
        if (cos_l > 0.0f && dist > 0.0f) {
          const float pdf = dist * dist / (cos_l * area);
          float3 f;
          if (scatter) {
            const float ph = hg_p(wi, wo, S.g);
            f = make_float3(ph, ph, ph);
          } else {
            const float cos_s = fabsf(f3dot(wi, ng));
            f = make_float3(S.albedo[0] * (1.0f / 3.14159265358979f) * cos_s,
                            S.albedo[1] * (1.0f / 3.14159265358979f) * cos_s,
                            S.albedo[2] * (1.0f / 3.14159265358979f) * cos_s);
          }
          const float k = inv_spp / (pdf * light_pdf);
          contrib = make_float3(beta.x * f.x * S.le[0] * k, beta.y * f.y * S.le[1] * k, beta.z * f.z * S.le[2] * k);
          so = scatter ? ps : offset_origin(p, ng, wi);  // a medium vertex has no normal to offset along
          sd = wi;
          smax = dist - 1e-4f;  // SpawnRayTo: tMax = |p' - p| - SHADOW_EPS
          shadow = contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f;
        }
        const float u1 = halton(H, index, cnt), u2 = halton(H, index, cnt + 1);
        cnt += 2;
        if (scatter) {
          // HGSampleP: the phase function and its pdf cancel in beta
          nd = hg_sample(wo, u1, u2, S.g);
          no = ps;
          cont = true;
        } else {
          // Lambertian sampleF in the frame of the normal (material_base.hpp:14-41)
          float3 bn;
          if (fabsf(ng.x) > fabsf(ng.z)) bn = make_float3(-ng.y, ng.x, 0.0f);
          else bn = make_float3(0.0f, -ng.z, ng.y);
          bn = f3norm(bn);
          const float3 tg = f3cross(bn, ng);
          const float woz = f3dot(wo, ng);
          // CosineSampleHemisphere (ConcentricSampleDisk, math_utils.h:69-88)
          const float ux = u1 * 2.0f - 1.0f, uy = u2 * 2.0f - 1.0f;
          float dx = 0.0f, dy = 0.0f;
          if (ux != 0.0f || uy != 0.0f) {
            float r, theta;
            if (fabsf(ux) > fabsf(uy)) {
              r = ux;
              theta = 0.78539816f * (uy / ux);
            } else {
              r = uy;
              theta = 1.57079633f - 0.78539816f * (ux / uy);
            }
            dx = cosf(theta) * r;
            dy = sinf(theta) * r;
          }
          const float dz = sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy));
          const float pdf_b = woz * dz > 0.0f ? fabsf(dz) * (1.0f / 3.14159265358979f) : 0.0f;
          if (pdf_b > 0.0f) {
            nd = make_float3(tg.x * dx + bn.x * dy + ng.x * dz, tg.y * dx + bn.y * dy + ng.y * dz,
                             tg.z * dx + bn.z * dy + ng.z * dz);
            const float fcos = (1.0f / 3.14159265358979f) * fabsf(f3dot(nd, ng)) / pdf_b;
            beta = make_float3(beta.x * S.albedo[0] * fcos, beta.y * S.albedo[1] * fcos, beta.z * S.albedo[2] * fcos);
            nd = f3norm(nd);
            no = offset_origin(p, ng, nd);
            cont = true;
          }
        }
        }
      }
    }
    if (!cont && s == 0) Q.cnt_end[pix] = cnt;
  }
  const int ss = queue_slot(valid && shadow, Q.counts + 1);
  if (ss >= 0) {
    Q.sx[0][ss] = so.x; Q.sx[1][ss] = so.y; Q.sx[2][ss] = so.z;
    Q.sx[3][ss] = sd.x; Q.sx[4][ss] = sd.y; Q.sx[5][ss] = sd.z;
    Q.sx[6][ss] = smax;
    // Occlusion is traced from the light end: on a closed surface the
    // segments from the far side cross the hollow interior, where boxes of
    // large surface patches overlap the ray without holding an occluder, but
    // from the light the near side of the surface is found at once.  The
    // segment is the same: [so, so + smax sd] from its far end, with the
    // surface's own triangle (256 ulps behind so) still excluded.
    Q.rsx[0][ss] = so.x + sd.x * smax; Q.rsx[1][ss] = so.y + sd.y * smax; Q.rsx[2][ss] = so.z + sd.z * smax;
    Q.rsx[3][ss] = -sd.x; Q.rsx[4][ss] = -sd.y; Q.rsx[5][ss] = -sd.z;
    Q.scontrib[3 * ss] = contrib.x;
    Q.scontrib[3 * ss + 1] = contrib.y;
    Q.scontrib[3 * ss + 2] = contrib.z;
    Q.spath[ss] = pid;
    if (meshmed) Q.smed[0][ss] = smed ? 1 : 0;
  }
  const int ns = queue_slot(valid && cont, Q.counts);
  if (ns >= 0) {
    Q.rx[qb][0][ns] = no.x; Q.rx[qb][1][ns] = no.y; Q.rx[qb][2][ns] = no.z;
    Q.rx[qb][3][ns] = nd.x; Q.rx[qb][4][ns] = nd.y; Q.rx[qb][5][ns] = nd.z;
    Q.path[qb][ns] = pid;
    Q.beta[3 * pid] = beta.x;
    Q.beta[3 * pid + 1] = beta.y;
    Q.beta[3 * pid + 2] = beta.z;
    Q.cnt[pid] = cnt;
    if (meshmed) {
      Q.bnc[pid] = bnc;
      Q.seg[pid] = sg + 1;
      Q.inmed[pid] = nmed ? 1 : 0;
    }
  }
}

// One step of VolEstimateTr (integrator.cpp:40-66) for the shadow rays of a
// mesh-bounded medium, traced forward with closest hit: no hit within the
// segment adds the contribution; a material surface blocks; an interface
// multiplies HVolume::tr of the part travelled if inside, switches the
// medium as SInteraction::SpawnRay does and queues the rest of the segment
// from an offset origin.  Contributions carry the transmittance so far.
__global__ void k_pt_shadow_step(PtScene S, int64_t n, const int32_t *__restrict__ prim, const float *__restrict__ th,
                                 PtQueues Q, int in) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  float *const *sx = in == 0 ? Q.sx : Q.sx2;
  float *const *so_ = in == 0 ? Q.sx2 : Q.sx;
  const float *sc = in == 0 ? Q.scontrib : Q.scontrib2;
  float *sco = in == 0 ? Q.scontrib2 : Q.scontrib;
  const int32_t *sp = in == 0 ? Q.spath : Q.spath2;
  int32_t *spo = in == 0 ? Q.spath2 : Q.spath;
  bool requeue = false;
  float3 no = make_float3(0.f, 0.f, 0.f), d = no, c = no;
  float rem = 0.0f;
  bool nmed = false;
  int pid = 0;
  if (valid) {
    pid = sp[i];
    c = make_float3(sc[3 * i], sc[3 * i + 1], sc[3 * i + 2]);
    const int32_t h = prim[i];
    if (h < 0) {
      // the light is reached; the last segment is not attenuated (VolEstimateTr
      // returns tr as it stands when nothing more is hit)
      Q.rad[3 * pid] += c.x;
      Q.rad[3 * pid + 1] += c.y;
      Q.rad[3 * pid + 2] += c.z;
    } else if (pt_iface(S, h)) {
      const float t = th[i];
      if (Q.smed[in][i]) {
        const float3 tr = hvol_tr(S, t);
        c = make_float3(c.x * tr.x, c.y * tr.y, c.z * tr.z);
      }
      const float3 o = make_float3(sx[0][i], sx[1][i], sx[2][i]);
      d = make_float3(sx[3][i], sx[4][i], sx[5][i]);
      rem = sx[6][i] - t;
      if (rem < 0.0f) {
        Q.rad[3 * pid] += c.x;
        Q.rad[3 * pid + 1] += c.y;
        Q.rad[3 * pid + 2] += c.z;
      } else {
        const float3 a = pt_vertex(S, h, 0), b = pt_vertex(S, h, 1), cc = pt_vertex(S, h, 2);
        const float3 ng = f3norm(f3cross(f3sub(b, a), f3sub(cc, a)));
        const float3 ph = make_float3(o.x + d.x * t, o.y + d.y * t, o.z + d.z * t);
        no = offset_origin(ph, ng, d);
        nmed = f3dot(d, ng) < 0.0f;
        requeue = true;
      }
    }
  }
  const int slot = queue_slot(valid && requeue, Q.counts + 2);
  if (slot >= 0) {
    so_[0][slot] = no.x; so_[1][slot] = no.y; so_[2][slot] = no.z;
    so_[3][slot] = d.x; so_[4][slot] = d.y; so_[5][slot] = d.z;
    so_[6][slot] = rem;
    sco[3 * slot] = c.x;
    sco[3 * slot + 1] = c.y;
    sco[3 * slot + 2] = c.z;
    spo[slot] = pid;
    Q.smed[in ^ 1][slot] = nmed ? 1 : 0;
  }
}

// Unoccluded shadow rays add their contribution; with a medium, times the
// ratio-tracking transmittance of the shadow segment (VolEstimateTr,
// integrator.cpp:40-66).
__global__ void k_pt_shadow(PtScene S, int s0, int depth, int64_t n, const uint8_t *__restrict__ occ, PtQueues Q) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || occ[i]) return;
  const int pid = Q.spath[i];
  const int p = pid % Q.n_pix, s = s0 + pid / Q.n_pix;
  float tr = 1.0f;
  if (S.medium) {
    const float3 o = make_float3(Q.sx[0][i], Q.sx[1][i], Q.sx[2][i]);
    const float3 d = make_float3(Q.sx[3][i], Q.sx[4][i], Q.sx[5][i]);
    float ct, cc;
    uint32_t ck;
    const int64_t id = (int64_t)path_stream_id(p, s, depth, 1);
    tr = S.G.bidx ? ratio_track<true>(S.G, __ldg(S.G.params), __ldg(S.G.params + 1), o, d, Q.sx[6][i], S.seed, id,
                                      ct, ck, cc)
                  : ratio_track<false>(S.G, __ldg(S.G.params), __ldg(S.G.params + 1), o, d, Q.sx[6][i], S.seed, id,
                                       ct, ck, cc);
    if (tr == 0.0f) return;
  }
  // A path has at most one shadow ray per bounce: no other thread adds to it.
  Q.rad[3 * pid] += Q.scontrib[3 * i] * tr;
  Q.rad[3 * pid + 1] += Q.scontrib[3 * i + 1] * tr;
  Q.rad[3 * pid + 2] += Q.scontrib[3 * i + 2] * tr;
}

// Adds the wavefront's K samples of every pixel to the image, in sample
// order (a fixed summation order: the image does not depend on scheduling).
__global__ void k_pt_reduce(const float *__restrict__ rad, int n_pix, int k_samples, float *radiance) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // pixel * 3 + channel
  if (e >= 3 * (int64_t)n_pix) return;
  float acc = radiance[e];
  for (int j = 0; j < k_samples; ++j) acc += rad[(int64_t)j * 3 * n_pix + e];
  radiance[e] = acc;
}

static void host_halton(int width, int height, Halton &H) {
  // HaltonSampler constructor (sampler.h:145-160) with sample_interval =
  // (resX, resY) (integrator.cpp:173) and M_MAX_RESOLUTION = 128.
  const int res[2] = {width, height};
  uint64_t scale[2];
  int ex[2];
  for (int i = 0; i < 2; ++i) {
    const int base = i == 0 ? 2 : 3;
    uint64_t sc = 1;
    int e = 0;
    while (sc < (uint64_t)std::min(res[i], 128)) {
      sc *= base;
      ++e;
    }
    scale[i] = sc;
    ex[i] = e;
  }
  auto mul_inverse = [](int64_t a, int64_t b) {  // ExGCD / MulModInverse
    int64_t old_r = a, r = b, old_s = 1, s = 0;
    while (r != 0) {
      const int64_t qq = old_r / r;
      int64_t t = old_r - qq * r;
      old_r = r;
      r = t;
      t = old_s - qq * s;
      old_s = s;
      s = t;
    }
    int64_t x = old_s % b;
    if (x < 0) x += b;
    return (uint64_t)x;
  };
  H.scale0 = scale[0];
  H.scale1 = scale[1];
  H.exp0 = ex[0];
  H.exp1 = ex[1];
  H.stride = scale[0] * scale[1];
  H.inv0 = mul_inverse((int64_t)scale[1], (int64_t)scale[0]);
  H.inv1 = mul_inverse((int64_t)scale[0], (int64_t)scale[1]);
}

}  // namespace flg

using namespace flg;

static int pathtrace_run(flg_ctx ctx, flg_bvh bvh, flg_grid grid, const flg_mesh_medium *mm, uint64_t seed,
                         const flg_pt_scene *scene, const flg_pt_camera *cam, int32_t spp, int32_t max_depth,
                         const flg_trace_opts *opts, float *radiance, flg_pt_stats *stats) {
  if (!ctx || !bvh || !scene || !cam || !radiance) return ctx ? set_error(ctx, FLG_ERR_ARG, "NULL argument") : FLG_ERR_ARG;
  if (spp > 65535 || max_depth > 255) return set_error(ctx, FLG_ERR_ARG, "spp above 65535 or depth above 255");
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "path tracing synchronises per bounce; not capturable");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "path tracing takes a single-scene handle");
  if (cam->width < 1 || cam->height < 1 || spp < 1 || max_depth < 0)
    return set_error(ctx, FLG_ERR_ARG, "bad image size, spp or depth");
  if (scene->n_tri != bvh->n_tri) return set_error(ctx, FLG_ERR_ARG, "scene and handle differ in triangle count");
  if (scene->light_count < 1 || scene->light_first < 0 || scene->light_first + scene->light_count > scene->n_tri)
    return set_error(ctx, FLG_ERR_ARG, "light triangles out of range");
  if ((int64_t)cam->width * cam->height > (int64_t)1 << 26) return set_error(ctx, FLG_ERR_UNSUPPORTED, "image too large");
  if (mm) {
    if (mm->first < 0 || mm->count < 1 || (int64_t)mm->first + mm->count > scene->n_tri)
      return set_error(ctx, FLG_ERR_ARG, "medium boundary triangles out of range");
    if (mm->first < scene->light_first + scene->light_count && scene->light_first < mm->first + mm->count)
      return set_error(ctx, FLG_ERR_ARG, "medium boundary and light triangles overlap");
    for (int k = 0; k < 3; ++k)
      if (!(mm->sigma_s[k] >= 0.0f) || !(mm->sigma_a[k] >= 0.0f) || !(mm->sigma_s[k] + mm->sigma_a[k] > 0.0f))
        return set_error(ctx, FLG_ERR_ARG, "medium coefficients must be >= 0 with sigma_t > 0");
    if (!(mm->density > 0.0f) || !(mm->g > -1.0f && mm->g < 1.0f))
      return set_error(ctx, FLG_ERR_ARG, "medium density must be > 0 and |g| < 1");
  }
  PtScene S;
  std::memset(&S, 0, sizeof(S));
  S.medium = grid ? 1 : mm ? 2 : 0;
  if (mm) {
    S.iface_first = mm->first;
    S.iface_count = mm->count;
    for (int k = 0; k < 3; ++k) {
      S.msig_s[k] = mm->sigma_s[k];
      S.msig_t[k] = mm->sigma_s[k] + mm->sigma_a[k];
    }
    S.mdens = mm->density;
    S.g = mm->g;
  } else {
    S.iface_first = -1;
    S.iface_count = 0;
  }
  if (grid) {
    if (grid->ctx != ctx) return set_error(ctx, FLG_ERR_ARG, "grid belongs to another context");
    S.G = grid_dev(grid);
    S.g = grid->medium.g;
  } else if (!mm) {
    S.g = 0.0f;
  }
  S.seed = seed;
  S.pos = scene->pos;
  S.idx = scene->idx;
  S.light_first = scene->light_first;
  S.light_count = scene->light_count;
  for (int k = 0; k < 3; ++k) {
    S.le[k] = scene->light_le[k];
    S.albedo[k] = scene->albedo[k];
    S.eye[k] = cam->eye[k];
  }
  // Camera constructor (camera.h:14-20): forward, right = up x forward,
  // image up = forward x right.
  float f[3] = {cam->target[0] - cam->eye[0], cam->target[1] - cam->eye[1], cam->target[2] - cam->eye[2]};
  auto nrm = [](float *v) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
  };
  nrm(f);
  float r[3] = {cam->up[1] * f[2] - cam->up[2] * f[1], cam->up[2] * f[0] - cam->up[0] * f[2],
                cam->up[0] * f[1] - cam->up[1] * f[0]};
  nrm(r);
  float u[3] = {f[1] * r[2] - f[2] * r[1], f[2] * r[0] - f[0] * r[2], f[0] * r[1] - f[1] * r[0]};
  nrm(u);
  for (int k = 0; k < 3; ++k) {
    S.fwd[k] = f[k];
    S.right[k] = r[k];
    S.up[k] = u[k];
  }
  S.fov_ratio = std::tan(3.14159265358979f * cam->fov_deg / 360.0f);
  S.aspect = (float)cam->width / (float)cam->height;
  S.width = cam->width;
  S.height = cam->height;
  S.spp = spp;
  S.max_depth = max_depth;
  Halton H;
  host_halton(cam->width, cam->height, H);

  const int64_t n = (int64_t)cam->width * cam->height;
  // Samples per wavefront: sample 0 alone (sample 1 continues its Halton
  // dimensions), then up to kmax at a time, with up to 2^25 paths in flight,
  // so every bounce's trace launches fill the GPU.
  const int64_t kmax = std::max<int64_t>(1, std::min<int64_t>(spp, ((int64_t)1 << 25) / n));
  const int64_t np = kmax * n;  // path slots
  // Buffers (per path slot): 2 x 6 ray arrays, 2 path maps, 7 + 6 shadow
  // arrays + 3 contrib + path, beta 3, radiance 3, cnt, hits 4, occluded; cnt_end per
  // pixel; counters.  Each sub-buffer is rounded up to 256 bytes.
  // With a mesh-bounded medium also: bounce and segment counts, inside flags
  // (per path and per slot of both shadow queues), the second shadow queue.
  const size_t fl = sizeof(float) * np;
  const size_t extra = mm ? fl * (2 + 7 + 3 + 1) + 3 * (size_t)np + 14 * 256 : 0;
  const size_t need = fl * (12 + 2 + 7 + 6 + 3 + 1 + 3 + 3 + 1 + 4) + sizeof(int32_t) * n + np + 64 + 38 * 256 + extra;
  if (ctx->pt_bytes < need) {
    cudaFree(ctx->pt_buf);
    ctx->pt_buf = nullptr;
    ctx->pt_bytes = 0;
    FLG_CUDA(ctx, cudaMalloc(&ctx->pt_buf, need));
    ctx->pt_bytes = need;
  }
  char *bp = (char *)ctx->pt_buf;
  auto take = [&](size_t bytes) {
    char *p = bp;
    bp += (bytes + 255) & ~(size_t)255;
    return (void *)p;
  };
  PtQueues Q;
  Q.n_pix = (int32_t)n;
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < 6; ++k) Q.rx[a][k] = (float *)take(fl);
  Q.path[0] = (int32_t *)take(fl);
  Q.path[1] = (int32_t *)take(fl);
  for (int k = 0; k < 7; ++k) Q.sx[k] = (float *)take(fl);
  for (int k = 0; k < 6; ++k) Q.rsx[k] = (float *)take(fl);
  Q.scontrib = (float *)take(3 * fl);
  Q.spath = (int32_t *)take(fl);
  Q.beta = (float *)take(3 * fl);
  Q.rad = (float *)take(3 * fl);
  Q.cnt = (int32_t *)take(fl);
  Q.cnt_end = (int32_t *)take(sizeof(int32_t) * n);
  float *hbuf = (float *)take(4 * fl);
  uint8_t *occ = (uint8_t *)take(np);
  Q.counts = (int32_t *)take(64);
  Q.bnc = Q.seg = nullptr;
  Q.inmed = Q.smed[0] = Q.smed[1] = nullptr;
  for (int k = 0; k < 7; ++k) Q.sx2[k] = nullptr;
  Q.scontrib2 = nullptr;
  Q.spath2 = nullptr;
  if (mm) {
    Q.bnc = (int32_t *)take(fl);
    Q.seg = (int32_t *)take(fl);
    Q.inmed = (uint8_t *)take(np);
    Q.smed[0] = (uint8_t *)take(np);
    Q.smed[1] = (uint8_t *)take(np);
    for (int k = 0; k < 7; ++k) Q.sx2[k] = (float *)take(fl);
    Q.scontrib2 = (float *)take(3 * fl);
    Q.spath2 = (int32_t *)take(fl);
  }
  if (bp > (char *)ctx->pt_buf + need) return set_error(ctx, FLG_ERR_STATE, "internal buffer layout");

  cudaStream_t st = ctx->stream;
  FLG_CUDA(ctx, cudaMemsetAsync(radiance, 0, 3 * sizeof(float) * n, st));
  int64_t n_closest = 0, n_shadow = 0;
  int32_t counts[2];
  for (int s0 = 0; s0 < spp;) {
    const int k = s0 == 0 ? 1 : (int)std::min<int64_t>(kmax, spp - s0);
    const int64_t n_path = (int64_t)k * n;
    int qa = 0;
    k_pt_camera<<<(unsigned)ceil_div(n_path, 256), 256, 0, st>>>(S, H, s0, (int)n_path, Q, qa);
    FLG_LAUNCH_CHECK(ctx, "k_pt_camera");
    int64_t n_a = n_path;
    // Without interfaces an iteration is a bounce; with them a path may pass
    // through boundaries between bounces, up to 255 segments in all (the
    // segment count keys its tracking streams); paths beyond that end.
    const int iters = mm ? 255 : max_depth + 1;
    for (int depth = 0; depth < iters && n_a > 0; ++depth) {
      // t > 0 as the live renderer's Triangle::intersect (shape.cpp:100-148)
      flg_rays rr{Q.rx[qa][0], Q.rx[qa][1], Q.rx[qa][2], Q.rx[qa][3], Q.rx[qa][4], Q.rx[qa][5], nullptr, nullptr,
                  1e-30f, 3.402823466e+38f};
      flg_hits hh{(int32_t *)hbuf, hbuf + np, hbuf + 2 * np, hbuf + 3 * np};
      int rc = trace_enqueue(ctx, st, 0, bvh, &rr, n_a, opts, nullptr, 1, &hh, nullptr);
      if (rc) return rc;
      n_closest += n_a;
      FLG_CUDA(ctx, cudaMemsetAsync(Q.counts, 0, 2 * sizeof(int32_t), st));
      k_pt_shade<<<(unsigned)ceil_div(n_a, 256), 256, 0, st>>>(S, H, s0, depth, n_a, Q, qa, hh.prim, hh.t, hh.u,
                                                                hh.v);
      FLG_LAUNCH_CHECK(ctx, "k_pt_shade");
      FLG_CUDA(ctx, cudaMemcpyAsync(counts, Q.counts, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      FLG_CUDA(ctx, cudaStreamSynchronize(st));
      if (counts[1] > 0 && mm) {
        // VolEstimateTr: closest hits along the segment until it is blocked,
        // reaches the light or has crossed 64 interfaces (then it counts as
        // blocked)
        int64_t n_s = counts[1];
        for (int step = 0, in = 0; step < 64 && n_s > 0; ++step, in ^= 1) {
          float *const *sx = in == 0 ? Q.sx : Q.sx2;
          flg_rays sr{sx[0], sx[1], sx[2], sx[3], sx[4], sx[5], nullptr, sx[6], 1e-30f, 0.0f};
          flg_hits sh{(int32_t *)hbuf, hbuf + np, hbuf + 2 * np, hbuf + 3 * np};
          rc = trace_enqueue(ctx, st, 0, bvh, &sr, n_s, opts, nullptr, 1, &sh, nullptr);
          if (rc) return rc;
          n_shadow += n_s;
          FLG_CUDA(ctx, cudaMemsetAsync(Q.counts + 2, 0, sizeof(int32_t), st));
          k_pt_shadow_step<<<(unsigned)ceil_div(n_s, 256), 256, 0, st>>>(S, n_s, sh.prim, sh.t, Q, in);
          FLG_LAUNCH_CHECK(ctx, "k_pt_shadow_step");
          int32_t nn = 0;
          FLG_CUDA(ctx, cudaMemcpyAsync(&nn, Q.counts + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
          FLG_CUDA(ctx, cudaStreamSynchronize(st));
          n_s = nn;
        }
      } else if (counts[1] > 0) {
        flg_rays sr{Q.rsx[0], Q.rsx[1], Q.rsx[2], Q.rsx[3], Q.rsx[4], Q.rsx[5], nullptr, Q.sx[6], 1e-30f, 0.0f};
        rc = trace_enqueue(ctx, st, 0, bvh, &sr, counts[1], opts, nullptr, 1, nullptr, occ);
        if (rc) return rc;
        n_shadow += counts[1];
        k_pt_shadow<<<(unsigned)ceil_div(counts[1], 256), 256, 0, st>>>(S, s0, depth, counts[1], occ, Q);
        FLG_LAUNCH_CHECK(ctx, "k_pt_shadow");
      }
      n_a = counts[0];
      qa ^= 1;
    }
    k_pt_reduce<<<(unsigned)ceil_div(3 * n, 256), 256, 0, st>>>(Q.rad, (int)n, k, radiance);
    FLG_LAUNCH_CHECK(ctx, "k_pt_reduce");
    s0 += k;
  }
  if (stats) {
    stats->closest_rays = n_closest;
    stats->shadow_rays = n_shadow;
  }
  return FLG_OK;
}

FLG_API int flg_pathtrace(flg_ctx ctx, flg_bvh bvh, const flg_pt_scene *scene, const flg_pt_camera *cam, int32_t spp,
                          int32_t max_depth, const flg_trace_opts *opts, float *radiance, flg_pt_stats *stats) {
  return pathtrace_run(ctx, bvh, nullptr, nullptr, 0, scene, cam, spp, max_depth, opts, radiance, stats);
}

FLG_API int flg_volpath_mesh(flg_ctx ctx, flg_bvh bvh, const flg_mesh_medium *medium, uint64_t seed,
                             const flg_pt_scene *scene, const flg_pt_camera *cam, int32_t spp, int32_t max_depth,
                             const flg_trace_opts *opts, float *radiance, flg_pt_stats *stats) {
  if (!medium) return ctx ? set_error(ctx, FLG_ERR_ARG, "medium is NULL") : FLG_ERR_ARG;
  return pathtrace_run(ctx, bvh, nullptr, medium, seed, scene, cam, spp, max_depth, opts, radiance, stats);
}

FLG_API int flg_volpath(flg_ctx ctx, flg_bvh bvh, flg_grid grid, uint64_t seed, const flg_pt_scene *scene,
                        const flg_pt_camera *cam, int32_t spp, int32_t max_depth, const flg_trace_opts *opts,
                        float *radiance, flg_pt_stats *stats) {
  if (!grid) return ctx ? set_error(ctx, FLG_ERR_ARG, "grid is NULL") : FLG_ERR_ARG;
  return pathtrace_run(ctx, bvh, grid, nullptr, seed, scene, cam, spp, max_depth, opts, radiance, stats);
}
