// volume.cuh — device functions of the dense-grid medium shared by the
// volume kernels (volume.cu) and the volumetric path tracer (pathtrace.cu):
// the grid lookup, the box clip, ratio tracking (OpenVDBVolume::tr,
// volume.cpp:75-107), delta tracking (OpenVDBVolume::sample, :109-148) and
// the Henyey-Greenstein phase function (math_utils.h:103-128).
#pragma once

#include "common.cuh"
#include "internal.h"

namespace flg {

// Edge of a sparse grid's bricks (voxels per axis).
constexpr int kBrick = 8;

// Kernel-side grid: dense ([nz][ny][nx], x fastest) or, with bidx, sparse:
// bidx[bz][by][bx] is the slot of an 8^3 brick in rho (z, y, x inside the
// brick, x fastest) or -1 for a brick of background (0) values.
struct GridDev {
  const float *rho;
  int nx, ny, nz;
  float lo[3], hi[3], scale[3];
  float sigma_s, sigma_a, sigma_t, rr;
  const float *params;  // [0] majorant, [1] 1/majorant (double quotient as float)
  const int32_t *bidx;  // sparse bricks, or NULL for a dense grid
  int bnx, bny;
};

// Offset of voxel (x, y, z) in rho, or -1 outside the grid or in an empty
// brick.  SP selects the sparse lookup at compile time, so the dense kernels
// keep their plain index arithmetic.
template <bool SP>
__device__ __forceinline__ int64_t grid_voxel(const GridDev &G, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= G.nx || y >= G.ny || z >= G.nz) return -1;
  if (!SP) return ((int64_t)z * G.ny + y) * G.nx + x;
  const int32_t slot = __ldg(G.bidx + ((int64_t)(z / kBrick) * G.bny + y / kBrick) * G.bnx + x / kBrick);
  if (slot < 0) return -1;
  return (int64_t)slot * (kBrick * kBrick * kBrick) + ((z % kBrick) * kBrick + y % kBrick) * kBrick + x % kBrick;
}

// Density at lattice point (x, y, z), background 0 outside.  The dense path
// tests the bounds before forming the index (as a plain branch around the
// load): routing it through grid_voxel's -1 sentinel cost 25 % of the
// tracking throughput.
template <bool SP>
__device__ __forceinline__ float gat(const GridDev &G, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= G.nx || y >= G.ny || z >= G.nz) return 0.0f;
  if (!SP) return __ldg(G.rho + ((int64_t)z * G.ny + y) * G.nx + x);
  const int64_t o = grid_voxel<true>(G, x, y, z);
  return o < 0 ? 0.0f : __ldg(G.rho + o);
}

__device__ __forceinline__ float lerpf(float a, float b, float w) { return a + (b - a) * w; }

template <bool SP>
__device__ __forceinline__ float sample_grid(const GridDev &G, float px, float py, float pz, int &x, int &y, int &z,
                                             float &fx, float &fy, float &fz) {
  float gx = (px - G.lo[0]) * G.scale[0];
  float gy = (py - G.lo[1]) * G.scale[1];
  float gz = (pz - G.lo[2]) * G.scale[2];
  float x0 = floorf(gx), y0 = floorf(gy), z0 = floorf(gz);
  x = (int)x0;
  y = (int)y0;
  z = (int)z0;
  fx = gx - x0;
  fy = gy - y0;
  fz = gz - z0;
  float c00 = lerpf(gat<SP>(G, x, y, z), gat<SP>(G, x + 1, y, z), fx);
  float c10 = lerpf(gat<SP>(G, x, y + 1, z), gat<SP>(G, x + 1, y + 1, z), fx);
  float c01 = lerpf(gat<SP>(G, x, y, z + 1), gat<SP>(G, x + 1, y, z + 1), fx);
  float c11 = lerpf(gat<SP>(G, x, y + 1, z + 1), gat<SP>(G, x + 1, y + 1, z + 1), fx);
  float c0 = lerpf(c00, c10, fy);
  float c1 = lerpf(c01, c11, fy);
  return lerpf(c0, c1, fz);
}

// AABB::intersect_pbrt (common/aabb.h:38-59) with t1 starting at tMax.
__device__ __forceinline__ bool box_pbrt(const GridDev &G, const float3 &o, const float3 &d, float tmax, float &t0o,
                                         float &t1o) {
  float t0 = 0.0f, t1 = tmax;
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float inv = __frcp_rn(dd[i]);
    float tn = (G.lo[i] - oo[i]) * inv;
    float tf = (G.hi[i] - oo[i]) * inv;
    bool s = tn > tf;
    float a = s ? tf : tn, b = s ? tn : tf;
    t0 = a > t0 ? a : t0;
    t1 = b < t1 ? b : t1;
    if (t0 > t1) return false;
  }
  t0o = t0;
  t1o = t1;
  return true;
}

// Ratio tracking of one ray; returns T and the state after the last
// roulette survival.
template <bool SP>
__device__ __forceinline__ float ratio_track(const GridDev &G, float maj, float inv_maj, const float3 &o,
                                             const float3 &d, float tmax, uint64_t seed, int64_t ray, float &ck_t,
                                             uint32_t &ck_k, float &ck_c) {
  ck_t = 0.0f;
  ck_k = 0u;
  ck_c = 1.0f;
  float t_min, t_max;
  if (!box_pbrt(G, o, d, tmax, t_min, t_max)) return 1.0f;
  float tr = 1.0f, t = fmaxf(t_min, 0.0f);
  t_max = fminf(t_max, tmax);
  const float max_mu = G.sigma_t * maj;
  RayStream rs;
  rs.init(seed, (uint64_t)ray, 0u);
  ck_t = t;
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = rs.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    int x, y, z;
    float fx, fy, fz;
    float dens = sample_grid<SP>(G, o.x + d.x * t, o.y + d.y * t, o.z + d.z * t, x, y, z, fx, fy, fz);
    tr *= 1.0f - fmaxf(0.0f, dens * inv_maj);
    if (tr < G.rr) {
      float q = fmaxf(0.05f, 1.0f - tr);
      if (rs.next() < q) return 0.0f;
      tr /= 1.0f - q;
      ck_t = t;
      ck_k = rs.k;
      ck_c = tr;
    }
  }
  return tr;
}

// Kernel-side view of a grid handle.
inline GridDev grid_dev(flg_grid g) {
  GridDev G;
  G.rho = g->rho;
  G.nx = g->nx;
  G.ny = g->ny;
  G.nz = g->nz;
  for (int k = 0; k < 3; ++k) {
    G.lo[k] = g->lo[k];
    G.hi[k] = g->hi[k];
    G.scale[k] = g->scale[k];
  }
  G.sigma_s = g->medium.sigma_s;
  G.sigma_a = g->medium.sigma_a;
  G.sigma_t = g->sigma_t;
  G.rr = g->medium.rr_threshold;
  G.params = g->d_params;
  G.bidx = g->bidx;
  G.bnx = g->bnx;
  G.bny = g->bny;
  return G;
}

// Delta tracking of one ray over [0, tmax] (volume.cpp:109-148): true on a
// real collision, with its position in p.  Draws from rs: one uniform per
// step plus one for the collision test.
template <bool SP>
__device__ __forceinline__ bool delta_track(const GridDev &G, float maj, const float3 &o, const float3 &d,
                                            float tmax, RayStream &rs, float3 &p) {
  float t_min, t_max;
  if (!box_pbrt(G, o, d, tmax, t_min, t_max)) return false;
  float t = fmaxf(t_min, 0.0f);
  const float max_mu = G.sigma_t * maj;
  t_max = fminf(t_max, tmax);
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = rs.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    float qx = o.x + d.x * t, qy = o.y + d.y * t, qz = o.z + d.z * t;
    int x, y, z;
    float fx, fy, fz;
    float dens = sample_grid<SP>(G, qx, qy, qz, x, y, z, fx, fy, fz);
    float p_s = G.sigma_s * dens / max_mu;
    float p_a = G.sigma_a * dens / max_mu;
    float p_n = 1.0f - p_s - p_a;
    if (rs.next() > p_n) {
      p = make_float3(qx, qy, qz);
      return true;
    }
  }
  return false;
}

// Henyey-Greenstein phase function HGP(wi, wo, g) (math_utils.h:103-107).
__device__ __forceinline__ float hg_p(const float3 &wi, const float3 &wo, float g) {
  const float cos_theta = wi.x * wo.x + wi.y * wo.y + wi.z * wo.z;
  const float denom = 1.0f + g * g + 2.0f * g * cos_theta;
  return (1.0f - g * g) / (denom * sqrtf(denom)) * 0.07957747154594766788f;
}

// HGSampleP (math_utils.h:111-128): direction wi around wo for uniforms u, v,
// in the frame of CoordinateSystem(wo) (math_utils.h:57-66).
__device__ __forceinline__ float3 hg_sample(const float3 &wo, float u, float v, float g) {
  float cos_theta;
  if (fabsf(g) < 1e-3f) {
    cos_theta = 1.0f - 2.0f * u;
  } else {
    const float tmp = (1.0f - g * g) / (1.0f + g - 2.0f * g * u);
    cos_theta = -(1.0f + g * g - tmp * tmp) / (2.0f * g);
  }
  const float phi = 2.0f * 3.14159265358979f * v;
  const float sin_theta = sqrtf(fmaxf(0.0f, 1.0f - cos_theta * cos_theta));
  float3 v1;
  if (fabsf(wo.x) > fabsf(wo.y)) {
    const float l = sqrtf(wo.x * wo.x + wo.z * wo.z);
    v1 = make_float3(-wo.z / l, 0.0f, wo.x / l);
  } else {
    const float l = sqrtf(wo.y * wo.y + wo.z * wo.z);
    v1 = make_float3(0.0f, wo.z / l, -wo.y / l);
  }
  const float3 v2 = make_float3(wo.y * v1.z - wo.z * v1.y, wo.z * v1.x - wo.x * v1.z, wo.x * v1.y - wo.y * v1.x);
  const float a = sin_theta * cosf(phi), b = sin_theta * sinf(phi);
  return make_float3(a * v1.x + b * v2.x + cos_theta * wo.x, a * v1.y + b * v2.y + cos_theta * wo.y,
                     a * v1.z + b * v2.z + cos_theta * wo.z);
}

// Philox stream of one tracking call of the volumetric path tracer: pixel,
// sample, bounce and purpose (0: free-flight sampling along the path,
// 1: transmittance of the shadow ray).
__device__ __host__ __forceinline__ uint64_t path_stream_id(int64_t pix, int s, int depth, int purpose) {
  return (uint64_t)pix | ((uint64_t)s << 26) | ((uint64_t)depth << 42) | ((uint64_t)purpose << 50);
}

}  // namespace flg
