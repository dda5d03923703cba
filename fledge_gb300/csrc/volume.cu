// volume.cu — participating media on a dense density grid:
//   k_volume_tr        ratio-tracking transmittance (OpenVDBVolume::tr,
//                      volume.cpp:75-107), one ray per thread, optional
//                      checkpoint of the state after the last roulette
//   k_volume_tr_adj    its adjoint with respect to the grid, replaying the
//                      ray's Philox stream from the checkpoint (or from the
//                      start) and scattering fp32 atomics into dL/dgrid
//   k_volume_sample    delta tracking (OpenVDBVolume::sample, :109-148)
// The grid is a vertex-centred lattice (x fastest) over the box; trilinear
// interpolation with background 0, the dense restatement of OpenVDB's
// tools::Sampler<1> lookups (volume.cpp:94,133).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace flg {

struct GridDev {
  const float *rho;
  int nx, ny, nz;
  float lo[3], hi[3], scale[3];
  float sigma_s, sigma_a, sigma_t, rr;
  const float *params;  // [0] majorant, [1] 1/majorant (double quotient as float)
};

struct VRays {
  const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
  float tmax_c;
};

__device__ __forceinline__ float gat(const GridDev &G, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= G.nx || y >= G.ny || z >= G.nz) return 0.0f;
  return __ldg(G.rho + ((int64_t)z * G.ny + y) * G.nx + x);
}

__device__ __forceinline__ float lerpf(float a, float b, float w) { return a + (b - a) * w; }

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
  float c00 = lerpf(gat(G, x, y, z), gat(G, x + 1, y, z), fx);
  float c10 = lerpf(gat(G, x, y + 1, z), gat(G, x + 1, y + 1, z), fx);
  float c01 = lerpf(gat(G, x, y, z + 1), gat(G, x + 1, y, z + 1), fx);
  float c11 = lerpf(gat(G, x, y + 1, z + 1), gat(G, x + 1, y + 1, z + 1), fx);
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

__device__ __forceinline__ void load_vray(const VRays &R, int64_t i, float3 &o, float3 &d, float &tmax) {
  o = make_float3(__ldg(R.ox + i), __ldg(R.oy + i), __ldg(R.oz + i));
  d = make_float3(__ldg(R.dx + i), __ldg(R.dy + i), __ldg(R.dz + i));
  tmax = R.tmax ? __ldg(R.tmax + i) : R.tmax_c;
}

// Ratio tracking of one ray; returns T and the state after the last
// roulette survival.
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
    float dens = sample_grid(G, o.x + d.x * t, o.y + d.y * t, o.z + d.z * t, x, y, z, fx, fy, fz);
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

__global__ void __launch_bounds__(256)
    k_volume_tr(GridDev G, VRays R, int64_t n, uint64_t seed, float *__restrict__ T, float *__restrict__ ck_t,
                uint32_t *__restrict__ ck_k, float *__restrict__ ck_c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float maj = __ldg(G.params), inv_maj = __ldg(G.params + 1);
  float3 o, d;
  float tmax;
  load_vray(R, i, o, d, tmax);
  float ct, cc;
  uint32_t ck;
  T[i] = ratio_track(G, maj, inv_maj, o, d, tmax, seed, i, ct, ck, cc);
  if (ck_t) {
    ck_t[i] = ct;
    ck_k[i] = ck;
    ck_c[i] = cc;
  }
}

// Adjoint: T = c * prod_{last segment} (1 - d_i/rho_max); with the majorant
// fixed, dT/drho_v = sum_i -T/(1 - d_i/rho_max) * w_iv / rho_max.
__global__ void __launch_bounds__(256)
    k_volume_tr_adj(GridDev G, VRays R, int64_t n, uint64_t seed, const float *__restrict__ dLdT,
                    const float *__restrict__ T, const float *__restrict__ ck_t, const uint32_t *__restrict__ ck_k,
                    float *__restrict__ grad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = __ldg(dLdT + i);
  const float Tf = __ldg(T + i);
  if (g == 0.0f || Tf == 0.0f) return;
  const float maj = __ldg(G.params), inv_maj = __ldg(G.params + 1);
  float3 o, d;
  float tmax;
  load_vray(R, i, o, d, tmax);
  float t;
  uint32_t k;
  if (ck_t) {
    t = __ldg(ck_t + i);
    k = __ldg(ck_k + i);
  } else {
    float cc;
    ratio_track(G, maj, inv_maj, o, d, tmax, seed, i, t, k, cc);
  }
  float t_min, t_max;
  if (!box_pbrt(G, o, d, tmax, t_min, t_max)) return;
  t_max = fminf(t_max, tmax);
  const float max_mu = G.sigma_t * maj;
  const float base = -g * Tf * inv_maj;
  RayStream rs;
  rs.init(seed, (uint64_t)i, k);
  for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
    float u = rs.next();
    t += -flg_logf(1.0f - u) / max_mu;
    if (t >= t_max) break;
    int x, y, z;
    float fx, fy, fz;
    float dens = sample_grid(G, o.x + d.x * t, o.y + d.y * t, o.z + d.z * t, x, y, z, fx, fy, fz);
    float xr = dens * inv_maj;
    if (!(xr > 0.0f)) continue;
    float coef = base / (1.0f - xr);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
      const int X = x + cx, Y = y + cy, Z = z + cz;
      if (X < 0 || Y < 0 || Z < 0 || X >= G.nx || Y >= G.ny || Z >= G.nz) continue;
      float w = (cx ? fx : 1.0f - fx) * (cy ? fy : 1.0f - fy) * (cz ? fz : 1.0f - fz);
      atomicAdd(grad + ((int64_t)Z * G.ny + Y) * G.nx + X, coef * w);
    }
  }
}

__global__ void __launch_bounds__(256)
    k_volume_sample(GridDev G, VRays R, int64_t n, uint64_t seed, uint8_t *__restrict__ success,
                    float *__restrict__ p, float *__restrict__ weight) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float maj = __ldg(G.params);
  float3 o, d;
  float tmax;
  load_vray(R, i, o, d, tmax);
  uint8_t ok = 0;
  float px = 0.0f, py = 0.0f, pz = 0.0f, w = 1.0f;
  float t_min, t_max;
  if (box_pbrt(G, o, d, tmax, t_min, t_max)) {
    float t = fmaxf(t_min, 0.0f);
    const float max_mu = G.sigma_t * maj;
    t_max = fminf(t_max, tmax);
    RayStream rs;
    rs.init(seed, (uint64_t)i, 0u);
    for (int step_ = 0; step_ < kMaxTrackSteps; ++step_) {
      float u = rs.next();
      t += -flg_logf(1.0f - u) / max_mu;
      if (t >= t_max) break;
      float qx = o.x + d.x * t, qy = o.y + d.y * t, qz = o.z + d.z * t;
      int x, y, z;
      float fx, fy, fz;
      float dens = sample_grid(G, qx, qy, qz, x, y, z, fx, fy, fz);
      float p_s = G.sigma_s * dens / max_mu;
      float p_a = G.sigma_a * dens / max_mu;
      float p_n = 1.0f - p_s - p_a;
      if (rs.next() > p_n) {
        ok = 1;
        px = qx;
        py = qy;
        pz = qz;
        w = G.sigma_s / G.sigma_t;
        break;
      }
    }
  }
  success[i] = ok;
  p[3 * i] = px;
  p[3 * i + 1] = py;
  p[3 * i + 2] = pz;
  weight[i] = w;
}

__device__ __forceinline__ void atomic_max_nonneg(float *a, float v) {
  if (v >= 0.0f) atomicMax((int *)a, __float_as_int(v));
}

__global__ void k_grid_max(const float *__restrict__ rho, int64_t nv, float *params) {
  float m = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, rho[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(params, m);
}

__global__ void k_grid_inv(float *params) {
  // volume.cpp:55: 1.0 / m_maxDensity in double, stored as Float.
  params[1] = (float)(1.0 / (double)params[0]);
}

static GridDev grid_dev(flg_grid g) {
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
  return G;
}

static int vrays(flg_ctx ctx, const flg_rays *r, int64_t n, VRays &V) {
  if (!r) return set_error(ctx, FLG_ERR_ARG, "rays is NULL");
  if (n < 0) return set_error(ctx, FLG_ERR_ARG, "n < 0");
  if (n > 0 && (!r->ox || !r->oy || !r->oz || !r->dx || !r->dy || !r->dz))
    return set_error(ctx, FLG_ERR_ARG, "ray pointer is NULL");
  V = VRays{r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->tmax, r->tmax_const};
  return FLG_OK;
}

}  // namespace flg

using namespace flg;

FLG_API int flg_grid_create(flg_ctx ctx, const float *density, int32_t nx, int32_t ny, int32_t nz,
                            const float *lo, const float *hi, const flg_medium *medium, flg_grid *out) {
  if (!ctx || !out) return FLG_ERR_ARG;
  *out = nullptr;
  if (!density || !lo || !hi || !medium) return set_error(ctx, FLG_ERR_ARG, "NULL argument");
  if (nx < 2 || ny < 2 || nz < 2) return set_error(ctx, FLG_ERR_ARG, "grid needs at least 2 samples per axis");
  for (int k = 0; k < 3; ++k)
    if (!(hi[k] > lo[k])) return set_error(ctx, FLG_ERR_ARG, "empty box");
  if (!(medium->sigma_s >= 0.0f) || !(medium->sigma_a >= 0.0f) || !(medium->sigma_s + medium->sigma_a > 0.0f))
    return set_error(ctx, FLG_ERR_ARG, "sigma_s, sigma_a must be >= 0 with a positive sum");
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "grid creation allocates");
  flg_grid g = new flg_grid_t();
  g->ctx = ctx;
  g->rho = density;
  g->nx = nx;
  g->ny = ny;
  g->nz = nz;
  const int dims[3] = {nx, ny, nz};
  for (int k = 0; k < 3; ++k) {
    g->lo[k] = lo[k];
    g->hi[k] = hi[k];
    g->scale[k] = (float)(dims[k] - 1) / (hi[k] - lo[k]);
  }
  g->medium = *medium;
  g->sigma_t = medium->sigma_a + medium->sigma_s;  // volume.cpp:38
  cudaError_t e = cudaMalloc((void **)&g->d_params, 4 * sizeof(float));
  if (e != cudaSuccess) {
    delete g;
    cudaGetLastError();
    return set_error(ctx, FLG_ERR_OOM, "cudaMalloc failed");
  }
  cudaStream_t st = ctx->stream;
  if (medium->majorant > 0.0f) {
    float prm[4] = {medium->majorant, (float)(1.0 / (double)medium->majorant), 0.0f, 0.0f};
    e = cudaMemcpyAsync(g->d_params, prm, sizeof(prm), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  } else {
    e = cudaMemsetAsync(g->d_params, 0, 4 * sizeof(float), st);
    const int64_t nv = (int64_t)nx * ny * nz;
    if (e == cudaSuccess) {
      k_grid_max<<<grid_for(nv, 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(density, nv, g->d_params);
      k_grid_inv<<<1, 1, 0, st>>>(g->d_params);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) {
    cudaFree(g->d_params);
    delete g;
    return cuda_fail(ctx, e, "grid create");
  }
  *out = g;
  return FLG_OK;
}

FLG_API int flg_grid_destroy(flg_grid g) {
  if (!g) return FLG_OK;
  cudaFree(g->d_params);
  delete g;
  return FLG_OK;
}

FLG_API int flg_grid_majorant(flg_grid g, float *maj) {
  if (!g || !maj) return FLG_ERR_ARG;
  cudaError_t e = cudaMemcpyAsync(maj, g->d_params, sizeof(float), cudaMemcpyDeviceToHost, g->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->ctx->stream);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "majorant");
  return FLG_OK;
}

FLG_API int flg_volume_tr(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n, uint64_t seed, float *T,
                          const flg_tr_ckpt *ckpt) {
  if (!ctx || !grid) return FLG_ERR_ARG;
  VRays V;
  int rc = vrays(ctx, rays, n, V);
  if (rc) return rc;
  if (n > 0 && !T) return set_error(ctx, FLG_ERR_ARG, "T is NULL");
  if (ckpt && (!ckpt->t || !ckpt->k || !ckpt->c)) return set_error(ctx, FLG_ERR_ARG, "checkpoint array is NULL");
  if (n == 0) return FLG_OK;
  k_volume_tr<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(grid_dev(grid), V, n, seed, T,
                                                                    ckpt ? ckpt->t : nullptr,
                                                                    ckpt ? ckpt->k : nullptr,
                                                                    ckpt ? ckpt->c : nullptr);
  FLG_LAUNCH_CHECK(ctx, "k_volume_tr");
  return FLG_OK;
}

FLG_API int flg_volume_tr_adjoint(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n, uint64_t seed,
                                  const float *dLdT, const float *T, const flg_tr_ckpt *ckpt, float *grad) {
  if (!ctx || !grid) return FLG_ERR_ARG;
  VRays V;
  int rc = vrays(ctx, rays, n, V);
  if (rc) return rc;
  if (n > 0 && (!dLdT || !T || !grad)) return set_error(ctx, FLG_ERR_ARG, "NULL argument");
  if (ckpt && (!ckpt->t || !ckpt->k)) return set_error(ctx, FLG_ERR_ARG, "checkpoint array is NULL");
  if (n == 0) return FLG_OK;
  k_volume_tr_adj<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(grid_dev(grid), V, n, seed, dLdT, T,
                                                                        ckpt ? ckpt->t : nullptr,
                                                                        ckpt ? ckpt->k : nullptr, grad);
  FLG_LAUNCH_CHECK(ctx, "k_volume_tr_adj");
  return FLG_OK;
}

FLG_API int flg_volume_sample(flg_ctx ctx, flg_grid grid, const flg_rays *rays, int64_t n, uint64_t seed,
                              uint8_t *success, float *p, float *weight) {
  if (!ctx || !grid) return FLG_ERR_ARG;
  VRays V;
  int rc = vrays(ctx, rays, n, V);
  if (rc) return rc;
  if (n > 0 && (!success || !p || !weight)) return set_error(ctx, FLG_ERR_ARG, "NULL output");
  if (n == 0) return FLG_OK;
  k_volume_sample<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(grid_dev(grid), V, n, seed, success, p,
                                                                        weight);
  FLG_LAUNCH_CHECK(ctx, "k_volume_sample");
  return FLG_OK;
}
