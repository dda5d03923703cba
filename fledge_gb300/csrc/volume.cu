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
#include "volume.cuh"

namespace flg {

struct VRays {
  const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
  float tmax_c;
};

__device__ __forceinline__ void load_vray(const VRays &R, int64_t i, float3 &o, float3 &d, float &tmax) {
  o = make_float3(__ldg(R.ox + i), __ldg(R.oy + i), __ldg(R.oz + i));
  d = make_float3(__ldg(R.dx + i), __ldg(R.dy + i), __ldg(R.dz + i));
  tmax = R.tmax ? __ldg(R.tmax + i) : R.tmax_c;
}

// The tracking kernels are latency-bound on dependent grid taps: they run at
// 4 CTAs per SM (64 registers, no spills), 32 % faster than at the 3 that 74
// registers allowed; 5 CTAs spill and lose again.
template <bool SP>
__global__ void __launch_bounds__(256, 4)
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
  T[i] = ratio_track<SP>(G, maj, inv_maj, o, d, tmax, seed, i, ct, ck, cc);
  if (ck_t) {
    ck_t[i] = ct;
    ck_k[i] = ck;
    ck_c[i] = cc;
  }
}

// Adjoint: T = c * prod_{last segment} (1 - d_i/rho_max); with the majorant
// fixed, dT/drho_v = sum_i -T/(1 - d_i/rho_max) * w_iv / rho_max.
template <bool SP>
__global__ void __launch_bounds__(256, 4)
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
    ratio_track<SP>(G, maj, inv_maj, o, d, tmax, seed, i, t, k, cc);
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
    float dens = sample_grid<SP>(G, o.x + d.x * t, o.y + d.y * t, o.z + d.z * t, x, y, z, fx, fy, fz);
    float xr = dens * inv_maj;
    if (!(xr > 0.0f)) continue;
    float coef = base / (1.0f - xr);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
      const int X = x + cx, Y = y + cy, Z = z + cz;
      if (X < 0 || Y < 0 || Z < 0 || X >= G.nx || Y >= G.ny || Z >= G.nz) continue;
      int64_t off = ((int64_t)Z * G.ny + Y) * G.nx + X;
      if (SP) {
        off = grid_voxel<true>(G, X, Y, Z);
        if (off < 0) continue;  // an empty brick of a sparse grid is not a parameter
      }
      float w = (cx ? fx : 1.0f - fx) * (cy ? fy : 1.0f - fy) * (cz ? fz : 1.0f - fz);
      atomicAdd(grad + off, coef * w);
    }
  }
}

template <bool SP>
__global__ void __launch_bounds__(256, 4)
    k_volume_sample(GridDev G, VRays R, int64_t n, uint64_t seed, uint8_t *__restrict__ success,
                    float *__restrict__ p, float *__restrict__ weight) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float maj = __ldg(G.params);
  float3 o, d;
  float tmax;
  load_vray(R, i, o, d, tmax);
  RayStream rs;
  rs.init(seed, (uint64_t)i, 0u);
  float3 q = make_float3(0.0f, 0.0f, 0.0f);
  const uint8_t ok = delta_track<SP>(G, maj, o, d, tmax, rs, q) ? 1 : 0;
  const float px = q.x, py = q.y, pz = q.z, w = ok ? G.sigma_s / G.sigma_t : 1.0f;
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

static int vrays(flg_ctx ctx, const flg_rays *r, int64_t n, VRays &V) {
  if (!r) return set_error(ctx, FLG_ERR_ARG, "rays is NULL");
  if (n < 0) return set_error(ctx, FLG_ERR_ARG, "n < 0");
  if (n > 0 && (!r->ox || !r->oy || !r->oz || !r->dx || !r->dy || !r->dz))
    return set_error(ctx, FLG_ERR_ARG, "ray pointer is NULL");
  V = VRays{r->ox, r->oy, r->oz, r->dx, r->dy, r->dz, r->tmax, r->tmax_const};
  return FLG_OK;
}

// Sparse grids.  One CTA of 128 threads per brick; a brick is kept when one
// of its voxels differs from +0 (background), and keeps its slot in brick
// order (k_brick_scan), so the layout is deterministic.
__global__ void k_brick_flags(const float *__restrict__ rho, int nx, int ny, int nz, int bnx, int bny,
                              int32_t *__restrict__ bidx) {
  const int64_t b = blockIdx.x;
  const int bx = (int)(b % bnx), by = (int)((b / bnx) % bny), bz = (int)(b / ((int64_t)bnx * bny));
  int any = 0;
  for (int v = threadIdx.x; v < kBrick * kBrick * kBrick; v += blockDim.x) {
    const int x = bx * kBrick + v % kBrick, y = by * kBrick + (v / kBrick) % kBrick, z = bz * kBrick + v / (kBrick * kBrick);
    if (x < nx && y < ny && z < nz && __float_as_uint(rho[((int64_t)z * ny + y) * nx + x]) != 0u) any = 1;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) bidx[b] = any;
}

// Exclusive scan of the 0/1 flags into slots (-1 for empty bricks), one CTA.
__global__ void k_brick_scan(int32_t *bidx, int64_t nb, int64_t *count) {
  __shared__ int64_t s_part[1024];
  const int t = threadIdx.x;
  const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
  const int64_t a = t * per, e = min(a + per, nb);
  int64_t c = 0;
  for (int64_t i = a; i < e; ++i) c += bidx[i];
  s_part[t] = c;
  __syncthreads();
  if (t == 0) {
    int64_t run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const int64_t x = s_part[i];
      s_part[i] = run;
      run += x;
    }
    *count = run;
  }
  __syncthreads();
  int64_t run = s_part[t];
  for (int64_t i = a; i < e; ++i) {
    const int32_t f = bidx[i];
    bidx[i] = f ? (int32_t)run : -1;
    run += f;
  }
}

__global__ void k_brick_copy(const float *__restrict__ rho, int nx, int ny, int nz, int bnx, int bny,
                             const int32_t *__restrict__ bidx, float *__restrict__ bricks) {
  const int64_t b = blockIdx.x;
  const int32_t slot = bidx[b];
  if (slot < 0) return;
  const int bx = (int)(b % bnx), by = (int)((b / bnx) % bny), bz = (int)(b / ((int64_t)bnx * bny));
  for (int v = threadIdx.x; v < kBrick * kBrick * kBrick; v += blockDim.x) {
    const int x = bx * kBrick + v % kBrick, y = by * kBrick + (v / kBrick) % kBrick, z = bz * kBrick + v / (kBrick * kBrick);
    const float val = (x < nx && y < ny && z < nz) ? rho[((int64_t)z * ny + y) * nx + x] : 0.0f;
    bricks[(int64_t)slot * (kBrick * kBrick * kBrick) + v] = val;
  }
}

}  // namespace flg

using namespace flg;

// Shared by the dense and the sparse constructors: rho holds nv values (the
// dense lattice, or the bricks), over which the majorant is taken.
static int grid_new(flg_ctx ctx, const float *density, int64_t nv, const int32_t *bidx, int64_t n_bricks,
                    int32_t nx, int32_t ny, int32_t nz, const float *lo, const float *hi, const flg_medium *medium,
                    flg_grid *out) {
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
  g->bidx = bidx;
  g->n_bricks = n_bricks;
  g->bnx = (nx + kBrick - 1) / kBrick;
  g->bny = (ny + kBrick - 1) / kBrick;
  g->bnz = (nz + kBrick - 1) / kBrick;
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
    if (e == cudaSuccess && nv > 0) {
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

FLG_API int flg_grid_create(flg_ctx ctx, const float *density, int32_t nx, int32_t ny, int32_t nz,
                            const float *lo, const float *hi, const flg_medium *medium, flg_grid *out) {
  return grid_new(ctx, density, (int64_t)nx * ny * nz, nullptr, 0, nx, ny, nz, lo, hi, medium, out);
}

FLG_API int flg_grid_create_sparse(flg_ctx ctx, const int32_t *brick_index, const float *bricks, int64_t n_bricks,
                                   int32_t nx, int32_t ny, int32_t nz, const float *lo, const float *hi,
                                   const flg_medium *medium, flg_grid *out) {
  if (!ctx) return FLG_ERR_ARG;
  if (!brick_index) return set_error(ctx, FLG_ERR_ARG, "brick_index is NULL");
  if (n_bricks < 0 || (n_bricks > 0 && !bricks)) return set_error(ctx, FLG_ERR_ARG, "bad brick array");
  static const float kNoBricks[1] = {0.0f};  // never read: every slot is -1
  return grid_new(ctx, n_bricks > 0 ? bricks : kNoBricks, n_bricks * kBrick * kBrick * kBrick, brick_index,
                  n_bricks, nx, ny, nz, lo, hi, medium, out);
}

FLG_API int flg_grid_sparsify(flg_ctx ctx, const float *density, int32_t nx, int32_t ny, int32_t nz,
                              int32_t *brick_index, float *bricks, int64_t max_bricks, int64_t *n_bricks) {
  if (!ctx || !n_bricks) return FLG_ERR_ARG;
  if (!density || !brick_index) return set_error(ctx, FLG_ERR_ARG, "NULL argument");
  if (nx < 1 || ny < 1 || nz < 1) return set_error(ctx, FLG_ERR_ARG, "bad grid size");
  if (ctx->capturing) return set_error(ctx, FLG_ERR_STATE, "sparsify reads its count back to the host");
  const int bnx = (nx + kBrick - 1) / kBrick, bny = (ny + kBrick - 1) / kBrick, bnz = (nz + kBrick - 1) / kBrick;
  const int64_t nb = (int64_t)bnx * bny * bnz;
  if (nb > ((int64_t)1 << 31) - 1) return set_error(ctx, FLG_ERR_UNSUPPORTED, "too many bricks");
  cudaStream_t st = ctx->stream;
  int64_t *d_count = nullptr;
  FLG_CUDA(ctx, cudaMalloc((void **)&d_count, sizeof(int64_t)));
  k_brick_flags<<<(unsigned)nb, kBrick * kBrick * kBrick / 4, 0, st>>>(density, nx, ny, nz, bnx, bny, brick_index);
  cudaError_t e = cudaGetLastError();
  ++ctx->launches;
  if (e == cudaSuccess) {
    k_brick_scan<<<1, 1024, 0, st>>>(brick_index, nb, d_count);
    e = cudaGetLastError();
    ++ctx->launches;
  }
  int64_t count = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&count, d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_count);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sparsify");
  *n_bricks = count;
  if (!bricks) return FLG_OK;  // counting call
  if (count > max_bricks) return set_error(ctx, FLG_ERR_ARG, "brick array too small (%lld bricks)", (long long)count);
  k_brick_copy<<<(unsigned)nb, kBrick * kBrick * kBrick / 4, 0, st>>>(density, nx, ny, nz, bnx, bny, brick_index,
                                                                       bricks);
  FLG_LAUNCH_CHECK(ctx, "k_brick_copy");
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
  auto *kern = grid->bidx ? k_volume_tr<true> : k_volume_tr<false>;
  kern<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(
      grid_dev(grid), V, n, seed, T, ckpt ? ckpt->t : nullptr, ckpt ? ckpt->k : nullptr, ckpt ? ckpt->c : nullptr);
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
  auto *kern = grid->bidx ? k_volume_tr_adj<true> : k_volume_tr_adj<false>;
  kern<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(
      grid_dev(grid), V, n, seed, dLdT, T, ckpt ? ckpt->t : nullptr, ckpt ? ckpt->k : nullptr, grad);
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
  auto *kern = grid->bidx ? k_volume_sample<true> : k_volume_sample<false>;
  kern<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(grid_dev(grid), V, n, seed, success, p, weight);
  FLG_LAUNCH_CHECK(ctx, "k_volume_sample");
  return FLG_OK;
}
