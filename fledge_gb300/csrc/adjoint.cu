// adjoint.cu — gradient of a fixed hit's (t, u, v) with respect to the three
// triangle vertices (no counterpart in the reference).
//
// With P = O + tD = (1-u-v) p0 + u p1 + v p2, a perturbation of the vertices
// satisfies M [dt, du, dv]^T = sum_k b_k dp_k with M = [D, -(p1-p0), -(p2-p0)]
// and b = (1-u-v, u, v).  Hence dL/dp_k = b_k M^{-T} (dL/dt, dL/du, dL/dv),
// and M^{-T} g = ((c2 x c3) g_t + (c3 x c1) g_u + (c1 x c2) g_v) / det M for
// the columns c1, c2, c3 of M.
#include "common.cuh"
#include "internal.h"

namespace flg {

__device__ __forceinline__ float3 crossf(float3 a, float3 b) {
  return make_float3(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}

__global__ void __launch_bounds__(256)
    k_hit_adjoint(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
                  const float *__restrict__ dx, const float *__restrict__ dy, const float *__restrict__ dz,
                  int64_t n, const int32_t *__restrict__ prim, const float *__restrict__ hu,
                  const float *__restrict__ hv, const float *__restrict__ gt, const float *__restrict__ gu,
                  const float *__restrict__ gv, float *__restrict__ grad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t p = prim[i];
  if (p < 0 || p >= n_tri) return;
  const float g0 = gt ? gt[i] : 0.0f, g1 = gu ? gu[i] : 0.0f, g2 = gv ? gv[i] : 0.0f;
  if (g0 == 0.0f && g1 == 0.0f && g2 == 0.0f) return;
  int64_t vi[3];
  for (int k = 0; k < 3; ++k) vi[k] = idx ? (int64_t)idx[3 * (int64_t)p + k] : 3 * (int64_t)p + k;
  const float3 p0 = make_float3(pos[3 * vi[0]], pos[3 * vi[0] + 1], pos[3 * vi[0] + 2]);
  const float3 p1 = make_float3(pos[3 * vi[1]], pos[3 * vi[1] + 1], pos[3 * vi[1] + 2]);
  const float3 p2 = make_float3(pos[3 * vi[2]], pos[3 * vi[2] + 1], pos[3 * vi[2] + 2]);
  const float3 c1 = make_float3(dx[i], dy[i], dz[i]);
  const float3 c2 = make_float3(p0.x - p1.x, p0.y - p1.y, p0.z - p1.z);
  const float3 c3 = make_float3(p0.x - p2.x, p0.y - p2.y, p0.z - p2.z);
  const float3 x23 = crossf(c2, c3), x31 = crossf(c3, c1), x12 = crossf(c1, c2);
  const float det = fmaf(c1.x, x23.x, fmaf(c1.y, x23.y, c1.z * x23.z));
  if (det == 0.0f) return;
  const float r = 1.0f / det;
  const float3 w = make_float3(fmaf(x23.x, g0, fmaf(x31.x, g1, x12.x * g2)) * r,
                               fmaf(x23.y, g0, fmaf(x31.y, g1, x12.y * g2)) * r,
                               fmaf(x23.z, g0, fmaf(x31.z, g1, x12.z * g2)) * r);
  const float u = hu[i], v = hv[i];
  const float b[3] = {1.0f - u - v, u, v};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    atomicAdd(grad + 3 * vi[k], b[k] * w.x);
    atomicAdd(grad + 3 * vi[k] + 1, b[k] * w.y);
    atomicAdd(grad + 3 * vi[k] + 2, b[k] * w.z);
  }
}

}  // namespace flg

using namespace flg;

FLG_API int flg_hit_adjoint(flg_ctx ctx, const float *pos, const int32_t *idx, int64_t n_tri, int64_t n_vert,
                            const flg_rays *rays, int64_t n, const flg_hits *hits, const float *dL_dt,
                            const float *dL_du, const float *dL_dv, float *dL_dpos) {
  if (!ctx) return FLG_ERR_ARG;
  if (!rays || !hits || n < 0 || n_tri < 0) return set_error(ctx, FLG_ERR_ARG, "bad argument");
  if (n == 0) return FLG_OK;
  if (!pos || !dL_dpos || !rays->dx || !rays->dy || !rays->dz || !hits->prim || !hits->u || !hits->v)
    return set_error(ctx, FLG_ERR_ARG, "NULL pointer");
  if (!idx && n_vert != 3 * n_tri) return set_error(ctx, FLG_ERR_ARG, "soup needs n_vert == 3*n_tri");
  k_hit_adjoint<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(pos, idx, n_tri, rays->dx, rays->dy, rays->dz,
                                                                      n, hits->prim, hits->u, hits->v, dL_dt, dL_du,
                                                                      dL_dv, dL_dpos);
  FLG_LAUNCH_CHECK(ctx, "k_hit_adjoint");
  return FLG_OK;
}
