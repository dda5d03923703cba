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

__device__ __forceinline__ double3 crossd(double3 a, double3 b) {
  return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
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
  // The 3x3 solve runs in double precision: for grazing rays det M is small
  // and an fp32 solve loses the digits the 1e-3 gradient bar needs.  It is
  // one solve per hit, negligible next to the traversal.
  const double3 p0 = make_double3(pos[3 * vi[0]], pos[3 * vi[0] + 1], pos[3 * vi[0] + 2]);
  const double3 p1 = make_double3(pos[3 * vi[1]], pos[3 * vi[1] + 1], pos[3 * vi[1] + 2]);
  const double3 p2 = make_double3(pos[3 * vi[2]], pos[3 * vi[2] + 1], pos[3 * vi[2] + 2]);
  const double3 c1 = make_double3(dx[i], dy[i], dz[i]);
  const double3 c2 = make_double3(p0.x - p1.x, p0.y - p1.y, p0.z - p1.z);
  const double3 c3 = make_double3(p0.x - p2.x, p0.y - p2.y, p0.z - p2.z);
  const double3 x23 = crossd(c2, c3), x31 = crossd(c3, c1), x12 = crossd(c1, c2);
  const double det = c1.x * x23.x + c1.y * x23.y + c1.z * x23.z;
  if (det == 0.0) return;
  const double w[3] = {(x23.x * g0 + x31.x * g1 + x12.x * g2) / det, (x23.y * g0 + x31.y * g1 + x12.y * g2) / det,
                       (x23.z * g0 + x31.z * g1 + x12.z * g2) / det};
  const double u = hu[i], v = hv[i];
  const double b[3] = {1.0 - u - v, u, v};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    atomicAdd(grad + 3 * vi[k], (float)(b[k] * w[0]));
    atomicAdd(grad + 3 * vi[k] + 1, (float)(b[k] * w[1]));
    atomicAdd(grad + 3 * vi[k] + 2, (float)(b[k] * w[2]));
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
