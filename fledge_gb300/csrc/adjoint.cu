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

__device__ __forceinline__ void crossdf(const dfl *a, const dfl *b, dfl *r) {
  r[0] = df_sub(df_mul(a[1], b[2]), df_mul(a[2], b[1]));
  r[1] = df_sub(df_mul(a[2], b[0]), df_mul(a[0], b[2]));
  r[2] = df_sub(df_mul(a[0], b[1]), df_mul(a[1], b[0]));
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
  // The 3x3 solve runs in float-float arithmetic (common.cuh): for grazing
  // rays det M is small and a plain fp32 solve loses the digits the 1e-3
  // gradient bar needs; the edges p0-p1, p0-p2 are formed exactly.
  float pv[3][3];
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 3; ++a) pv[k][a] = pos[3 * vi[k] + a];
  const dfl c1[3] = {dfl{dx[i], 0.0f}, dfl{dy[i], 0.0f}, dfl{dz[i], 0.0f}};
  dfl c2[3], c3[3];
  for (int a = 0; a < 3; ++a) {
    c2[a] = two_sum(pv[0][a], -pv[1][a]);
    c3[a] = two_sum(pv[0][a], -pv[2][a]);
  }
  dfl x23[3], x31[3], x12[3];
  crossdf(c2, c3, x23);
  crossdf(c3, c1, x31);
  crossdf(c1, c2, x12);
  const dfl det = df_add(df_add(df_mul(c1[0], x23[0]), df_mul(c1[1], x23[1])), df_mul(c1[2], x23[2]));
  if (det.hi == 0.0f) return;
  float w[3];
  for (int a = 0; a < 3; ++a) {
    const dfl num = df_add(df_add(df_mulf(x23[a], g0), df_mulf(x31[a], g1)), df_mulf(x12[a], g2));
    const dfl q = df_div(num, det);
    w[a] = q.hi + q.lo;
  }
  const float u = hu[i], v = hv[i];
  const float b[3] = {1.0f - u - v, u, v};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    atomicAdd(grad + 3 * vi[k], b[k] * w[0]);
    atomicAdd(grad + 3 * vi[k] + 1, b[k] * w[1]);
    atomicAdd(grad + 3 * vi[k] + 2, b[k] * w[2]);
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

namespace flg {

// Normal of a fixed hit.  kind 0: the Pluecker test's Ng (intersector.hpp:
// 86-88), StableTriangleNormal of the ray-relative edges in fp32 and the
// Euclidean normalisation in double; kind 1: the live renderer's
// normalize(cross(p1 - p0, p2 - p0)) in fp32 (shape.cpp:141, vector.h:
// 364-404).  Same operation order as those functions; zeros on a miss.
__global__ void __launch_bounds__(256)
    k_hit_normals(const float *__restrict__ pos, const int32_t *__restrict__ idx, int64_t n_tri,
                  const float *__restrict__ ox, const float *__restrict__ oy, const float *__restrict__ oz,
                  int64_t n, const int32_t *__restrict__ prim, int kind, float *__restrict__ ng) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t p = prim[i];
  float3 N = make_float3(0.0f, 0.0f, 0.0f);
  if (p >= 0 && p < n_tri) {
    float3 a, b, c;
    tri_verts(pos, idx, p, a, b, c);
    if (kind == 0) {
      const float3 O = make_float3(ox[i], oy[i], oz[i]);
      const float3 v0 = f3sub(a, O), v1 = f3sub(b, O), v2 = f3sub(c, O);
      const float3 e0 = f3sub(v2, v0), e1 = f3sub(v0, v1), e2 = f3sub(v1, v2);
      const float ab_x = e0.z * e1.y, ab_y = e0.x * e1.z, ab_z = e0.y * e1.x;
      const float bc_x = e1.z * e2.y, bc_y = e1.x * e2.z, bc_z = e1.y * e2.x;
      float3 S;
      S.x = fabsf(ab_x) < fabsf(bc_x) ? e0.y * e1.z - ab_x : e1.y * e2.z - bc_x;
      S.y = fabsf(ab_y) < fabsf(bc_y) ? e0.z * e1.x - ab_y : e1.z * e2.x - bc_y;
      S.z = fabsf(ab_z) < fabsf(bc_z) ? e0.x * e1.y - ab_z : e1.x * e2.y - bc_z;
      const double x = S.x, y = S.y, z = S.z;
      const double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
      N = make_float3((float)__ddiv_rn(x, r), (float)__ddiv_rn(y, r), (float)__ddiv_rn(z, r));
    } else {
      const float3 C = f3cross(f3sub(b, a), f3sub(c, a));
      const float s = __fsqrt_rn(f3dot(C, C));
      N = make_float3(__fdiv_rn(C.x, s), __fdiv_rn(C.y, s), __fdiv_rn(C.z, s));
    }
  }
  ng[3 * i] = N.x;
  ng[3 * i + 1] = N.y;
  ng[3 * i + 2] = N.z;
}

}  // namespace flg

FLG_API int flg_hit_normals(flg_ctx ctx, flg_bvh bvh, const flg_rays *rays, int64_t n, const int32_t *prim,
                            int32_t kind, float *ng) {
  if (!ctx) return FLG_ERR_ARG;
  if (!bvh || !rays || !prim || !ng || n < 0) return set_error(ctx, FLG_ERR_ARG, "NULL argument or negative n");
  if (kind != FLG_NORMAL_PLUECKER && kind != FLG_NORMAL_GEOMETRIC)
    return set_error(ctx, FLG_ERR_ARG, "kind must be FLG_NORMAL_PLUECKER or FLG_NORMAL_GEOMETRIC");
  if (bvh->n_scenes != 1) return set_error(ctx, FLG_ERR_ARG, "batched handle: normals take one scene");
  if (kind == FLG_NORMAL_PLUECKER && (!rays->ox || !rays->oy || !rays->oz))
    return set_error(ctx, FLG_ERR_ARG, "ray origins are NULL");
  if (n == 0) return FLG_OK;
  k_hit_normals<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(bvh->pos, bvh->idx, bvh->n_tri, rays->ox,
                                                                      rays->oy, rays->oz, n, prim, kind, ng);
  FLG_LAUNCH_CHECK(ctx, "k_hit_normals");
  return FLG_OK;
}
