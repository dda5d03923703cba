// gen.cu — seeded synthetic workloads, generated on the device from Philox
// streams: random triangle soups, rays aimed into the unit cube from a
// sphere, and a 4-octave value-noise density lattice.
#include "common.cuh"
#include "internal.h"

namespace flg {

__device__ __forceinline__ float4 u4(uint64_t seed, uint32_t a, uint32_t b, uint32_t tag, uint32_t j) {
  uint4 r = philox4x32_10(make_uint4(a, b, tag, j), (uint32_t)seed, (uint32_t)(seed >> 32));
  return make_float4(u01(r.x), u01(r.y), u01(r.z), u01(r.w));
}

// Triangle i: centroid U[0,1]^3, each vertex centroid + U[-h,h]^3.
__global__ void k_gen_triangles(uint64_t seed, int64_t first, int64_t n, float h, float *__restrict__ pos) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t g = (uint64_t)(first + i);
  const float4 a = u4(seed, (uint32_t)g, (uint32_t)(g >> 32), 0x7415u, 0u);
  const float4 b = u4(seed, (uint32_t)g, (uint32_t)(g >> 32), 0x7415u, 1u);
  const float4 c = u4(seed, (uint32_t)g, (uint32_t)(g >> 32), 0x7415u, 2u);
  const float r[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
  float *o = pos + 9 * i;
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) o[3 * k + ax] = r[ax] + (2.0f * r[3 + 3 * k + ax] - 1.0f) * h;
}

// Ray r: origin center + radius * s, s uniform on the unit sphere
// (z = 1 - 2u, phi = 2 pi u'); direction normalised toward U[0,1]^3.
__global__ void k_gen_rays(uint64_t seed, int64_t first, int64_t n, float cx, float cy, float cz, float radius,
                           float *__restrict__ ox, float *__restrict__ oy, float *__restrict__ oz,
                           float *__restrict__ dx, float *__restrict__ dy, float *__restrict__ dz) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t g = (uint64_t)(first + i);
  const float4 a = u4(seed, (uint32_t)g, (uint32_t)(g >> 32), 0x7a75u, 0u);
  const float4 b = u4(seed, (uint32_t)g, (uint32_t)(g >> 32), 0x7a75u, 1u);
  const float z = 1.0f - 2.0f * a.x;
  const float phi = 6.283185307179586f * a.y;
  const float s = sqrtf(fmaxf(0.0f, 1.0f - z * z));
  float sp, cp;
  sincosf(phi, &sp, &cp);
  const float px = cx + radius * s * cp, py = cy + radius * s * sp, pz = cz + radius * z;
  const float tx = a.z - px, ty = a.w - py, tz = b.x - pz;
  const float inv = 1.0f / sqrtf(tx * tx + ty * ty + tz * tz);
  ox[i] = px;
  oy[i] = py;
  oz[i] = pz;
  dx[i] = tx * inv;
  dy[i] = ty * inv;
  dz[i] = tz * inv;
}

__device__ __forceinline__ float lattice(uint64_t seed, int x, int y, int z, int o) {
  uint4 r = philox4x32_10(make_uint4((uint32_t)x, (uint32_t)y, (uint32_t)z, 0x4e00u + (uint32_t)o),
                          (uint32_t)seed, (uint32_t)(seed >> 32));
  return 2.0f * u01(r.x) - 1.0f;
}

__device__ __forceinline__ float smooth(float t) { return t * t * (3.0f - 2.0f * t); }

// Value noise: lattice values in [-1,1], smoothstep-trilinear; 4 octaves of
// frequency 4 * 2^o and amplitude 2^-o, normalised; mapped to [0, scale].
__global__ void k_gen_noise(uint64_t seed, int nx, int ny, int nz, float scale, float *__restrict__ rho) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nv = (int64_t)nx * ny * nz;
  if (i >= nv) return;
  const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
  const float p[3] = {(float)x / (float)(nx - 1), (float)y / (float)(ny - 1), (float)z / (float)(nz - 1)};
  float acc = 0.0f, norm = 0.0f, amp = 1.0f, freq = 4.0f;
  for (int o = 0; o < 4; ++o) {
    float q[3], f[3];
    int b[3];
    for (int k = 0; k < 3; ++k) {
      q[k] = p[k] * freq;
      float fl = floorf(q[k]);
      b[k] = (int)fl;
      f[k] = smooth(q[k] - fl);
    }
    float v = 0.0f;
    for (int c = 0; c < 8; ++c) {
      const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
      const float w = (cx ? f[0] : 1.0f - f[0]) * (cy ? f[1] : 1.0f - f[1]) * (cz ? f[2] : 1.0f - f[2]);
      v += w * lattice(seed, b[0] + cx, b[1] + cy, b[2] + cz, o);
    }
    acc += amp * v;
    norm += amp;
    amp *= 0.5f;
    freq *= 2.0f;
  }
  const float nval = acc / norm;
  rho[i] = scale * fminf(1.0f, fmaxf(0.0f, 0.5f * (nval + 1.0f)));
}

}  // namespace flg

using namespace flg;

FLG_API int flg_gen_triangles(flg_ctx ctx, uint64_t seed, int64_t first_tri, int64_t n_tri, float half_extent,
                              float *pos) {
  if (!ctx) return FLG_ERR_ARG;
  if (n_tri < 0 || first_tri < 0 || (n_tri > 0 && !pos)) return set_error(ctx, FLG_ERR_ARG, "bad argument");
  if (n_tri == 0) return FLG_OK;
  k_gen_triangles<<<(unsigned)ceil_div(n_tri, 256), 256, 0, ctx->stream>>>(seed, first_tri, n_tri, half_extent, pos);
  FLG_LAUNCH_CHECK(ctx, "k_gen_triangles");
  return FLG_OK;
}

FLG_API int flg_gen_rays(flg_ctx ctx, uint64_t seed, int64_t first_ray, int64_t n, const float *c, float radius,
                         float *ox, float *oy, float *oz, float *dx, float *dy, float *dz) {
  if (!ctx) return FLG_ERR_ARG;
  if (n < 0 || first_ray < 0 || !c || (n > 0 && (!ox || !oy || !oz || !dx || !dy || !dz)))
    return set_error(ctx, FLG_ERR_ARG, "bad argument");
  if (n == 0) return FLG_OK;
  k_gen_rays<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(seed, first_ray, n, c[0], c[1], c[2], radius, ox, oy,
                                                                   oz, dx, dy, dz);
  FLG_LAUNCH_CHECK(ctx, "k_gen_rays");
  return FLG_OK;
}

FLG_API int flg_gen_noise_grid(flg_ctx ctx, uint64_t seed, int32_t nx, int32_t ny, int32_t nz, float scale,
                               float *rho) {
  if (!ctx) return FLG_ERR_ARG;
  if (nx < 2 || ny < 2 || nz < 2 || !rho) return set_error(ctx, FLG_ERR_ARG, "bad argument");
  const int64_t nv = (int64_t)nx * ny * nz;
  k_gen_noise<<<(unsigned)ceil_div(nv, 256), 256, 0, ctx->stream>>>(seed, nx, ny, nz, scale, rho);
  FLG_LAUNCH_CHECK(ctx, "k_gen_noise");
  return FLG_OK;
}
