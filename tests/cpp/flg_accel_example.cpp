// Example caller of the C++ adapters (include/flg_accel.hpp): builds a BVH
// over a triangle soup read from a binary file, traces host BVHRayHit records
// (BVHBuilderBase::intersect shape) and writes prim/t/u/v/hit_ng to a binary
// file (hit_ns must equal hit_ng, as in the reference; else exit 6).
// Usage: flg_accel_example <tris.bin> <rays.bin> <out.bin>
//   tris.bin: int64 n_tri, then 9*n_tri float32
//   rays.bin: int64 n, then 8*n float32 (ox oy oz dx dy dz tnear tfar, SoA)
//   out.bin:  n int32 prim, then 3*n float32 (t, u, v), then 3*n float32
//             hit_ng (xyz per ray)
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "flg_accel.hpp"

static bool read_file(const char *path, std::vector<char> &buf) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf.resize(sz);
  bool ok = std::fread(buf.data(), 1, sz, f) == (size_t)sz;
  std::fclose(f);
  return ok;
}

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  std::vector<char> tb, rb;
  if (!read_file(argv[1], tb) || !read_file(argv[2], rb)) return 3;
  const int64_t n_tri = *(const int64_t *)tb.data();
  const float *tris = (const float *)(tb.data() + 8);
  const int64_t n = *(const int64_t *)rb.data();
  const float *rays = (const float *)(rb.data() + 8);
  try {
    flg::Context ctx(0);
    float *d_pos = nullptr;
    if (cudaMalloc(&d_pos, sizeof(float) * 9 * n_tri) != cudaSuccess) return 4;
    cudaMemcpy(d_pos, tris, sizeof(float) * 9 * n_tri, cudaMemcpyHostToDevice);
    flg::RadixBVHBuilder bvh(ctx, flg::DeviceMesh{d_pos, nullptr, n_tri, 3 * n_tri}, 4);
    bvh.build();
    ctx.sync();
    std::vector<flg::BVHRayHit> rh(n);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) {
        rh[i].ray_o[k] = rays[k * n + i];
        rh[i].ray_d[k] = rays[(3 + k) * n + i];
      }
      rh[i].tnear = rays[6 * n + i];
      rh[i].tfar = rays[7 * n + i];
    }
    bvh.intersect(rh.data(), n);
    std::vector<int32_t> prim(n);
    std::vector<float> tuv(3 * n), ng(3 * n);
    for (int64_t i = 0; i < n; ++i) {
      prim[i] = rh[i].prim;
      tuv[i] = rh[i].tfar;
      tuv[n + i] = rh[i].u;
      tuv[2 * n + i] = rh[i].v;
      for (int k = 0; k < 3; ++k) {
        ng[3 * i + k] = rh[i].hit_ng[k];
        if (rh[i].hit_ns[k] != rh[i].hit_ng[k]) return 6;
      }
    }
    FILE *f = std::fopen(argv[3], "wb");
    std::fwrite(prim.data(), sizeof(int32_t), n, f);
    std::fwrite(tuv.data(), sizeof(float), 3 * n, f);
    std::fwrite(ng.data(), sizeof(float), 3 * n, f);
    std::fclose(f);
    cudaFree(d_pos);
  } catch (const flg::Error &e) {
    std::fprintf(stderr, "flg error %d: %s\n", e.code, e.what());
    return 5;
  }
  return 0;
}
