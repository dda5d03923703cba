// flg_accel.hpp — header-only C++ adapters over the C ABI (flg.h), shaped
// like the reference's interfaces so an integrator can drop them in:
//
//   flg::RadixBVHBuilder  ~ BVHBuilderBase / RadixBVHBuilder
//                           (src/experimental/base_bvh.hpp:38-125,
//                            src/experimental/radix_bvh.hpp:32-84):
//                           build(), getBound(), intersect(BVHRayHit*, n)
//   flg::DenseGridVolume  ~ Volume / OpenVDBVolume (src/volume.hpp:16-70):
//                           tr(), sample()
//
// The reference's calls take one ray; these take arrays of rays (device
// pointers, or host BVHRayHit records staged through flg_trace_closest_host).
// Errors throw flg::Error carrying the status and the context's message.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "flg.h"

namespace flg {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &msg) : std::runtime_error(msg), code(code) {}
  int code;
};

inline void check(int rc, flg_ctx ctx = nullptr) {
  if (rc == FLG_OK) return;
  std::string msg = flg_status_string(rc);
  if (ctx) {
    char buf[512];
    flg_ctx_last_error(ctx, buf, sizeof(buf));
    if (buf[0]) msg += std::string(": ") + buf;
  }
  throw Error(rc, msg);
}

class Context {
 public:
  explicit Context(int device = 0, void *stream = nullptr) { check(flg_ctx_create(device, stream, &h_)); }
  ~Context() { flg_ctx_destroy(h_); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  void sync() { check(flg_ctx_sync(h_), h_); }
  flg_ctx get() const { return h_; }

 private:
  flg_ctx h_ = nullptr;
};

// Host ray/hit record: BVHBuilderBase::BVHRayHit (base_bvh.hpp:41-50) plus the
// primitive id and barycentrics the GPU path returns.
struct BVHRayHit {
  float ray_o[3] = {0, 0, 0};
  float ray_d[3] = {0, 0, 0};
  float tnear = 0.0f;
  float tfar = 3.402823466e+38f;
  bool hit = false;
  int32_t prim = -1;
  float u = 0.0f, v = 0.0f;
};

// Mesh arrays on the device (InternalTriangleMesh, base_bvh.hpp:26-31).
struct DeviceMesh {
  const float *p = nullptr;     // 3 * n_vert
  const int32_t *ind = nullptr; // 3 * n_tri or nullptr (soup)
  int64_t n_tri = 0, n_vert = 0;
};

class RadixBVHBuilder {
 public:
  // builder: FLG_BUILDER_LBVH (the Karras radix tree), FLG_BUILDER_PLOC or FLG_BUILDER_SAH.
  RadixBVHBuilder(Context &ctx, const DeviceMesh &mesh, int node_width = 4, int leaf_size = 1,
                  int builder = FLG_BUILDER_LBVH)
      : ctx_(ctx), mesh_(mesh), opts_{node_width, leaf_size, 1, builder} {}
  ~RadixBVHBuilder() { flg_bvh_destroy(h_); }
  RadixBVHBuilder(const RadixBVHBuilder &) = delete;
  RadixBVHBuilder &operator=(const RadixBVHBuilder &) = delete;

  // BVHBuilderBase::build
  void build() {
    if (h_) {
      check(flg_bvh_rebuild(ctx_.get(), h_, mesh_.p), ctx_.get());
      return;
    }
    check(flg_bvh_build(ctx_.get(), mesh_.p, mesh_.ind, mesh_.n_tri, mesh_.n_vert, &opts_, &h_), ctx_.get());
  }

  // BVHBuilderBase::getBound: {lower xyz, upper xyz}
  std::vector<float> getBound() const {
    flg_bvh_info info{};
    check(flg_bvh_info_get(h_, &info), ctx_.get());
    return std::vector<float>(info.bound, info.bound + 6);
  }

  // Closest hit on device arrays.
  void intersect(const flg_rays &rays, int64_t n, flg_hits &out, const flg_trace_opts *opts = nullptr) {
    check(flg_trace_closest(ctx_.get(), h_, &rays, n, opts, &out), ctx_.get());
  }

  // Any hit on device arrays.
  void intersectP(const flg_rays &rays, int64_t n, uint8_t *occluded, const flg_trace_opts *opts = nullptr) {
    check(flg_trace_any(ctx_.get(), h_, &rays, n, opts, occluded), ctx_.get());
  }

  // BVHBuilderBase::intersect over host records: fills tfar, hit, prim, u, v
  // (tfar is left unchanged on a miss, like the reference).
  void intersect(BVHRayHit *rh, int64_t n) {
    std::vector<float> soa(8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) {
        soa[k * n + i] = rh[i].ray_o[k];
        soa[(3 + k) * n + i] = rh[i].ray_d[k];
      }
      soa[6 * n + i] = rh[i].tnear;
      soa[7 * n + i] = rh[i].tfar;
    }
    std::vector<int32_t> prim(n);
    std::vector<float> t(n), u(n), v(n);
    flg_rays r{&soa[0], &soa[n], &soa[2 * n], &soa[3 * n], &soa[4 * n], &soa[5 * n], &soa[6 * n], &soa[7 * n],
               0.0f, 0.0f};
    flg_hits h{prim.data(), t.data(), u.data(), v.data()};
    check(flg_trace_closest_host(ctx_.get(), h_, &r, n, nullptr, &h), ctx_.get());
    for (int64_t i = 0; i < n; ++i) {
      rh[i].hit = prim[i] >= 0;
      rh[i].prim = prim[i];
      if (rh[i].hit) {
        rh[i].tfar = t[i];
        rh[i].u = u[i];
        rh[i].v = v[i];
      }
    }
  }

  flg_bvh get() const { return h_; }

 private:
  Context &ctx_;
  DeviceMesh mesh_;
  flg_build_opts opts_;
  flg_bvh h_ = nullptr;
};

class DenseGridVolume {
 public:
  DenseGridVolume(Context &ctx, const float *density, int nx, int ny, int nz, const float lo[3], const float hi[3],
                  const flg_medium &medium)
      : ctx_(ctx) {
    check(flg_grid_create(ctx.get(), density, nx, ny, nz, lo, hi, &medium, &h_), ctx.get());
  }
  ~DenseGridVolume() { flg_grid_destroy(h_); }
  DenseGridVolume(const DenseGridVolume &) = delete;
  DenseGridVolume &operator=(const DenseGridVolume &) = delete;

  // Volume::tr (ratio tracking), one Philox stream per ray.
  void tr(const flg_rays &rays, int64_t n, uint64_t seed, float *T, const flg_tr_ckpt *ckpt = nullptr) {
    check(flg_volume_tr(ctx_.get(), h_, &rays, n, seed, T, ckpt), ctx_.get());
  }
  // Volume::sample (delta tracking).
  void sample(const flg_rays &rays, int64_t n, uint64_t seed, uint8_t *success, float *p, float *weight) {
    check(flg_volume_sample(ctx_.get(), h_, &rays, n, seed, success, p, weight), ctx_.get());
  }
  void tr_adjoint(const flg_rays &rays, int64_t n, uint64_t seed, const float *dL_dT, const float *T,
                  const flg_tr_ckpt *ckpt, float *dL_dgrid) {
    check(flg_volume_tr_adjoint(ctx_.get(), h_, &rays, n, seed, dL_dT, T, ckpt, dL_dgrid), ctx_.get());
  }

 private:
  Context &ctx_;
  flg_grid h_ = nullptr;
};

}  // namespace flg
