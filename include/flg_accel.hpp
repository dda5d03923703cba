// flg_accel.hpp — header-only C++ adapters over the C ABI (flg.h), shaped
// like the reference's interfaces so an integrator can drop them in:
//
//   flg::RadixBVHBuilder  ~ BVHBuilderBase / RadixBVHBuilder
//                           (src/experimental/base_bvh.hpp:38-125,
//                            src/experimental/radix_bvh.hpp:32-84):
//                           build(), getBound(), intersect(BVHRayHit*, n)
//   flg::GpuLBVH<Ray, SInteraction>
//                         ~ Accel : Primitive of the live renderer
//                           (src/accel.hpp:12-54, src/primitive.hpp:26-72):
//                           getBound(), intersect(const Ray&, SInteraction&)
//   flg::DenseGridVolume  ~ Volume / OpenVDBVolume (src/volume.hpp:16-70):
//                           tr(const Ray&, Sampler&),
//                           sample(const Ray&, Sampler&, VInteraction&, bool&)
//
// The reference's calls take one ray; each adapter also takes arrays of rays
// (the form a wavefront integrator uses, and the only one that keeps a GPU
// busy: a one-ray call is one launch).  The templates bind to the caller's
// own Ray / SInteraction / VInteraction / Sampler types by member name, as the
// reference declares them (ray.h:126-128, interaction.hpp:44-80, sampler.h:
// 20-23), and to any 3-vector type constructible from three floats with
// operator[].  Errors throw flg::Error carrying the status and the context's
// message (the reference aborts instead, debug.hpp:60-69).  The reference's
// integrators call intersect / tr / sample from many threads at once
// (integrator.cpp:194-231): every adapter call holds its Context's mutex
// (calls share the context's stream and scratch and the adapter's staging
// buffers), so such calls are safe, one at a time per context; for
// throughput, batch the rays, or give threads their own contexts.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
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

inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(FLG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

class Context {
 public:
  explicit Context(int device = 0, void *stream = nullptr) { check(flg_ctx_create(device, stream, &h_)); }
  ~Context() { flg_ctx_destroy(h_); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  void sync() { check(flg_ctx_sync(h_), h_); }
  flg_ctx get() const { return h_; }
  cudaStream_t stream() const { return (cudaStream_t)flg_ctx_stream(h_); }
  // Held by every adapter call on this context: a context (its stream,
  // scratch and error word) serves one call at a time.
  std::mutex &mutex() const { return mu_; }

 private:
  flg_ctx h_ = nullptr;
  mutable std::mutex mu_;
};

// Device scratch owned by an adapter, grown on demand.
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  ~DeviceBuffer() { cudaFree(p_); }
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  void *reserve(size_t bytes) {
    if (bytes > cap_) {
      cudaFree(p_);
      p_ = nullptr;
      cap_ = 0;
      check_cuda(cudaMalloc(&p_, bytes), "cudaMalloc");
      cap_ = bytes;
    }
    return p_;
  }

 private:
  void *p_ = nullptr;
  size_t cap_ = 0;
};

// Rays and hits of one batch in device memory: 8 ray arrays (o, d, tmin,
// tmax), prim / t / u / v and 3 normal floats per ray, in one allocation.
struct Staging {
  DeviceBuffer buf;
  float *r = nullptr;
  int32_t *prim = nullptr;
  float *t = nullptr, *u = nullptr, *v = nullptr, *ng = nullptr;
  void reserve(int64_t n) {
    char *p = (char *)buf.reserve((size_t)n * 4 * (8 + 4 + 3));
    r = (float *)p;
    prim = (int32_t *)(p + (size_t)n * 32);
    t = (float *)(p + (size_t)n * 36);
    u = t + n;
    v = u + n;
    ng = v + n;
  }
  flg_rays rays(int64_t n) const { return {r, r + n, r + 2 * n, r + 3 * n, r + 4 * n, r + 5 * n, r + 6 * n, r + 7 * n, 0.f, 0.f}; }
  flg_hits hits() const { return {prim, t, u, v}; }
};

// Host ray/hit record: BVHBuilderBase::BVHRayHit (base_bvh.hpp:41-50) plus the
// primitive id and barycentrics the GPU path returns.
struct BVHRayHit {
  float ray_o[3] = {0, 0, 0};
  float ray_d[3] = {0, 0, 0};
  float tnear = 0.0f;
  float tfar = 3.402823466e+38f;
  float hit_ng[3] = {0, 0, 0};
  float hit_ns[3] = {0, 0, 0};
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
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    if (h_) {
      check(flg_bvh_rebuild(ctx_.get(), h_, mesh_.p), ctx_.get());
      return;
    }
    check(flg_bvh_build(ctx_.get(), mesh_.p, mesh_.ind, mesh_.n_tri, mesh_.n_vert, &opts_, &h_), ctx_.get());
  }

  // BVHBuilderBase::getBound: {lower xyz, upper xyz}
  std::array<float, 6> getBound() const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    flg_bvh_info info{};
    check(flg_bvh_info_get(h_, &info), ctx_.get());
    return {info.bound[0], info.bound[1], info.bound[2], info.bound[3], info.bound[4], info.bound[5]};
  }

  // Closest hit on device arrays.
  void intersect(const flg_rays &rays, int64_t n, flg_hits &out, const flg_trace_opts *opts = nullptr) const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    check(flg_trace_closest(ctx_.get(), h_, &rays, n, opts, &out), ctx_.get());
  }

  // Any hit on device arrays.
  void intersectP(const flg_rays &rays, int64_t n, uint8_t *occluded, const flg_trace_opts *opts = nullptr) const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    check(flg_trace_any(ctx_.get(), h_, &rays, n, opts, occluded), ctx_.get());
  }

  // BVHBuilderBase::intersect over host records (RadixBVHBuilder::intersect,
  // radix_bvh.cpp:26-30, 202-245): on a hit, sets hit, tfar, prim, u, v and
  // hit_ng = hit_ns = the Pluecker test's normal (FLG_NORMAL_PLUECKER: the
  // reference's arithmetic with the Euclidean norm where its StableNormalize
  // adds z for z*z); a miss leaves the record as it was, like the reference.
  // tnear is honoured as the ray's tmin.  Synchronous.
  void intersect(BVHRayHit *rh, int64_t n) const {
    if (n <= 0) return;
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    std::vector<float> soa(8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) {
        soa[k * n + i] = rh[i].ray_o[k];
        soa[(3 + k) * n + i] = rh[i].ray_d[k];
      }
      soa[6 * n + i] = rh[i].tnear;
      soa[7 * n + i] = rh[i].tfar;
    }
    stage_.reserve(n);
    cudaStream_t st = ctx_.stream();
    check_cuda(cudaMemcpyAsync(stage_.r, soa.data(), soa.size() * 4, cudaMemcpyHostToDevice, st), "copy rays");
    flg_rays r = stage_.rays(n);
    flg_hits h = stage_.hits();
    check(flg_trace_closest(ctx_.get(), h_, &r, n, nullptr, &h), ctx_.get());
    check(flg_hit_normals(ctx_.get(), h_, &r, n, stage_.prim, FLG_NORMAL_PLUECKER, stage_.ng), ctx_.get());
    std::vector<int32_t> prim(n);
    std::vector<float> tuvn(6 * (size_t)n);
    check_cuda(cudaMemcpyAsync(prim.data(), stage_.prim, 4 * (size_t)n, cudaMemcpyDeviceToHost, st), "copy hits");
    check_cuda(cudaMemcpyAsync(tuvn.data(), stage_.t, 24 * (size_t)n, cudaMemcpyDeviceToHost, st), "copy hits");
    ctx_.sync();
    const float *t = tuvn.data(), *u = t + n, *v = u + n, *ng = v + n;
    for (int64_t i = 0; i < n; ++i) {
      if (prim[i] < 0) continue;
      rh[i].hit = true;
      rh[i].prim = prim[i];
      rh[i].tfar = t[i];
      rh[i].u = u[i];
      rh[i].v = v[i];
      for (int k = 0; k < 3; ++k) rh[i].hit_ng[k] = rh[i].hit_ns[k] = ng[3 * i + k];
    }
  }

  flg_bvh get() const { return h_; }

 private:
  Context &ctx_;
  DeviceMesh mesh_;
  flg_build_opts opts_;
  flg_bvh h_ = nullptr;
  mutable Staging stage_;
};

// The live renderer's acceleration structure (Accel : Primitive, accel.hpp:
// 12-54, with every triangle a ShapePrimitive over Triangle::intersect,
// shape.cpp:100-148), on the GPU: a 2-wide LBVH over the whole mesh traced
// with the Moller-Trumbore test (flg_trace_opts.tri_test = 1).
// Ray needs m_o, m_d and a mutable m_tMax (ray.h:126-128); SInteraction needs
// m_p, m_ns, m_ng, m_wo (interaction.hpp:44-45).  The contract of
// Primitive::intersect (primitive.hpp:31-41, accel.cpp:12-15): a hit with
// 0 < t < ray.m_tMax shortens ray.m_tMax to t and fills isect
//   m_p  = ray(t) = m_o + m_d * t,  m_wo = -m_d,
//   m_ng = normalize(cross(p1 - p0, p2 - p0)) (FLG_NORMAL_GEOMETRIC),
//   m_ns = u n[i0] + v n[i1] + (1 - u - v) n[i2] with vertex normals (the
//          reference's weights, shape.cpp:142-145), else m_ng,
// and returns true; a miss leaves both untouched and returns false.  t is the
// hit distance refined to within 1e-5 of FP64 (the reference returns the fp32
// Moller-Trumbore value).  The mesh is copied to the device.
template <class Ray, class SInteraction>
class GpuLBVH {
 public:
  GpuLBVH(Context &ctx, const float *pos_host, int64_t n_vert, const int32_t *ind_host, int64_t n_tri,
          const float *normals_host = nullptr)
      : ctx_(ctx), n_tri_(n_tri), n_vert_(n_vert) {
    char *p = (char *)mesh_.reserve((size_t)n_vert * 12 + (size_t)n_tri * 12);
    d_pos_ = (float *)p;
    d_ind_ = (int32_t *)(p + (size_t)n_vert * 12);
    check_cuda(cudaMemcpy(d_pos_, pos_host, (size_t)n_vert * 12, cudaMemcpyHostToDevice), "copy positions");
    check_cuda(cudaMemcpy(d_ind_, ind_host, (size_t)n_tri * 12, cudaMemcpyHostToDevice), "copy indices");
    ind_.assign(ind_host, ind_host + 3 * n_tri);
    if (normals_host) normals_.assign(normals_host, normals_host + 3 * n_vert);
    flg_build_opts o{2, 1, 1, FLG_BUILDER_LBVH};
    check(flg_bvh_build(ctx_.get(), d_pos_, d_ind_, n_tri, n_vert, &o, &h_), ctx_.get());
  }
  ~GpuLBVH() { flg_bvh_destroy(h_); }
  GpuLBVH(const GpuLBVH &) = delete;
  GpuLBVH &operator=(const GpuLBVH &) = delete;

  // Primitive::getBound: {lower xyz, upper xyz}
  std::array<float, 6> getBound() const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    flg_bvh_info info{};
    check(flg_bvh_info_get(h_, &info), ctx_.get());
    return {info.bound[0], info.bound[1], info.bound[2], info.bound[3], info.bound[4], info.bound[5]};
  }

  // Primitive::intersect for one ray (one trace launch; prefer the batch).
  // prim (optional) receives the hit triangle's index, -1 on a miss, so that
  // a caller can set isect.m_primitive from its own primitive list.
  bool intersect(const Ray &ray, SInteraction &isect, int32_t *prim = nullptr) const {
    bool hit = false;
    intersect(&ray, &isect, &hit, 1, prim);
    return hit;
  }

  // Primitive::intersect for n rays: hit[i] as the one-ray call returns it;
  // prim_out (optional, n entries) the hit triangles.
  void intersect(const Ray *rays, SInteraction *isect, bool *hit, int64_t n, int32_t *prim_out = nullptr) const {
    if (n <= 0) return;
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    std::vector<float> soa(8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) {
        soa[k * n + i] = rays[i].m_o[k];
        soa[(3 + k) * n + i] = rays[i].m_d[k];
      }
      soa[6 * n + i] = 0.0f;  // the test itself requires 0 < t
      soa[7 * n + i] = rays[i].m_tMax;
    }
    stage_.reserve(n);
    cudaStream_t st = ctx_.stream();
    check_cuda(cudaMemcpyAsync(stage_.r, soa.data(), soa.size() * 4, cudaMemcpyHostToDevice, st), "copy rays");
    flg_rays r = stage_.rays(n);
    flg_hits h = stage_.hits();
    flg_trace_opts op{};
    op.tri_test = 1;
    check(flg_trace_closest(ctx_.get(), h_, &r, n, &op, &h), ctx_.get());
    check(flg_hit_normals(ctx_.get(), h_, &r, n, stage_.prim, FLG_NORMAL_GEOMETRIC, stage_.ng), ctx_.get());
    std::vector<int32_t> prim(n);
    std::vector<float> tuvn(6 * (size_t)n);
    check_cuda(cudaMemcpyAsync(prim.data(), stage_.prim, 4 * (size_t)n, cudaMemcpyDeviceToHost, st), "copy hits");
    check_cuda(cudaMemcpyAsync(tuvn.data(), stage_.t, 24 * (size_t)n, cudaMemcpyDeviceToHost, st), "copy hits");
    ctx_.sync();
    const float *t = tuvn.data(), *u = t + n, *v = u + n, *ng = v + n;
    using V = std::decay_t<decltype(isect[0].m_p)>;
    for (int64_t i = 0; i < n; ++i) {
      hit[i] = prim[i] >= 0;
      if (prim_out) prim_out[i] = prim[i];
      if (!hit[i]) continue;
      const Ray &ray = rays[i];
      const float th = t[i];
      ray.m_tMax = th;
      SInteraction &it = isect[i];
      it.m_p = V(ray.m_o[0] + ray.m_d[0] * th, ray.m_o[1] + ray.m_d[1] * th, ray.m_o[2] + ray.m_d[2] * th);
      it.m_wo = V(-ray.m_d[0], -ray.m_d[1], -ray.m_d[2]);
      it.m_ng = V(ng[3 * i], ng[3 * i + 1], ng[3 * i + 2]);
      if (!normals_.empty()) {
        const float *n0 = &normals_[3 * (size_t)ind_[3 * (size_t)prim[i]]];
        const float *n1 = &normals_[3 * (size_t)ind_[3 * (size_t)prim[i] + 1]];
        const float *n2 = &normals_[3 * (size_t)ind_[3 * (size_t)prim[i] + 2]];
        const float w = 1.0f - u[i] - v[i];
        it.m_ns = V(u[i] * n0[0] + v[i] * n1[0] + w * n2[0], u[i] * n0[1] + v[i] * n1[1] + w * n2[1],
                    u[i] * n0[2] + v[i] * n1[2] + w * n2[2]);
      } else {
        it.m_ns = it.m_ng;
      }
    }
  }

  flg_bvh get() const { return h_; }

 private:
  Context &ctx_;
  int64_t n_tri_, n_vert_;
  DeviceBuffer mesh_;
  float *d_pos_ = nullptr;
  int32_t *d_ind_ = nullptr;
  std::vector<int32_t> ind_;
  std::vector<float> normals_;
  flg_bvh h_ = nullptr;
  mutable Staging stage_;
};

// Philox stream key of a one-ray volume call, drawn from the caller's
// Sampler: two get1D() draws in [0, 1), 32 bits each.  The tracking draws of
// the call then come from stream (key, 0) instead of the sampler (whose
// dimension count would otherwise depend on the medium).
template <class Sampler>
inline uint64_t stream_key(Sampler &rng) {
  const double a = (double)rng.get1D(), b = (double)rng.get1D();
  const uint64_t hi = (uint64_t)(a * 4294967296.0) & 0xFFFFFFFFull;
  const uint64_t lo = (uint64_t)(b * 4294967296.0) & 0xFFFFFFFFull;
  return hi << 32 | lo;
}

class DenseGridVolume {
 public:
  DenseGridVolume(Context &ctx, const float *density, int nx, int ny, int nz, const float lo[3], const float hi[3],
                  const flg_medium &medium)
      : ctx_(ctx), g_(medium.g) {
    check(flg_grid_create(ctx.get(), density, nx, ny, nz, lo, hi, &medium, &h_), ctx.get());
  }
  ~DenseGridVolume() { flg_grid_destroy(h_); }
  DenseGridVolume(const DenseGridVolume &) = delete;
  DenseGridVolume &operator=(const DenseGridVolume &) = delete;

  // Volume::tr (ratio tracking) on device arrays: ray i draws from Philox
  // stream (seed, i).
  void tr(const flg_rays &rays, int64_t n, uint64_t seed, float *T, const flg_tr_ckpt *ckpt = nullptr) const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    check(flg_volume_tr(ctx_.get(), h_, &rays, n, seed, T, ckpt), ctx_.get());
  }
  // Volume::sample (delta tracking) on device arrays.
  void sample(const flg_rays &rays, int64_t n, uint64_t seed, uint8_t *success, float *p, float *weight) const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    check(flg_volume_sample(ctx_.get(), h_, &rays, n, seed, success, p, weight), ctx_.get());
  }
  void tr_adjoint(const flg_rays &rays, int64_t n, uint64_t seed, const float *dL_dT, const float *T,
                  const flg_tr_ckpt *ckpt, float *dL_dgrid) const {
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    check(flg_volume_tr_adjoint(ctx_.get(), h_, &rays, n, seed, dL_dT, T, ckpt, dL_dgrid), ctx_.get());
  }

  // Volume::tr for host rays (Ray: m_o, m_d, m_tMax), ray i on stream
  // (seed, i); T: n floats.  Synchronous.
  template <class Ray>
  void tr(const Ray *rays, int64_t n, uint64_t seed, float *T) const {
    if (n <= 0) return;
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    flg_rays r = upload(rays, n);
    float *dT = stage_.t;
    check(flg_volume_tr(ctx_.get(), h_, &r, n, seed, dT, nullptr), ctx_.get());
    check_cuda(cudaMemcpyAsync(T, dT, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx_.stream()), "copy T");
    ctx_.sync();
  }

  // Volume::tr(const Ray&, Sampler&) (volume.hpp:22): transmittance from the
  // ray's origin to ray(m_tMax), as a grey 3-vector; one launch per call.
  template <class Ray, class Sampler>
  auto tr(const Ray &ray, Sampler &rng) const -> std::decay_t<decltype(ray.m_o)> {
    using V = std::decay_t<decltype(ray.m_o)>;
    float T = 1.0f;
    tr(&ray, 1, stream_key(rng), &T);
    return V(T, T, T);
  }

  // Volume::sample(const Ray&, Sampler&, VInteraction&, bool&) (volume.hpp:
  // 23-24): on a real collision sets success, vi = VInteraction(p, -m_d, g)
  // and returns sigma_s / sigma_t; otherwise success = false and 1.
  template <class Ray, class Sampler, class VInteraction>
  auto sample(const Ray &ray, Sampler &rng, VInteraction &vi, bool &success) const
      -> std::decay_t<decltype(ray.m_o)> {
    using V = std::decay_t<decltype(ray.m_o)>;
    const uint64_t key = stream_key(rng);
    std::lock_guard<std::mutex> lock(ctx_.mutex());
    flg_rays r = upload(&ray, 1);
    uint8_t *ok = (uint8_t *)stage_.prim;
    check(flg_volume_sample(ctx_.get(), h_, &r, 1, key, ok, stage_.ng, stage_.u), ctx_.get());
    uint8_t okh = 0;
    float pw[4];
    cudaStream_t st = ctx_.stream();
    check_cuda(cudaMemcpyAsync(&okh, ok, 1, cudaMemcpyDeviceToHost, st), "copy sample");
    check_cuda(cudaMemcpyAsync(pw, stage_.ng, 12, cudaMemcpyDeviceToHost, st), "copy sample");
    check_cuda(cudaMemcpyAsync(pw + 3, stage_.u, 4, cudaMemcpyDeviceToHost, st), "copy sample");
    ctx_.sync();
    success = okh != 0;
    if (success) vi = VInteraction(V(pw[0], pw[1], pw[2]), V(-ray.m_d[0], -ray.m_d[1], -ray.m_d[2]), g_);
    return V(pw[3], pw[3], pw[3]);
  }

 private:
  template <class Ray>
  flg_rays upload(const Ray *rays, int64_t n) const {
    std::vector<float> soa(8 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) {
        soa[k * n + i] = rays[i].m_o[k];
        soa[(3 + k) * n + i] = rays[i].m_d[k];
      }
      soa[6 * n + i] = 0.0f;
      soa[7 * n + i] = rays[i].m_tMax;
    }
    stage_.reserve(n);
    check_cuda(cudaMemcpyAsync(stage_.r, soa.data(), soa.size() * 4, cudaMemcpyHostToDevice, ctx_.stream()),
               "copy rays");
    return stage_.rays(n);
  }

  Context &ctx_;
  float g_;
  flg_grid h_ = nullptr;
  mutable Staging stage_;
};

}  // namespace flg
