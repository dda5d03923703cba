// Example caller of the live-renderer adapters of include/flg_accel.hpp:
// flg::GpuLBVH (Accel / Primitive::intersect) and flg::DenseGridVolume's
// Volume::tr / Volume::sample, over caller types with the reference's member
// names (Ray: m_o, m_d, mutable m_tMax; SInteraction: m_p, m_ns, m_ng, m_wo;
// VInteraction(p, wo, g); Sampler::get1D()).
// Usage: live_renderer_example <mesh.bin> <rays.bin> <grid.bin> <out.bin>
//   mesh.bin: int64 n_vert, int64 n_tri, int64 has_normals, 3 n_vert float32
//             positions, 3 n_tri int32 indices, [3 n_vert float32 normals]
//   rays.bin: int64 n, then 7 n float32 (ox oy oz dx dy dz tMax, SoA)
//   grid.bin: int32 res, then res^3 float32 densities over the unit box
//   out.bin:  accel: n uint8 hit, n float32 tMax, 12 n float32 (m_p, m_ng,
//             m_ns, m_wo per ray); one-ray calls on the first 64 rays agree
//             with the batch (else exit 6), also when 8 threads make them at
//             once on the first 512 rays, as the reference's tile-parallel
//             integrator does (else exit 7); volume: n float32 T of the batch
//             (seed 11), then for the first 256 rays: uint64 stream key,
//             float32 T of tr(ray, sampler), then uint64 key, uint8 success,
//             3 float32 position, float32 weight of sample(ray, sampler, ...)
#include <atomic>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "flg_accel.hpp"

struct Vec3 {
  float v[3] = {0, 0, 0};
  Vec3() = default;
  Vec3(float x, float y, float z) : v{x, y, z} {}
  float &operator[](int i) { return v[i]; }
  const float &operator[](int i) const { return v[i]; }
};
struct Ray {
  Vec3 m_o, m_d;
  mutable float m_tMax = 3.402823466e+38f;
};
struct SInteraction {
  Vec3 m_p, m_ns, m_ng, m_wo;
};
struct VInteraction {
  Vec3 m_p, m_ns, m_ng, m_wo;
  float m_g = 0.0f;
  VInteraction() = default;
  VInteraction(const Vec3 &p, const Vec3 &wo, float g) : m_p(p), m_wo(wo), m_g(g) {}
};
// A deterministic sampler: 24-bit uniforms from a 64-bit LCG.
struct Sampler {
  uint64_t s;
  explicit Sampler(uint64_t seed) : s(seed) {}
  float get1D() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (float)(s >> 40) * (1.0f / 16777216.0f);
  }
};

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
  if (argc != 5) return 2;
  std::vector<char> mb, rb, gb;
  if (!read_file(argv[1], mb) || !read_file(argv[2], rb) || !read_file(argv[3], gb)) return 3;
  const int64_t *mh = (const int64_t *)mb.data();
  const int64_t n_vert = mh[0], n_tri = mh[1], has_n = mh[2];
  const float *pos = (const float *)(mb.data() + 24);
  const int32_t *ind = (const int32_t *)(pos + 3 * n_vert);
  const float *nrm = has_n ? (const float *)(ind + 3 * n_tri) : nullptr;
  const int64_t n = *(const int64_t *)rb.data();
  const float *rs = (const float *)(rb.data() + 8);
  const int res = *(const int32_t *)gb.data();
  const float *rho = (const float *)(gb.data() + 4);
  std::vector<Ray> rays(n);
  for (int64_t i = 0; i < n; ++i) {
    rays[i].m_o = Vec3(rs[i], rs[n + i], rs[2 * n + i]);
    rays[i].m_d = Vec3(rs[3 * n + i], rs[4 * n + i], rs[5 * n + i]);
    rays[i].m_tMax = rs[6 * n + i];
  }
  std::vector<char> out;
  auto put = [&](const void *p, size_t bytes) { out.insert(out.end(), (const char *)p, (const char *)p + bytes); };
  try {
    flg::Context ctx(0);
    // ---- Accel ----
    flg::GpuLBVH<Ray, SInteraction> accel(ctx, pos, n_vert, ind, n_tri, nrm);
    const std::vector<Ray> rays0 = rays;  // before the batch shortens m_tMax
    std::vector<SInteraction> isect(n);
    std::unique_ptr<bool[]> hit(new bool[n]);
    accel.intersect(rays.data(), isect.data(), hit.get(), n);
    for (int64_t i = 0; i < 64 && i < n; ++i) {
      Ray r = rays0[i];
      SInteraction it;
      const bool h = accel.intersect(r, it);
      if (h != hit[i] || r.m_tMax != rays[i].m_tMax) return 6;
      if (h && std::memcmp(&it, &isect[i], sizeof(SInteraction)) != 0) return 6;
    }
    {
      std::atomic<int> bad{0};
      std::vector<std::thread> pool;
      const int64_t m = n < 512 ? n : 512;
      for (int w = 0; w < 8; ++w)
        pool.emplace_back([&, w] {
          for (int64_t i = w; i < m; i += 8) {
            Ray r = rays0[i];
            SInteraction it;
            const bool h = accel.intersect(r, it);
            if (h != hit[i] || r.m_tMax != rays[i].m_tMax ||
                (h && std::memcmp(&it, &isect[i], sizeof(SInteraction)) != 0))
              bad.fetch_add(1);
          }
        });
      for (auto &t : pool) t.join();
      if (bad.load() != 0) return 7;
    }
    for (int64_t i = 0; i < n; ++i) {
      const uint8_t b = hit[i] ? 1 : 0;
      put(&b, 1);
    }
    for (int64_t i = 0; i < n; ++i) put(&rays[i].m_tMax, 4);
    for (int64_t i = 0; i < n; ++i) {
      put(isect[i].m_p.v, 12);
      put(isect[i].m_ng.v, 12);
      put(isect[i].m_ns.v, 12);
      put(isect[i].m_wo.v, 12);
    }
    // ---- Volume ----
    float *d_rho = nullptr;
    flg::check_cuda(cudaMalloc(&d_rho, sizeof(float) * res * res * res), "cudaMalloc");
    flg::check_cuda(cudaMemcpy(d_rho, rho, sizeof(float) * res * res * res, cudaMemcpyHostToDevice), "copy grid");
    const float lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    flg_medium med{0.8f, 0.2f, 0.3f, 0.1f, 0.0f};
    {
      flg::DenseGridVolume vol(ctx, d_rho, res, res, res, lo, hi, med);
      std::vector<float> T(n);
      vol.tr(rays0.data(), n, 11, T.data());
      put(T.data(), 4 * n);
      for (int64_t i = 0; i < 256 && i < n; ++i) {
        Sampler s(1000 + i), s2(1000 + i);
        const uint64_t key = flg::stream_key(s2);
        Vec3 t = vol.tr(rays0[i], s);
        put(&key, 8);
        put(&t.v[0], 4);
        Sampler s3(5000 + i), s4(5000 + i);
        const uint64_t key2 = flg::stream_key(s4);
        VInteraction vi;
        bool ok = false;
        Vec3 w = vol.sample(rays0[i], s3, vi, ok);
        const uint8_t okb = ok ? 1 : 0;
        const Vec3 none;
        put(&key2, 8);
        put(&okb, 1);
        put(ok ? vi.m_p.v : none.v, 12);
        put(&w.v[0], 4);
      }
    }
    cudaFree(d_rho);
  } catch (const flg::Error &e) {
    std::fprintf(stderr, "flg error %d: %s\n", e.code, e.what());
    return 5;
  }
  FILE *f = std::fopen(argv[4], "wb");
  if (!f) return 4;
  std::fwrite(out.data(), 1, out.size(), f);
  std::fclose(f);
  return 0;
}
