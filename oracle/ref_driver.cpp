// ref_driver.cpp — builds the reference's own Karras LBVH (RadixBVHBuilder,
// src/experimental/radix_bvh.cpp of the fledge project) and its live
// renderer's triangle test (Triangle::intersect, src/shape.cpp:100-148), and
// exposes their results through a C ABI, so that tests can check the oracle
// against the reference's code on the same inputs.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `ref`) into
// oracle/_ref/libfledge_ref.so, and only where the reference sources exist.
// The reference file is compiled unchanged, as one translation unit with this
// driver (its headers define non-inline functions), together with
// src/shape.cpp and src/interaction.cpp (whose SInteraction the triangle test
// fills), against the stand-in headers under oracle/refshim/ for oneTBB, fmt,
// Embree, miniply and boost::container::flat_map:
//   - tbb::parallel_for / parallel_reduce run sequentially; tbb::parallel_sort
//     is std::stable_sort, so equal Morton codes keep their input (triangle
//     index) order, where TBB leaves the order unspecified;
//   - tbb::cache_aligned_resource returns zero-filled memory: the reference
//     allocates its nodes without constructing them (radix_bvh.cpp:37-40) and
//     its refit counts arrivals in their `flag` words;
//   - fmt calls print nothing; no Embree or miniply function is referenced;
//     flat_map (the Resource arena's destructor registry) is a std::map.
// Nothing here changes the arithmetic of the reference's build or traversal.
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <memory_resource>
#include <vector>

#include "experimental/radix_bvh.cpp"
#include "interaction.cpp"
#include "shape.cpp"

namespace {
using fledge::Vector3f;
using fledge::experimental::InternalTriangleMesh;
using fledge::experimental::RadixBVHBuilder;

// Exposes the builder's protected arrays (radix_bvh.hpp:75-78).
struct Probe : RadixBVHBuilder {
  using RadixBVHBuilder::RadixBVHBuilder;
  using RadixBVHBuilder::m_bound;
  using RadixBVHBuilder::m_internal_nodes;
  using RadixBVHBuilder::m_n_triangles;
  using RadixBVHBuilder::m_triangles;
};

struct Handle {
  std::vector<Vector3f> p;
  std::vector<int> ind;
  InternalTriangleMesh mesh{};
  Probe *builder = nullptr;
};
}  // namespace

extern "C" {

// Builds the reference LBVH over pos (3 * n_vert floats) and ind (3 * n_tri
// vertex indices, or NULL for a soup with n_vert = 3 n_tri).  n_tri >= 2 (the
// reference reads an unset parent for a single triangle).
void *ref_radix_build(const float *pos, int32_t n_vert, const int32_t *ind, int32_t n_tri) {
  auto *h = new Handle;
  h->p.resize(n_vert);
  for (int32_t i = 0; i < n_vert; ++i) h->p[i] = Vector3f(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  h->ind.resize(3 * (size_t)n_tri);
  for (int64_t k = 0; k < 3 * (int64_t)n_tri; ++k) h->ind[k] = ind ? ind[k] : (int32_t)k;
  h->mesh.nInd = 3 * n_tri;
  h->mesh.nVert = n_vert;
  h->mesh.ind = h->ind.data();
  h->mesh.p = h->p.data();
  h->mesh.n = nullptr;
  h->mesh.uv = nullptr;
  h->builder = new Probe(&h->mesh, std::pmr::new_delete_resource());
  h->builder->build();
  return h;
}

// The builder's arrays after build(), in its own numbering: leaves in sorted
// order, internal node i = m_internal_nodes[i].  NULL outputs are skipped.
//   morton, perm (original triangle of each sorted leaf), leaf_parent: n
//   split, leaf_flags (bit0 left leaf, bit1 right leaf), n_triangles
//   (j - i + 1, signed as the reference stores it), direction, parent: n - 1
//   bounds: 6 (n - 1) (lower xyz, upper xyz); scene_bound: 6
void ref_radix_arrays(void *vh, uint32_t *morton, int32_t *perm, int32_t *leaf_parent, int32_t *split,
                      uint8_t *leaf_flags, int32_t *n_triangles, int32_t *direction, int32_t *parent,
                      float *bounds, float *scene_bound) {
  auto *h = static_cast<Handle *>(vh);
  Probe &b = *h->builder;
  const int n = b.m_n_triangles;
  for (int i = 0; i < n; ++i) {
    const auto &t = b.m_triangles[i];
    if (morton) morton[i] = t.morton_code;
    if (perm) perm[i] = (int32_t)((t.m_v - h->mesh.ind) / 3);
    if (leaf_parent) leaf_parent[i] = (int32_t)t.parent;
  }
  for (int i = 0; i + 1 < n; ++i) {
    const auto &nd = b.m_internal_nodes[i];
    if (split) split[i] = nd.split_point;
    if (leaf_flags) leaf_flags[i] = (uint8_t)((nd.left_node_type ? 1 : 0) | (nd.right_node_type ? 2 : 0));
    if (n_triangles) n_triangles[i] = nd.n_triangles;
    if (direction) direction[i] = nd.direction;
    if (parent) parent[i] = nd.parent;
    if (bounds)
      for (int k = 0; k < 3; ++k) {
        bounds[6 * (int64_t)i + k] = nd.bound.lower[k];
        bounds[6 * (int64_t)i + 3 + k] = nd.bound.upper[k];
      }
  }
  if (scene_bound)
    for (int k = 0; k < 3; ++k) {
      scene_bound[k] = b.m_bound.lower[k];
      scene_bound[3 + k] = b.m_bound.upper[k];
    }
}

// RadixBVHBuilder::intersect (radix_bvh.cpp:26-30, 202-245) for n rays given
// as 8 arrays of n floats (ox oy oz dx dy dz tnear tfar).  tfar initialises
// BVHRayHit::tfar; the reference ignores tnear.  Outputs hit (0/1), the final
// tfar and hit_ng (3 n floats, left untouched by a miss: zeros).
void ref_radix_intersect(void *vh, const float *rays, int64_t n, uint8_t *hit, float *tfar, float *ng) {
  auto *h = static_cast<Handle *>(vh);
  for (int64_t i = 0; i < n; ++i) {
    RadixBVHBuilder::BVHRayHit rh;
    rh.ray_o = Vector3f(rays[i], rays[n + i], rays[2 * n + i]);
    rh.ray_d = Vector3f(rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]);
    rh.tnear = rays[6 * n + i];
    rh.tfar = rays[7 * n + i];
    h->builder->intersect(rh);
    hit[i] = rh.hit ? 1 : 0;
    tfar[i] = rh.tfar;
    for (int k = 0; k < 3; ++k) ng[3 * i + k] = rh.hit_ng[k];
  }
}

void ref_radix_destroy(void *vh) {
  auto *h = static_cast<Handle *>(vh);
  delete h->builder;
  delete h;
}

// Triangle::intersect of the live renderer (shape.cpp:100-148) for n
// independent (triangle, ray) pairs.  tri: 9 n floats (p0 p1 p2 of pair i);
// rays: 8 arrays of n floats (ox oy oz dx dy dz, unused, tMax).  Outputs hit
// (0/1), t_hit and isect.m_ng (3 n floats) where hit, untouched otherwise.
void ref_triangle_intersect(const float *tri, const float *rays, int64_t n, uint8_t *hit, float *t,
                            float *ng) {
  for (int64_t i = 0; i < n; ++i) {
    Vector3f p[3];
    for (int k = 0; k < 3; ++k)
      p[k] = Vector3f(tri[9 * i + 3 * k], tri[9 * i + 3 * k + 1], tri[9 * i + 3 * k + 2]);
    int ind[3] = {0, 1, 2};
    fledge::TriangleMesh mesh{3, 3, ind, p, nullptr, nullptr};
    fledge::Triangle triangle(&mesh, 0);
    fledge::Ray ray(Vector3f(rays[i], rays[n + i], rays[2 * n + i]),
                    Vector3f(rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]), rays[7 * n + i]);
    fledge::SInteraction isect;
    float th = 0.0f;
    const bool ok = triangle.intersect(ray, th, isect);
    hit[i] = ok ? 1 : 0;
    if (ok) {
      t[i] = th;
      for (int k = 0; k < 3; ++k) ng[3 * i + k] = isect.m_ng[k];
    }
  }
}

}  // extern "C"
