"""Pins the CPU oracle to the reference's own code: RadixBVHBuilder
(src/experimental/radix_bvh.cpp) and the live renderer's Triangle::intersect
(src/shape.cpp:100-148), compiled unchanged into oracle/_ref/libfledge_ref.so
against stand-in headers for oneTBB, fmt and Embree (oracle/ref_driver.cpp).

Checked bit for bit on the same inputs:
  * Morton codes, sorted leaf order, Karras topology (split, leaf flags,
    range, parents), refit bounds and the scene bound;
  * closest-hit traversal: RadixBVHBuilder::intersect's hit flag, tfar and
    hit_ng against the oracle in MODE_DEFECT, which restates the reference's
    StableNormalize literally (the other modes differ only in that line);
  * Triangle::intersect's hit decision and t against the oracle's MODE_MT.
The stand-in parallel_sort is stable, so equal Morton codes keep index order,
the order the oracle defines (TBB's is unspecified).  Scenes with a
zero-extent axis are left out: the reference converts 0/0 to an integer
there (undefined behaviour), which the oracle defines as a zero digit.

The library is built where the reference sources are present; elsewhere
those tests skip.  The committed fixture of the reference's outputs
(tests/golden/reference_lbvh.npz) is checked against the oracle everywhere.
"""
import os

import numpy as np
import pytest

import geometry as G

REF_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_lbvh.npz")


@pytest.fixture(scope="module")
def ref():
    from oracle import reference as R
    if not R.build():
        pytest.skip("reference sources not present: oracle/_ref not built")
    return R


def _same_build(oracle, ref, pos, ind=None):
    r = ref.RadixBVH(pos, ind)
    a = r.arrays()
    t = oracle.build_bvh(pos, ind)
    n = r.n
    for k in ("morton", "perm", "split", "leaf_flags", "parent", "leaf_parent", "bounds", "scene_bound"):
        x, y = a[k], np.asarray(t[k]).reshape(a[k].shape)
        assert np.array_equal(x, y), f"{k}: {np.count_nonzero(x != y)} of {x.size} differ"
    i = np.arange(n - 1)
    # the reference stores j - i + 1 (signed) and the direction sign(j - i)
    assert np.array_equal(a["n_triangles"], t["range_j"] - i + 1)
    assert np.array_equal(a["direction"], np.sign(t["range_j"] - i))
    return r, t


def _same_hits(oracle, r, t, pos, ind, rays):
    hr = r.intersect(rays)
    ho = oracle.trace_closest(pos, ind, t, rays, oracle.MODE_DEFECT)
    hit = ho["prim"] >= 0
    assert np.array_equal(hr["hit"], hit)
    assert np.array_equal(hr["tfar"], ho["t"])
    ng = oracle.hit_normals(pos, ind, r.n, rays, ho["prim"], oracle.MODE_DEFECT)
    assert np.array_equal(hr["ng"], ng)
    return hit.mean()


def _rays_far(n, seed):
    # BVHRayHit starts with tfar = FLT_MAX (base_bvh.hpp:45); tnear is ignored
    return G.sphere_rays(n, np.random.default_rng(seed), tmin=0.0, tmax=np.finfo(np.float32).max)


@pytest.mark.parametrize("n", [2, 3, 5, 17, 1000, 65536])
def test_random_soup_build_and_trace(oracle, ref, n):
    """Config-0 style soups up to its full 65,536 triangles."""
    pos = G.random_soup(n, np.random.default_rng(100 + n))
    r, t = _same_build(oracle, ref, pos)
    rate = _same_hits(oracle, r, t, pos, None, _rays_far(4096 if n > 1000 else 2048, 200 + n))
    if n >= 1000:
        assert rate > 0.005  # 1.3 % of rays hit 1000 triangles, 57 % hit 65,536
    r.close()


def test_duplicate_morton_codes(oracle, ref):
    """Identical triangles: every delta falls back to clz(i ^ j) + 32."""
    pos = np.tile(G.random_soup(1, np.random.default_rng(3)), (300, 1))
    pos = np.concatenate([pos, G.random_soup(50, np.random.default_rng(4))])
    r, t = _same_build(oracle, ref, pos)
    _same_hits(oracle, r, t, pos, None, _rays_far(1024, 5))
    r.close()


def test_indexed_meshed_sphere_watertight(oracle, ref):
    """MakeMeshedSphere with Triangle.Watertight's interior rays
    (shape_tests.cpp:22-48): indexed input, shared vertices."""
    v, ind = G.meshed_sphere(40, 40, 1.0)
    r, t = _same_build(oracle, ref, v, ind)
    rays = G.interior_rays(4000, np.random.default_rng(114514))
    rays[7] = np.finfo(np.float32).max
    _same_hits(oracle, r, t, v, ind, rays)
    r.close()


def test_deep_clustered_tree(oracle, ref):
    """Clusters at geometrically shrinking scales: long Morton prefixes."""
    pos = G.geometric_clusters(12, 64, np.random.default_rng(9))
    r, t = _same_build(oracle, ref, pos)
    _same_hits(oracle, r, t, pos, None, _rays_far(2048, 10))
    r.close()


def test_triangle_intersect_moller_trumbore(oracle, ref):
    """Triangle::intersect (shape.cpp:100-148) against MODE_MT on pairs aimed
    around each triangle (barycentrics in [-0.2, 1.2], edges included), with
    infinite and finite tMax."""
    rng = np.random.default_rng(11)
    n = 6000
    tri = G.random_soup(n, rng).reshape(n, 3, 3)
    b = rng.uniform(-0.2, 1.2, (n, 2)).astype(np.float32)
    tgt = tri[:, 0] + b[:, :1] * (tri[:, 1] - tri[:, 0]) + b[:, 1:] * (tri[:, 2] - tri[:, 0])
    o = rng.uniform(-1.0, 2.0, (n, 3)).astype(np.float32)
    d = (tgt - o).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for tmax in (np.inf, 1.5):
        rays = np.zeros((8, n), np.float32)
        rays[0:3], rays[3:6], rays[7] = o.T, d.T, tmax
        hr = ref.triangle_intersect(tri, rays)
        ok = np.zeros(n, bool)
        t = np.zeros(n, np.float32)
        for i in range(n):
            k, tuv = oracle.pluecker(tri[i, 0], tri[i, 1], tri[i, 2], o[i], d[i], oracle.MODE_MT)
            ok[i], t[i] = k and tuv[0] < tmax, tuv[0]
        assert np.array_equal(ok, hr["hit"])
        assert np.array_equal(t[ok], hr["t"][ok])
        assert 0.1 < ok.mean() < 0.9


@pytest.mark.parametrize("name", ["soup", "sphere"])
def test_oracle_matches_reference_fixture(oracle, name):
    """The committed outputs of the reference's RadixBVHBuilder
    (tests/golden/make_reference_golden.py) against the oracle.  Needs no
    reference sources, so it also runs where oracle/_ref cannot be built."""
    g = np.load(REF_GOLDEN)
    pos = g[name + "_pos"]
    ind = g[name + "_ind"] if name + "_ind" in g else None
    t = oracle.build_bvh(pos, ind)
    for k in ("morton", "perm", "split", "leaf_flags", "parent", "leaf_parent", "bounds", "scene_bound"):
        assert np.array_equal(np.asarray(t[k]).reshape(g[f"{name}_{k}"].shape), g[f"{name}_{k}"]), k
    n = t["n"]
    assert np.array_equal(g[name + "_n_triangles"], t["range_j"] - np.arange(n - 1) + 1)
    rays = g[name + "_rays"]
    ho = oracle.trace_closest(pos, ind, t, rays, oracle.MODE_DEFECT)
    assert np.array_equal(g[name + "_ref_hit"], ho["prim"] >= 0)
    assert np.array_equal(g[name + "_ref_tfar"], ho["t"])
    assert np.array_equal(g[name + "_ref_ng"], oracle.hit_normals(pos, ind, n, rays, ho["prim"], oracle.MODE_DEFECT))
