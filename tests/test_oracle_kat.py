"""Pins the CPU oracle against known answers that do not come from the oracle
itself, and against the reference's own property tests for this path.

  * Philox-4x32-10 test vectors of Random123 (Salmon et al., SC'11)
  * Morton spread / encode bit patterns (experimental_utils.hpp:33-45),
    checked against a bit-by-bit interleave
  * the radix tree of Karras 2012 (HPG), Figure 3, on its 8 example keys
  * exact Pluecker hits on axis-aligned triangles (intersector.hpp:63-101)
  * Triangle.Watertight (shape_tests.cpp:22-48): every ray from inside the
    reference's meshed sphere hits
  * Accel.NaiveBVHAccel (accel_tests.cpp:16-56): two accelerators with the
    same primitive test agree exactly (here: the Karras BVH vs brute force)
  * regression against the committed golden fixtures
"""
import os

import numpy as np
import pytest

import geometry as G

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


class Med:
    sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0


def test_philox_known_answers(oracle):
    kat = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
           ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
           ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, want in kat:
        assert list(oracle.philox(ctr, key)) == want


def test_logf_accuracy(oracle):
    x = np.random.default_rng(0).random(200000).astype(np.float32)
    x = np.concatenate([x, np.float32(2.0 ** -24) * np.arange(1, 4000, dtype=np.float32), [1.0, 0.5, 2.0]])
    x = x[x > 0].astype(np.float32)
    y = oracle.logf(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    ulp = np.spacing(np.maximum(np.abs(ref), 1e-30).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(y - ref) <= 2.0 * ulp + 1e-12)
    assert oracle.logf(np.array([1.0], np.float32))[0] == 0.0


def _interleave(x, y, z):
    c = 0
    for b in range(10):
        c |= ((x >> b) & 1) << (3 * b)
        c |= ((y >> b) & 1) << (3 * b + 1)
        c |= ((z >> b) & 1) << (3 * b + 2)
    return c


def test_morton_bit_patterns(oracle):
    # Three point-like triangles: scene box [0,1]^3.  (0,0,0) -> 0, (1,1,1)
    # -> 1024 clamped to 1023 on every axis, (0.5,0.25,0.75) -> (512,256,768).
    pts = [(0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (0.5, 0.25, 0.75), (0.1, 0.9, 0.3)]
    pos = np.repeat(np.array(pts, np.float32), 3, axis=0)
    b = oracle.scene_bound(pos, None, 4)
    assert list(b) == [0, 0, 0, 1, 1, 1]
    codes = oracle.morton(pos, None, 4, b)
    want = [0, _interleave(1023, 1023, 1023), _interleave(512, 256, 768),
            _interleave(int(np.float32(0.1) * np.float32(1024)), int(np.float32(0.9) * np.float32(1024)),
                        int(np.float32(0.3) * np.float32(1024)))]
    assert [int(c) for c in codes] == want
    assert int(codes[1]) == 0x3FFFFFFF


def test_morton_zero_extent_axis(oracle):
    # All triangles in the plane z = 0.5: the reference divides 0 by 0; the
    # defined result is a zero z digit.
    rng = np.random.default_rng(7)
    pos = G.random_soup(64, rng)
    pos[:, 2] = 0.5
    b = oracle.scene_bound(pos, None, 64)
    codes = oracle.morton(pos, None, 64, b)
    assert np.all((codes & 0x24924924) == 0)  # every z bit is zero


def test_karras_paper_figure(oracle):
    codes = np.array([0b00001, 0b00010, 0b00100, 0b00101, 0b10011, 0b11000, 0b11001, 0b11110], np.uint32)
    k = oracle.karras(codes)
    # node: (range end j, split, left leaf?, right leaf?)
    want = {0: (7, 3, 0, 0), 1: (0, 0, 1, 1), 2: (3, 2, 1, 1), 3: (0, 1, 0, 0), 4: (7, 4, 1, 0),
            5: (7, 6, 0, 1), 6: (5, 5, 1, 1)}
    for i, (j, s, ll, rl) in want.items():
        assert k["range_j"][i] == j and k["split"][i] == s
        assert (k["leaf_flags"][i] & 1) == ll and ((k["leaf_flags"][i] >> 1) & 1) == rl
    assert list(k["leaf_parent"]) == [1, 1, 2, 2, 4, 6, 6, 5]


def test_karras_duplicate_keys_is_a_tree(oracle):
    # All codes equal: delta falls back to clz(i ^ j) + 32 (radix_bvh.hpp:68-74).
    for n in (2, 3, 5, 17, 64, 1000):
        k = oracle.karras(np.zeros(n, np.uint32))
        _check_tree(k, n)


def _check_tree(k, n):
    """Every leaf and every non-root node has exactly one parent; ranges nest."""
    seen_leaf = np.zeros(n, int)
    seen_node = np.zeros(max(n - 1, 1), int)
    for i in range(n - 1):
        s, lf = k["split"][i], k["leaf_flags"][i]
        lo, hi = min(i, k["range_j"][i]), max(i, k["range_j"][i])
        assert lo <= s < hi
        for side, c in ((0, s), (1, s + 1)):
            if lf >> side & 1:
                seen_leaf[c] += 1
            else:
                seen_node[c] += 1
                clo, chi = min(c, k["range_j"][c]), max(c, k["range_j"][c])
                assert (clo, chi) == ((lo, s) if side == 0 else (s + 1, hi))
    assert np.all(seen_leaf == 1)
    if n > 1:
        assert seen_node[0] == 0 and np.all(seen_node[1:n - 1] == 1)


def test_sort_is_stable_on_ties(oracle):
    codes = np.array([5, 1, 5, 0, 1, 5], np.uint32)
    s, p = oracle.sort(codes)
    assert list(s) == [0, 1, 1, 5, 5, 5] and list(p) == [3, 1, 4, 0, 2, 5]


def test_refit_matches_bruteforce(oracle):
    pos = G.random_soup(777, np.random.default_rng(3))
    t = oracle.build_bvh(pos)
    _check_tree(t, 777)
    tri = pos.reshape(-1, 3, 3)
    lo, hi = tri.min(1), tri.max(1)
    # node bound = union of its sorted range's triangle boxes
    for i in range(776):
        a, b = min(i, t["range_j"][i]), max(i, t["range_j"][i])
        ids = t["perm"][a:b + 1]
        assert np.array_equal(t["bounds"][i, :3], lo[ids].min(0))
        assert np.array_equal(t["bounds"][i, 3:], hi[ids].max(0))
    assert np.array_equal(t["bounds"][0], t["scene_bound"])


def test_pluecker_exact(oracle):
    a, b, c = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    for mode in (oracle.MODE_REF, oracle.MODE_DEV):
        ok, tuv = oracle.pluecker(a, b, c, [0.25, 0.25, 1.0], [0, 0, -1], mode)
        assert ok and list(tuv) == [1.0, 0.25, 0.25]
        ok, tuv = oracle.pluecker(a, b, c, [0.25, 0.5, -2.0], [0, 0, 1], mode)
        assert ok and list(tuv) == [2.0, 0.25, 0.5]
        assert not oracle.pluecker(a, b, c, [1.0, 1.0, 1.0], [0, 0, -1], mode)[0]
        assert not oracle.pluecker(a, b, c, [0.25, 0.25, 1.0], [0, 0, 1], mode)[0]  # behind


def test_moller_trumbore_known_answers(oracle):
    """The live renderer's Triangle::intersect (shape.cpp:100-148) as restated
    in the oracle: exact hits, barycentrics (u on p1, v on p2), and the cases
    it rejects — zero area, parallel rays, hits behind the origin, outside the
    triangle."""
    a, b, c = (0, 0, 0), (1, 0, 0), (0, 1, 0)
    ok, h = oracle.pluecker(a, b, c, (0.25, 0.5, 1.0), (0, 0, -1), oracle.MODE_MT)
    assert ok and h[0] == 1.0 and h[1] == 0.25 and h[2] == 0.5
    assert not oracle.pluecker(a, b, (2, 0, 0), (0.25, 0.0, 1.0), (0, 0, -1), oracle.MODE_MT)[0]  # area 0
    assert not oracle.pluecker(a, b, c, (0.25, 0.25, 1.0), (1, 0, 0), oracle.MODE_MT)[0]  # parallel
    assert not oracle.pluecker(a, b, c, (0.25, 0.25, -1.0), (0, 0, -1), oracle.MODE_MT)[0]  # behind
    assert not oracle.pluecker(a, b, c, (0.75, 0.75, 1.0), (0, 0, -1), oracle.MODE_MT)[0]  # u + v > 1
    # a hit on the watertight test's side agrees on t and barycentrics with it
    okp, hp = oracle.pluecker(a, b, c, (0.25, 0.5, 1.0), (0, 0, -1), oracle.MODE_REF)
    assert okp and np.allclose(hp, h)


def test_reference_normalize_defect(oracle):
    # common/vector.h:495-503 sums z instead of z*z: a normal with a large
    # negative z gives sqrt(negative) = NaN and the reference misses.
    a, b, c = [0, 0, 0], [0, 1, 0], [1, 0, 0]  # winding with normal -z
    ok_ref, _ = oracle.pluecker(a, b, c, [0.25, 0.25, 1.0], [0, 0, -1], oracle.MODE_REF)
    ok_def, _ = oracle.pluecker(a, b, c, [0.25, 0.25, 1.0], [0, 0, -1], oracle.MODE_DEFECT)
    assert ok_ref and not ok_def


def test_watertight_meshed_sphere(oracle):
    v, ind = G.meshed_sphere(16, 16, 1.0)
    tree = oracle.build_bvh(v, ind)
    rays = G.interior_rays(1000, np.random.default_rng(114514))
    for mode in (oracle.MODE_REF, oracle.MODE_DEV):
        h = oracle.trace_closest(v, ind, tree, rays, mode)
        assert np.all(h["prim"] >= 0)


def test_bvh_agrees_with_bruteforce(oracle):
    """Accel.NaiveBVHAccel pattern: the BVH and a linear scan with the same
    triangle test return identical hits."""
    pos = G.random_soup(300, np.random.default_rng(11), half=0.05)
    tree = oracle.build_bvh(pos)
    rays = G.sphere_rays(400, np.random.default_rng(12), tmin=0.0)
    h = oracle.trace_closest(pos, None, tree, rays, oracle.MODE_DEV)
    tri = pos.reshape(-1, 3, 3)
    for i in range(400):
        best, bp = np.inf, -1
        for k in range(300):
            ok, tuv = oracle.pluecker(tri[k, 0], tri[k, 1], tri[k, 2], rays[0:3, i], rays[3:6, i], oracle.MODE_DEV)
            if ok and tuv[0] < best:
                best, bp = tuv[0], k
        assert h["prim"][i] == bp
    # reported t, u, v are the selected triangle's FP64 values rounded once
    tuv, ok = oracle.hit_values64(pos, None, 300, rays, h["prim"])
    hit = h["prim"] >= 0
    assert np.array_equal(h["t"][hit], tuv[hit, 0].astype(np.float32))
    assert np.array_equal(h["u"][hit], tuv[hit, 1].astype(np.float32))


def test_any_hit_consistent_with_closest(oracle):
    pos = G.random_soup(500, np.random.default_rng(21), half=0.04)
    tree = oracle.build_bvh(pos)
    rays = G.sphere_rays(2000, np.random.default_rng(22), tmax=2.0)
    h = oracle.trace_closest(pos, None, tree, rays, oracle.MODE_DEV)
    occ = oracle.trace_any(pos, None, tree, rays, oracle.MODE_DEV)
    assert np.array_equal(occ.astype(bool), h["prim"] >= 0)


def test_ratio_tracking_vs_fp64(oracle):
    rho = G.value_noise_grid(24, np.random.default_rng(3))
    rays = G.sphere_rays(4096, np.random.default_rng(4))
    T = oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], Med, rays, 99)
    T64, _ = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], Med, rays, 99)
    close = np.abs(T - T64) <= 1e-5 * np.maximum(np.abs(T64), 1e-30) + 1e-6
    assert close.mean() > 0.999


def test_ratio_tracking_homogeneous_expectation(oracle):
    # Constant density: E[T] = exp(-sigma_t * rho * L) along each ray.
    rho = np.full((8, 8, 8), 2.0, np.float32)
    n = 20000
    r = np.zeros((8, n), np.float32)
    r[0], r[1], r[2] = -1.0, 0.5, 0.5
    r[3] = 1.0
    r[7] = np.inf
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=0.0, majorant=4.0))
    T = oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], med, r, 5)
    assert abs(T.mean() - np.exp(-2.0)) < 4 * T.std() / np.sqrt(n)


def test_delta_tracking_collision_rate(oracle):
    # Constant density, no roulette: P(collision within length 1) = 1 - exp(-sigma_t rho).
    rho = np.full((8, 8, 8), 1.5, np.float32)
    n = 20000
    r = np.zeros((8, n), np.float32)
    r[0], r[1], r[2] = -1.0, 0.5, 0.5
    r[3] = 1.0
    r[7] = np.inf
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=0.1, majorant=3.0))
    ok, p, w = oracle.volume_sample(rho, [0, 0, 0], [1, 1, 1], med, r, 8)
    pr = 1 - np.exp(-1.5)
    assert abs(ok.mean() - pr) < 4 * np.sqrt(pr * (1 - pr) / n)
    assert np.all(w[ok.astype(bool)] == np.float32(0.8) / np.float32(1.0))
    assert np.all((p[ok.astype(bool), 0] >= 0) & (p[ok.astype(bool), 0] <= 1))


def test_volume_adjoint_matches_fd64(oracle):
    """Analytic adjoint (fp32 forward, fp64 accumulation) vs FP64 central
    finite differences of summed transmittance, majorant held fixed."""
    res = 12
    rho = G.value_noise_grid(res, np.random.default_rng(31))
    rays = G.sphere_rays(3000, np.random.default_rng(32))
    maj = float(rho.max())
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=0.1, majorant=maj))
    seed = 1234
    dLdT = np.ones(3000, np.float32)
    grad = oracle.volume_tr_adjoint(rho, [0, 0, 0], [1, 1, 1], med, rays, seed, dLdT)
    rng = np.random.default_rng(33)
    flat = rho.reshape(-1)
    cand = np.argsort(-np.abs(grad.reshape(-1)))[:200]
    picks = rng.choice(cand, 16, replace=False)
    for v in picks:
        if flat[v] > maj - 1e-3:
            continue
        h = 1e-4 * max(1.0, abs(float(flat[v])))
        r64p = rho.astype(np.float64).copy().reshape(-1)
        r64m = r64p.copy()
        r64p[v] += h
        r64m[v] -= h
        Tp, np_ = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], med, rays, seed, r64p.reshape(rho.shape))
        Tm, nm = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], med, rays, seed, r64m.reshape(rho.shape))
        keep = np_ == nm  # exclude rays whose roulette decisions flip
        assert (~keep).sum() <= 2
        fd = (Tp[keep].sum() - Tm[keep].sum()) / (2 * h)
        g = grad.reshape(-1)[v]
        assert abs(fd - g) <= 1e-3 * abs(fd) + 1e-6, (v, fd, g)


def test_hit_adjoint_matches_fd64(oracle):
    pos = G.random_soup(200, np.random.default_rng(41), half=0.05)
    tree = oracle.build_bvh(pos)
    rays = G.sphere_rays(3000, np.random.default_rng(42), tmin=0.0)
    h = oracle.trace_closest(pos, None, tree, rays, oracle.MODE_DEV)
    hit = np.nonzero(h["prim"] >= 0)[0][:40]
    assert hit.size >= 20
    rays = np.ascontiguousarray(rays[:, hit])
    prim = h["prim"][hit]
    g = np.random.default_rng(43).standard_normal((3, hit.size)).astype(np.float32)
    grad = oracle.hit_adjoint64(pos, None, 200, 600, rays, prim, g[0], g[1], g[2])
    for r in range(hit.size):
        p = prim[r]
        for c in range(3):
            for ax in range(3):
                vi = 3 * p + c
                eps = 1e-6
                pp, pm = pos.astype(np.float64).copy(), pos.astype(np.float64).copy()
                pp[vi, ax] += eps
                pm[vi, ax] -= eps
                # FP64 central difference of L = g . (t, u, v) for this ray
                fdv = (_L64(pp, p, rays[:, r], g[:, r]) - _L64(pm, p, rays[:, r], g[:, r])) / (2 * eps)
                gv = grad[vi, ax] if np.count_nonzero(prim == p) == 1 else None
                if gv is not None:
                    assert abs(fdv - gv) <= 1e-3 * max(1.0, abs(fdv)), (r, c, ax, fdv, gv)


def _L64(P, prim, ray, g):
    a, b, c = P[3 * prim], P[3 * prim + 1], P[3 * prim + 2]
    o, d = ray[0:3].astype(np.float64), ray[3:6].astype(np.float64)
    e1, e2 = b - a, c - a
    M = np.stack([d, -e1, -e2], 1)
    t, u, v = np.linalg.solve(M, a - o)
    return float(g[0] * t + g[1] * u + g[2] * v)


def test_golden_regression(oracle):
    d = np.load(GOLDEN)
    pos = d["soup_pos"]
    t = oracle.build_bvh(pos)
    for k in ("morton", "perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds",
              "scene_bound"):
        assert np.array_equal(t[k], d["soup_" + k]), k
    for name, mode in (("ref", oracle.MODE_REF), ("dev", oracle.MODE_DEV)):
        h = oracle.trace_closest(pos, None, t, d["soup_rays"], mode)
        for k in ("prim", "t", "u", "v"):
            assert np.array_equal(h[k], d[f"soup_hit_{name}_{k}"]), (name, k)
    assert np.array_equal(oracle.trace_any(pos, None, t, d["soup_rays_short"], oracle.MODE_DEV), d["soup_occ"])
    T, ck = oracle.volume_tr(d["vol_rho"], [0, 0, 0], [1, 1, 1], Med, d["vol_rays"], int(d["vol_seed"]), True)
    assert np.array_equal(T, d["vol_T"]) and np.array_equal(ck["k"], d["vol_ck_k"])
    ok, p, w = oracle.volume_sample(d["vol_rho"], [0, 0, 0], [1, 1, 1], Med, d["vol_rays"], int(d["vol_seed"]))
    assert np.array_equal(ok, d["vol_ok"]) and np.array_equal(p, d["vol_p"])


def test_reference_performance_build_matches(oracle):
    pos = G.random_soup(5000, np.random.default_rng(51))
    a = oracle.build_bvh(pos)
    b = oracle.build_timed(pos, None, 5000)
    for k in ("morton", "perm", "split", "leaf_flags", "range_j", "bounds"):
        assert np.array_equal(a[k], b[k]), k
