"""GPU traversal parity against the oracle's restatement of recursiveIntersect
(radix_bvh.cpp:202-245) with the Pluecker test (intersector.hpp:63-101).

  * DEV mode (the GPU's arithmetic): prim ids equal except recorded exact
    ties, t/u/v bit-equal where the ids agree
  * REF mode (the reference's normalised-normal arithmetic): prim ids equal
    except ties within a few ulps
  * FP64 oracle: t within 1e-5 relative, barycentrics within 1e-5
  * any-hit: occlusion bits equal
"""
import os

import numpy as np
import pytest

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")

LAYOUTS = [(2, 1, {}), (4, 1, {}), (4, 4, {}), (8, 1, {}), (8, 2, {"stack_depth": 32}),
           (4, 1, {"persistent": 1, "refill_lanes": 16}), (8, 4, {"persistent": 1, "refill_lanes": 8}),
           (4, 1, {"persistent": 2, "refill_lanes": 16}), (8, 2, {"persistent": 2, "refill_lanes": 1}),
           (4, 4, {"persistent": 2, "refill_lanes": 32, "stack_depth": 32})]


def _ids(v):
    return f"w{v[0]}l{v[1]}" + "".join(f"-{k}{x}" for k, x in v[2].items())


@pytest.fixture(scope="module")
def c0_case(oracle):
    pos = G.random_soup(65536, np.random.default_rng(100))
    rays = G.sphere_rays(1 << 18, np.random.default_rng(101))
    return pos, rays, oracle.build_bvh(pos)


@pytest.mark.parametrize("layout", LAYOUTS, ids=_ids)
def test_closest_matches_oracle_dev(ctx, oracle, c0_case, layout):
    pos, r8, tree = c0_case
    w, leaf, opts = layout
    b, _ = U.gpu_build(ctx, pos, width=w, leaf=leaf)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, **opts))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    assert (hg["prim"] >= 0).mean() > 0.3


def test_closest_vs_reference_arithmetic_and_fp64(ctx, oracle, c0_case):
    pos, r8, tree = c0_case
    b, _ = U.gpu_build(ctx, pos, width=4)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd))
    bad, ties, _ = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_REF, allow_rel=4e-7)
    assert bad == 0, f"{bad} mismatches vs the reference arithmetic ({ties} near-ties)"
    U.check_t_fp64(oracle, pos, None, 65536, r8, hg, rel=1e-5)


@pytest.mark.parametrize("w", [2, 4, 8])
def test_any_hit_matches_oracle(ctx, oracle, c0_case, w):
    pos, r8, tree = c0_case
    short = r8.copy()
    short[7] = np.random.default_rng(5).uniform(1.0, 2.5, r8.shape[1]).astype(np.float32)
    b, _ = U.gpu_build(ctx, pos, width=w)
    rd, _ = U.rays_dev(short)
    occ = b.intersectP(rd).cpu().numpy()
    ref = oracle.trace_any(pos, None, tree, short, oracle.MODE_DEV)
    assert np.array_equal(occ, ref), np.count_nonzero(occ != ref)
    assert 0.05 < occ.mean() < 0.95


@pytest.mark.parametrize("w", [2, 4, 8])
def test_watertight_sphere(ctx, oracle, w):
    """Triangle.Watertight (shape_tests.cpp:22-48) at 16x16 and at the
    bvh_test sphere resolution 1000x1000 (1,994,004 triangles)."""
    for nt, npn, nr in ((16, 16, 1000), (1000, 1000, 200000)):
        v, ind = G.meshed_sphere(nt, npn, 1.0)
        b, _ = U.gpu_build(ctx, v, ind, width=w)
        rays = G.interior_rays(nr, np.random.default_rng(114514))
        rd, _ = U.rays_dev(rays)
        hg = U.host(b.intersect(rd))
        assert np.all(hg["prim"] >= 0), np.count_nonzero(hg["prim"] < 0)
        occ = b.intersectP(rd).cpu().numpy()
        assert np.all(occ == 1)


def test_sphere_matches_oracle(ctx, oracle):
    v, ind = G.meshed_sphere(128, 128, 1.0)
    tree = oracle.build_bvh(v, ind)
    rays = G.interior_rays(50000, np.random.default_rng(7))
    for w in (2, 4, 8):
        b, _ = U.gpu_build(ctx, v, ind, width=w)
        rd, _ = U.rays_dev(rays)
        hg = U.host(b.intersect(rd))
        bad, ties, _ = U.compare_closest(oracle, v, ind, tree, rays, hg, oracle.MODE_DEV)
        assert bad == 0, (w, bad, ties)


def test_golden_fixture_hits(ctx):
    d = np.load(GOLDEN)
    b, _ = U.gpu_build(ctx, d["soup_pos"], width=4)
    rd, _ = U.rays_dev(d["soup_rays"])
    hg = U.host(b.intersect(rd))
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(hg[k], d["soup_hit_dev_" + k]), k
    rs, _ = U.rays_dev(d["soup_rays_short"])
    assert np.array_equal(b.intersectP(rs).cpu().numpy(), d["soup_occ"])
    bs, _ = U.gpu_build(ctx, d["sphere_pos"], d["sphere_ind"], width=8)
    rd, _ = U.rays_dev(d["sphere_rays"])
    hs = U.host(bs.intersect(rd))
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(hs[k], d["sphere_hit_" + k]), k


@pytest.mark.parametrize("layout", [(2, 1, {}), (4, 1, {}), (4, 3, {"persistent": 2, "refill_lanes": 16,
                                                                    "stack_depth": 32}),
                                    (8, 2, {"persistent": 1, "refill_lanes": 8})], ids=_ids)
def test_edge_case_rays_match_oracle(ctx, oracle, layout):
    """Rays through shared vertices and edges of an axis-aligned grid
    (watertight: every interior one hits), rays in and next to the grid's
    plane (zero direction components: NaN slabs), degenerate triangles, a
    zero direction and NaN origins: closest hits and occlusion equal the
    oracle's, but for the extra hits that leaf ranges find at flat-box
    vertices (below)."""
    pos, r8 = G.edge_case_scene(np.random.default_rng(5))
    tree = oracle.build_bvh(pos)
    w, leaf, opts = layout
    b, _ = U.gpu_build(ctx, pos, width=w, leaf=leaf)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, **opts))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    # A leaf range is tested once its range box passes the slab test, where
    # the reference tests each triangle pair's parent box.  A ray through a
    # vertex shared by flat (zero-thickness) boxes can pass the range box and
    # fail the tighter parent boxes by one rounding: then the GPU finds a hit
    # that the reference's traversal misses.  Such a hit must be one the
    # triangle test accepts at exactly the reported t; nothing else may differ.
    tri = pos.reshape(-1, 3, 3)
    extra_rays = np.nonzero((hg["prim"] >= 0) & (ho["prim"] < 0))[0]
    for i in extra_rays:
        ok, t = oracle.pluecker(tri[hg["prim"][i], 0], tri[hg["prim"][i], 1], tri[hg["prim"][i], 2],
                                r8[0:3, i], r8[3:6, i], oracle.MODE_DEV)
        assert ok and float(t[0]) >= r8[6, i], i
    extra = len(extra_rays)
    assert bad - extra == 0, f"{bad - extra} prim mismatches ({ties} exact ties)"
    assert extra == 0 if leaf == 1 else extra <= 8, extra
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    down = 17 * 17 * 2
    inside = (r8[0, :down] < 1.0) & (r8[1, :down] < 1.0)
    assert np.all(hg["prim"][:down][inside] >= 0)
    assert np.all(hg["prim"][-3:] == -1)
    occ = b.intersectP(rd, **opts).cpu().numpy()
    ref = oracle.trace_any(pos, None, tree, r8, oracle.MODE_DEV)
    ref[extra_rays] = 1  # the same rays, occluded by the same accepted hits
    assert np.array_equal(occ, ref), np.count_nonzero(occ != ref)


def test_tmin_tmax_and_constants(ctx, oracle):
    pos = G.random_soup(20000, np.random.default_rng(31), half=0.03)
    tree = oracle.build_bvh(pos)
    r8 = G.sphere_rays(50000, np.random.default_rng(32))
    r8[6] = np.random.default_rng(33).uniform(0.0, 2.0, r8.shape[1])
    r8[7] = r8[6] + np.random.default_rng(34).uniform(0.0, 1.5, r8.shape[1])
    b, _ = U.gpu_build(ctx, pos, width=4)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd))
    bad, ties, _ = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0
    # constant tmin/tmax path
    import fledge_gb300 as F
    t = U.dev(r8)
    rc = F.Rays(*[t[k] for k in range(6)], tmin_const=1e-4, tmax_const=float("inf"))
    r8c = r8.copy()
    r8c[6], r8c[7] = 1e-4, np.inf
    hc = U.host(b.intersect(rc))
    bad, _, _ = U.compare_closest(oracle, pos, None, tree, r8c.astype(np.float32), hc, oracle.MODE_DEV)
    assert bad == 0


def test_empty_and_single_triangle_scenes(ctx, oracle):
    import fledge_gb300 as F
    r8 = G.sphere_rays(4096, np.random.default_rng(3))
    rd, _ = U.rays_dev(r8)
    e = F.RadixBVHBuilder(F.InternalTriangleMesh(U.dev(np.zeros((0, 3), np.float32))), ctx, node_width=4)
    e.build()
    h = U.host(e.intersect(rd))
    assert np.all(h["prim"] == -1) and np.all(np.isinf(h["t"]))
    big = np.array([[0.0, 0.0, 0.5], [1.0, 0.0, 0.5], [0.0, 1.0, 0.5]], np.float32)
    for w in (2, 4, 8):
        s, _ = U.gpu_build(ctx, big, width=w)
        h = U.host(s.intersect(rd))
        tree = oracle.build_bvh(big)
        ho = oracle.trace_closest(big, None, tree, r8, oracle.MODE_DEV)
        assert np.array_equal(h["prim"], ho["prim"]) and np.array_equal(h["t"], ho["t"])


def test_host_staged_entry_point(ctx, oracle):
    """flg_trace_closest_host: host buffers in, host buffers out, in chunks of
    2^22 rays through two staging buffers (three chunks: the first buffer is
    refilled once its hits are out)."""
    import ctypes as C

    import fledge_gb300 as F
    import torch
    pos = G.random_soup(30000, np.random.default_rng(61))
    b, _ = U.gpu_build(ctx, pos, width=4)
    n = (2 << 22) + 12345
    r8 = G.sphere_rays(n, np.random.default_rng(62))
    rh = torch.from_numpy(r8).pin_memory()
    out = {k: torch.empty(n, dtype=torch.int32 if k == "prim" else torch.float32).pin_memory()
           for k in ("prim", "t", "u", "v")}
    rs = F.Rays(*[rh[k] for k in range(8)])
    r, hs = rs.struct(), F._hits_struct(out)
    op = F.FlgTraceOpts(0, 0, 0, 0, 0)
    ctx.check(ctx.lib.flg_trace_closest_host(ctx.h, b.h, C.byref(r), n, C.byref(op), C.byref(hs)))
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd))
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(out[k].numpy(), hg[k]), k


def test_autotune_runs_and_keeps_parity(ctx, oracle, c0_case):
    import ctypes as C
    import json

    import fledge_gb300 as F
    pos, r8, tree = c0_case
    b, _ = U.gpu_build(ctx, pos, width=4)
    rd, _ = U.rays_dev(r8)
    best = F.FlgTraceOpts()
    w = C.c_int32()
    buf = C.create_string_buffer(1 << 16)
    r = rd.struct()
    ctx.check(ctx.lib.flg_autotune_trace(ctx.h, b.h, C.byref(r), rd.n, C.byref(best), C.byref(w), buf, 1 << 16))
    rec = json.loads(buf.value.decode())
    assert rec["best"]["node_width"] == w.value and len(rec["trials"]) > 10
    hg = U.host(b.intersect(rd, stack_depth=best.stack_depth, block_threads=best.block_threads,
                            persistent=best.persistent, refill_lanes=best.refill_lanes))
    bad, _, _ = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0


@pytest.mark.parametrize("w", [2, 4])
def test_moller_trumbore_mode_matches_oracle(ctx, oracle, c0_case, w):
    """tri_test=1: the live renderer's Moller-Trumbore Triangle::intersect
    (shape.cpp:100-148) with its strict t < tMax rule, over the BVH2 layout of
    any handle; closest hits and occlusion as the oracle's MT mode (ids equal
    except recorded exact ties, t/u/v equal where the ids agree)."""
    pos, r8, tree = c0_case
    b, _ = U.gpu_build(ctx, pos, width=w)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, tri_test=1))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_MT)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    assert (hg["prim"] >= 0).mean() > 0.3
    short = r8.copy()
    short[7] = np.random.default_rng(6).uniform(1.0, 2.5, r8.shape[1]).astype(np.float32)
    rs, _ = U.rays_dev(short)
    occ = b.intersectP(rs, tri_test=1).cpu().numpy()
    ref = oracle.trace_any(pos, None, tree, short, oracle.MODE_MT)
    assert np.array_equal(occ, ref), np.count_nonzero(occ != ref)



@pytest.mark.parametrize("w,opts", [(2, {}), (4, {"persistent": 2, "refill_lanes": 8}), (8, {"persistent": 1})])
def test_ray_sort_gives_identical_hits(ctx, c0_case, w, opts):
    """ray_sort=1 traces the rays in octant / origin-Morton order and writes
    the hits back in the caller's order: every ray's result is the same as
    without sorting (closest and any hit)."""
    pos, r8, _ = c0_case
    b, _ = U.gpu_build(ctx, pos, width=w)
    rd, _ = U.rays_dev(r8)
    h0 = U.host(b.intersect(rd, **opts))
    h1 = U.host(b.intersect(rd, ray_sort=1, **opts))
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(h0[k], h1[k]), k
    o0 = b.intersectP(rd, **opts).cpu().numpy()
    o1 = b.intersectP(rd, ray_sort=1, **opts).cpu().numpy()
    assert np.array_equal(o0, o1)
    ctx.sync()


def test_ray_sort_rejects_batched_traces(ctx):
    import fledge_gb300 as F
    offs = np.array([0, 100, 300], np.int64)
    pos = F.gen_triangles(ctx, 300, 3)
    soa = F.gen_rays(ctx, 300 * 4, 4)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(pos), offs, ctx, node_width=4)
    bb.build()
    with pytest.raises(F.FlgError):
        bb.intersect_batched(F.Rays.from_soa(soa), offs * 4, ray_sort=1)
