"""GPU LBVH build parity: Morton codes, sorted order, Karras topology and
refit bounds must equal the oracle's bit for bit (radix_bvh.cpp:32-200)."""
import os

import numpy as np
import pytest

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.mark.parametrize("n", [2, 3, 5, 17, 100, 1000, 65536])
def test_build_soup_matches_oracle(ctx, oracle, n):
    pos = G.random_soup(n, np.random.default_rng(n))
    b, _ = U.gpu_build(ctx, pos)
    U.assert_same_topology(b.topology(), oracle.build_bvh(pos))


def test_build_config0_generator(ctx, oracle):
    """65,536-triangle workload from the device generator (seeded Philox)."""
    import fledge_gb300 as F
    pos = F.gen_triangles(ctx, 65536, 0xF1ED0000)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=2)
    b.build()
    ph = pos.cpu().numpy()
    U.assert_same_topology(b.topology(), oracle.build_bvh(ph))


def test_build_indexed_sphere(ctx, oracle):
    v, ind = G.meshed_sphere(64, 64, 1.0)
    b, _ = U.gpu_build(ctx, v, ind)
    U.assert_same_topology(b.topology(), oracle.build_bvh(v, ind))


def test_build_duplicate_keys(ctx, oracle):
    # Identical triangles: every Morton code equal, delta falls back to the
    # index (radix_bvh.hpp:68-74).
    pos = np.tile(np.array([[0.1, 0.2, 0.3], [0.4, 0.2, 0.3], [0.1, 0.5, 0.3]], np.float32), (4097, 1))
    b, _ = U.gpu_build(ctx, pos)
    U.assert_same_topology(b.topology(), oracle.build_bvh(pos))


def test_build_planar_zero_extent(ctx, oracle):
    pos = G.random_soup(3000, np.random.default_rng(5))
    pos[:, 1] = 0.25
    b, _ = U.gpu_build(ctx, pos)
    U.assert_same_topology(b.topology(), oracle.build_bvh(pos))


def test_build_single_and_empty(ctx, oracle):
    import fledge_gb300 as F
    pos = G.random_soup(1, np.random.default_rng(1))
    b, _ = U.gpu_build(ctx, pos)
    t = b.topology()
    assert t["morton"].shape == (1,) and t["perm"][0] == 0
    e = F.RadixBVHBuilder(F.InternalTriangleMesh(U.dev(np.zeros((0, 3), np.float32))), ctx, node_width=2)
    e.build()
    assert e.info().n_tri == 0


def test_build_golden_fixture(ctx):
    d = np.load(GOLDEN)
    b, _ = U.gpu_build(ctx, d["soup_pos"])
    t = b.topology()
    for k in U.TOPO_KEYS:
        assert np.array_equal(t[k], d["soup_" + k]), k


def test_rebuild_is_deterministic(ctx):
    pos = G.random_soup(200000, np.random.default_rng(9))
    b, (p, _) = U.gpu_build(ctx, pos)
    t1 = b.topology()
    b.build()  # rebuild in place
    t2 = b.topology()
    for k in U.TOPO_KEYS:
        assert np.array_equal(t1[k], t2[k]), k


def test_large_build_properties(ctx):
    """2M triangles: size-independent properties (sorted codes, permutation,
    a valid tree whose root bound is the scene bound)."""
    import fledge_gb300 as F
    n = 1 << 21
    pos = F.gen_triangles(ctx, n, 77)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=2)
    b.build()
    ctx.sync()
    t = b.topology()
    assert np.all(np.diff(t["morton"].astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(t["perm"]), np.arange(n, dtype=np.int32))
    # ties keep ascending original index (stable sort)
    same = t["morton"][1:] == t["morton"][:-1]
    assert np.all(t["perm"][1:][same] > t["perm"][:-1][same])
    assert np.array_equal(t["bounds"][0], t["scene_bound"])
    lo, hi = t["bounds"][:, :3], t["bounds"][:, 3:]
    assert np.all(lo <= hi)
    ph = pos.view(-1, 3, 3)
    assert np.allclose(t["scene_bound"][:3], ph.amin((0, 1)).cpu().numpy(), atol=0)
    assert np.allclose(t["scene_bound"][3:], ph.amax((0, 1)).cpu().numpy(), atol=0)


def test_batched_build_matches_single_scenes(ctx, oracle):
    import fledge_gb300 as F
    rng = np.random.default_rng(17)
    counts = [0, 1, 2, 3, 700, 1, 5000, 0, 12345, 64]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), rng)
    p = U.dev(pos)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(p), offs, ctx, node_width=2)
    bb.build()
    for s, c in enumerate(counts):
        if c == 0:
            continue
        t = bb.topology(s)
        ref = oracle.build_bvh(pos[3 * offs[s]:3 * offs[s + 1]])
        U.assert_same_topology(t, ref)


def test_batched_build_300_scenes(ctx, oracle):
    """More than 256 scenes: two scene-digit sort passes."""
    import fledge_gb300 as F
    rng = np.random.default_rng(23)
    counts = rng.integers(1, 60, size=300)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), rng)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), offs, ctx, node_width=2)
    bb.build()
    for s in (0, 1, 255, 256, 299):
        U.assert_same_topology(bb.topology(s), oracle.build_bvh(pos[3 * offs[s]:3 * offs[s + 1]]))


@pytest.mark.gpu
def test_batched_build_segmented_sort(ctx, oracle):
    """Scenes averaging at least 4 sort tiles (3072 pairs each) are sorted in
    their own runs of tiles, with per-scene digit offsets and look-back
    chains: empty scenes, a one-triangle scene, a scene of exactly one tile,
    one just over a tile boundary and large ones between them."""
    import fledge_gb300 as F
    rng = np.random.default_rng(29)
    counts = [40000, 0, 1, 3072, 3073, 0, 65536, 25000, 2]
    assert sum(counts) >= 4 * 3072 * len(counts)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), rng)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), offs, ctx, node_width=2)
    for _ in range(2):  # a rebuild reuses the per-scene histograms and look-back words
        bb.build()
        for s, c in enumerate(counts):
            if c == 0:
                continue
            U.assert_same_topology(bb.topology(s), oracle.build_bvh(pos[3 * offs[s]:3 * offs[s + 1]]))
