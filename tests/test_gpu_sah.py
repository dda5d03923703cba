"""Binned-SAH trees (FLG_BUILDER_SAH, BasicBVHBuilder's ESAH rule at every
node): the downloaded topology, triangle order and node bounds equal the
oracle's restatement bit for bit (single and batched builds, degenerate
inputs, rebuilds), and traversal over them gives the oracle's closest hits
(ids equal except recorded exact ties) and occlusion bits for every node
width."""
import numpy as np
import pytest

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu

SAH_KEYS = ("perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds", "scene_bound")


def _sah(ctx, pos, ind=None, width=4, leaf=1):
    import fledge_gb300 as F
    p = U.dev(pos.reshape(-1, 3).astype(np.float32))
    i = None if ind is None else U.dev(ind.reshape(-1, 3).astype(np.int32))
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=width, leaf_size=leaf, builder="sah")
    b.build()
    return b, (p, i)


def _same(gpu, ref):
    for k in SAH_KEYS:
        a, b = np.asarray(gpu[k]), np.asarray(ref[k])
        assert np.array_equal(a, b.reshape(a.shape)), f"{k}: {np.count_nonzero(a != b.reshape(a.shape))} mismatches"


def _cases():
    rng = np.random.default_rng(300)
    yield "soup_2", G.random_soup(2, rng), None
    yield "soup_9", G.random_soup(9, rng), None
    yield "soup_33", G.random_soup(33, rng), None
    yield "soup_5000", G.random_soup(5000, rng), None
    yield "soup_120000", G.random_soup(120000, rng), None
    yield "wide_soup_20000", G.random_soup(20000, rng, half=0.2), None
    yield "duplicates_700", np.tile(G.random_soup(1, rng), (700, 1)), None
    flat = G.random_soup(30000, rng)
    flat.reshape(-1, 3)[:, 1] = 0.5
    yield "planar_30000", flat, None
    yield "deep_1000", G.geometric_clusters(100, 10, rng), None  # nodes past the depth limit of 26
    v, ind = G.meshed_sphere(96, 96, 1.0)
    yield "sphere", v, ind


@pytest.mark.parametrize("name,pos,ind", list(_cases()), ids=[c[0] for c in _cases()])
def test_sah_topology_matches_oracle(ctx, oracle, name, pos, ind):
    b, _ = _sah(ctx, pos, ind, width=2)
    ref = oracle.build_bvh_sah(pos, ind)
    _same(b.topology(), ref)
    b.build()  # a rebuild gives the same tree
    _same(b.topology(), ref)


def test_sah_batched_matches_per_scene_oracle(ctx, oracle):
    import fledge_gb300 as F
    counts = [1, 0, 2, 9, 5000, 37, 0, 40000, 3]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), np.random.default_rng(301))
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), offs, ctx, node_width=4, builder="sah")
    for _ in range(2):
        bb.build()
        for s, c in enumerate(counts):
            if c == 0:
                continue
            _same(bb.topology(s), oracle.build_bvh_sah(pos[3 * offs[s]:3 * offs[s + 1]]))


@pytest.fixture(scope="module")
def soup(oracle):
    pos = G.random_soup(30000, np.random.default_rng(302))
    rays = G.sphere_rays(1 << 17, np.random.default_rng(303))
    return pos, rays, oracle.build_bvh_sah(pos)


@pytest.mark.parametrize("width,leaf,opts", [(2, 1, {}), (4, 1, {}), (4, 3, {"persistent": 2, "refill_lanes": 16}),
                                             (8, 4, {"persistent": 1, "refill_lanes": 8})])
def test_sah_closest_matches_oracle(ctx, oracle, soup, width, leaf, opts):
    pos, r8, tree = soup
    b, _ = _sah(ctx, pos, width=width, leaf=leaf)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, **opts))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    assert (hg["prim"] >= 0).mean() > 0.3


@pytest.mark.parametrize("width", [2, 4])
def test_sah_any_hit_matches_oracle(ctx, oracle, soup, width):
    pos, r8, tree = soup
    short = r8.copy()
    short[7] = np.random.default_rng(6).uniform(1.0, 2.5, r8.shape[1]).astype(np.float32)
    b, _ = _sah(ctx, pos, width=width)
    rd, _ = U.rays_dev(short)
    occ = b.intersectP(rd).cpu().numpy()
    ref = oracle.trace_any(pos, None, tree, short, oracle.MODE_DEV)
    assert np.array_equal(occ, ref), np.count_nonzero(occ != ref)


def test_sah_large_build_agrees_with_lbvh_hits(ctx):
    """2M triangles: the download's consistency checks pass, and closest
    hits through the SAH tree equal those through the LBVH (same triangles,
    so the same nearest hit whatever the tree, up to exact ties)."""
    import fledge_gb300 as F
    n = 2_000_000
    pos = F.gen_triangles(ctx, n, 11)
    soa = F.gen_rays(ctx, 1 << 20, 12)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    mesh = F.InternalTriangleMesh(pos)
    sah = F.RadixBVHBuilder(mesh, ctx, node_width=4, leaf_size=3, builder="sah")
    sah.build()
    lb = F.RadixBVHBuilder(mesh, ctx, node_width=4, leaf_size=3)
    lb.build()
    hs = U.host(sah.intersect(rays, persistent=2, refill_lanes=16))
    hl = U.host(lb.intersect(rays, persistent=2, refill_lanes=16))
    ctx.sync()
    t = sah.topology(0, n)
    assert np.array_equal(np.sort(t["perm"]), np.arange(n))
    diff = hs["prim"] != hl["prim"]
    assert np.count_nonzero(diff) <= 16, np.count_nonzero(diff)
    assert (hs["prim"] >= 0).mean() > 0.1


def test_sah_build_is_not_capturable(ctx):
    import ctypes as C

    import torch

    import fledge_gb300 as F
    pos = G.random_soup(1000, np.random.default_rng(4))
    b, (p, _) = _sah(ctx, pos, width=4)
    s = torch.cuda.Stream()
    ctx2 = F.Context(0, s)
    with torch.cuda.stream(s):
        ctx2.check(ctx2.lib.flg_graph_begin(ctx2.h))
        rc = ctx2.lib.flg_bvh_rebuild(ctx2.h, b.h, C.c_void_p(p.data_ptr()))
        g = C.c_void_p()
        ctx2.lib.flg_graph_end(ctx2.h, C.byref(g))
    assert rc == F._lib.FLG_ERR_STATE
    if g.value:
        ctx2.lib.flg_graph_destroy(g)
    ctx2.close()
