"""GPU treelet restructuring (FLG_BUILDER_TREELET) against the oracle's
restatement: after the LBVH and three restructuring rounds (or the number
that treelet_rounds asks for) the leaf order,
topology (split, leaf flags, range end, parents) and node bounds are
bit-exact, for single scenes and per scene of a batched build; closest hits
over every layout equal the oracle's except recorded exact ties; rebuilds
and graph replay give the same tree."""
import ctypes as C

import numpy as np
import pytest
import torch

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu
KEYS = ("perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds", "scene_bound")


def _build(ctx, pos, ind=None, width=2, leaf=1, rounds=0):
    import fledge_gb300 as F
    p = U.dev(pos.reshape(-1, 3).astype(np.float32))
    i = None if ind is None else U.dev(ind.reshape(-1, 3).astype(np.int32))
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=width, leaf_size=leaf, builder="treelet",
                          treelet_rounds=rounds)
    b.build()
    return b, (p, i)


def _same(gpu, ref):
    for k in KEYS:
        a, b = np.asarray(gpu[k]), np.asarray(ref[k])
        assert np.array_equal(a, b.reshape(a.shape)), f"{k}: {np.count_nonzero(a != b.reshape(a.shape))} differ"


@pytest.mark.parametrize("n", [2, 3, 7, 8, 100, 5000, 65536, 400000])
def test_treelet_soup_matches_oracle(ctx, oracle, n):
    pos = G.random_soup(n, np.random.default_rng(300 + n))
    b, _ = _build(ctx, pos)
    _same(b.topology(), oracle.build_bvh_treelet(pos))


@pytest.mark.parametrize("rounds", [1, 2, 4])
def test_treelet_rounds_match_oracle(ctx, oracle, rounds):
    """treelet_rounds: one, two or four passes (thresholds 7, 14, 28, 56
    triangles) give the oracle's tree after the same number of passes."""
    pos = G.random_soup(70000, np.random.default_rng(900 + rounds))
    b, _ = _build(ctx, pos, rounds=rounds)
    _same(b.topology(), oracle.build_bvh_treelet(pos, rounds=rounds))


@pytest.mark.parametrize("rounds", [-1, 5])
def test_treelet_rounds_out_of_range_rejected(ctx, rounds):
    import fledge_gb300 as F
    from fledge_gb300 import _lib
    p = U.dev(G.random_soup(100, np.random.default_rng(1)).reshape(-1, 3).astype(np.float32))
    h = C.c_void_p()
    opts = F.FlgBuildOpts(4, 1, 1, _lib.FLG_BUILDER_TREELET, rounds)
    rc = ctx.lib.flg_bvh_build(ctx.h, C.c_void_p(p.data_ptr()), None, 100, 300, C.byref(opts), C.byref(h))
    assert rc == _lib.FLG_ERR_ARG and not h.value


@pytest.mark.parametrize("case", ["sphere", "clusters", "duplicates", "lattice"])
def test_treelet_special_inputs_match_oracle(ctx, oracle, case):
    rng = np.random.default_rng(7)
    ind = None
    if case == "sphere":
        pos, ind = G.meshed_sphere(120, 120, 1.0)
    elif case == "clusters":
        pos = G.geometric_clusters(40, 60, rng)
    elif case == "lattice":
        # equal triangles on an integer lattice: many splits of a treelet
        # cost exactly the same, so the first-minimum rule decides
        g = np.stack(np.meshgrid(*[np.arange(20, dtype=np.float32)] * 3, indexing="ij"), -1).reshape(-1, 1, 3)
        tri = np.array([[0, 0, 0], [0.5, 0, 0], [0, 0.5, 0.25]], np.float32)
        pos = (g + tri).reshape(-1, 3)
    else:
        pos = np.concatenate([np.tile(G.random_soup(1, rng), (3000, 1)), G.random_soup(500, rng)])
    b, _ = _build(ctx, pos, ind)
    _same(b.topology(), oracle.build_bvh_treelet(pos, ind))


@pytest.mark.parametrize("width,leaf,opts", [(2, 1, {}), (4, 1, {}), (4, 4, {"persistent": 2, "refill_lanes": 8}),
                                             (8, 2, {"persistent": 1, "refill_lanes": 16})])
def test_treelet_hits_match_oracle(ctx, oracle, width, leaf, opts):
    pos = G.random_soup(100000, np.random.default_rng(9))
    tree = oracle.build_bvh_treelet(pos)
    b, _ = _build(ctx, pos, width=width, leaf=leaf)
    r8 = G.sphere_rays(1 << 17, np.random.default_rng(10))
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, **opts))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} mismatches ({ties} ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    occ = b.intersectP(rd, **opts).cpu().numpy().astype(bool)
    assert np.array_equal(occ, ho["prim"] >= 0)


def test_treelet_batched_scenes_match_oracle(ctx, oracle):
    import fledge_gb300 as F
    counts = [30000, 0, 1, 2, 7, 3072, 50000, 12]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), np.random.default_rng(11))
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), offs, ctx, node_width=4, leaf_size=3,
                                  builder="treelet")
    for _ in range(2):  # a rebuild gives the same trees
        bb.build()
        for s, c in enumerate(counts):
            if c == 0:
                continue
            _same(bb.topology(s), oracle.build_bvh_treelet(pos[3 * offs[s]:3 * offs[s + 1]]))
    ctx.sync()


def test_treelet_graph_capture_replay(ctx, oracle):
    """Treelet builds need no host synchronisation: a rebuild captured into a
    graph and replayed over new vertices gives the oracle's tree."""
    import fledge_gb300 as F
    n = 40000
    pos = F.gen_triangles(ctx, n, 21)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=2, builder="treelet")
    b.build()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    ctx2 = F.Context(0, s)
    g = C.c_void_p()
    with torch.cuda.stream(s):
        ctx2.check(ctx2.lib.flg_graph_begin(ctx2.h))
        ctx2.check(ctx2.lib.flg_bvh_rebuild(ctx2.h, b.h, C.c_void_p(pos.data_ptr())))
        ctx2.check(ctx2.lib.flg_graph_end(ctx2.h, C.byref(g)))
    for trial in range(2):
        pos.copy_(F.gen_triangles(ctx, n, 500 + trial))
        torch.cuda.synchronize()
        ctx2.check(ctx2.lib.flg_graph_launch(ctx2.h, g))
        ctx2.sync()
        _same(b.topology(), oracle.build_bvh_treelet(pos.cpu().numpy()))
    ctx2.lib.flg_graph_destroy(g)
    ctx2.close()
