"""PLOC trees (FLG_BUILDER_PLOC, the high-quality alternative to the LBVH):
a different tree over the same triangles must give the same closest hits as
the oracle's LBVH traversal (ids equal except recorded exact ties, t/u/v
bit-equal where the ids agree, since the hit arithmetic does not depend on
the tree) and the same occlusion bits, for every node width, single and
batched builds, including empty and one-triangle scenes, and rebuilds."""
import numpy as np
import pytest

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu


def _ploc(ctx, pos, ind=None, width=4, leaf=1):
    import fledge_gb300 as F
    p = U.dev(pos.reshape(-1, 3).astype(np.float32))
    i = None if ind is None else U.dev(ind.reshape(-1, 3).astype(np.int32))
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=width, leaf_size=leaf, builder="ploc")
    b.build()
    return b, (p, i)


@pytest.fixture(scope="module")
def soup(oracle):
    pos = G.random_soup(30000, np.random.default_rng(200))
    rays = G.sphere_rays(1 << 17, np.random.default_rng(201))
    return pos, rays, oracle.build_bvh(pos)


@pytest.mark.parametrize("width,leaf,opts", [(2, 1, {}), (4, 1, {}), (4, 2, {"persistent": 2, "refill_lanes": 8}),
                                             (8, 4, {"persistent": 1, "refill_lanes": 8})])
def test_ploc_closest_matches_oracle(ctx, oracle, soup, width, leaf, opts):
    pos, r8, tree = soup
    b, _ = _ploc(ctx, pos, width=width, leaf=leaf)
    rd, _ = U.rays_dev(r8)
    hg = U.host(b.intersect(rd, **opts))
    ctx.sync()
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    assert (hg["prim"] >= 0).mean() > 0.3
    # a rebuild in place gives the same answers
    b.build()
    hg2 = U.host(b.intersect(rd, **opts))
    ctx.sync()
    assert np.array_equal(hg2["prim"], hg["prim"]) and np.array_equal(hg2["t"], hg["t"])


@pytest.mark.parametrize("width", [2, 4])
def test_ploc_any_hit_matches_oracle(ctx, oracle, soup, width):
    pos, r8, tree = soup
    short = r8.copy()
    short[7] = np.random.default_rng(5).uniform(1.0, 2.5, r8.shape[1]).astype(np.float32)
    b, _ = _ploc(ctx, pos, width=width)
    rd, _ = U.rays_dev(short)
    occ = b.intersectP(rd).cpu().numpy()
    ref = oracle.trace_any(pos, None, tree, short, oracle.MODE_DEV)
    assert np.array_equal(occ, ref), np.count_nonzero(occ != ref)


@pytest.mark.parametrize("w", [2, 4])
def test_ploc_indexed_sphere_watertight_and_oracle(ctx, oracle, w):
    """Triangle.Watertight (shape_tests.cpp:22-48) on an indexed sphere, and
    the oracle's hits for the same rays."""
    v, ind = G.meshed_sphere(128, 128, 1.0)
    b, _ = _ploc(ctx, v, ind, width=w)
    rays = G.interior_rays(50000, np.random.default_rng(7))
    rd, _ = U.rays_dev(rays)
    hg = U.host(b.intersect(rd))
    assert np.all(hg["prim"] >= 0), np.count_nonzero(hg["prim"] < 0)
    tree = oracle.build_bvh(v, ind)
    bad, ties, _ = U.compare_closest(oracle, v, ind, tree, rays, hg, oracle.MODE_DEV)
    assert bad == 0, (bad, ties)


def test_ploc_batched_with_empty_and_single_scenes(ctx, oracle):
    import fledge_gb300 as F
    counts = [1, 0, 2, 1000, 37, 5000, 0, 3]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    roffs = offs * 8
    pos = F.gen_triangles(ctx, int(offs[-1]), 17)
    soa = F.gen_rays(ctx, int(roffs[-1]), 18)
    for width in (2, 4):
        bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(pos), offs, ctx, node_width=width, builder="ploc")
        bb.build()
        rays = F.Rays.from_soa(soa, tmin=1e-4)
        hb = U.host(bb.intersect_batched(rays, roffs, persistent=2, refill_lanes=8))
        ph, rh = pos.cpu().numpy(), soa.cpu().numpy()
        for s in range(len(counts)):
            if counts[s] == 0:
                continue
            sp = ph[3 * offs[s]:3 * offs[s + 1]]
            r8 = np.zeros((8, roffs[s + 1] - roffs[s]), np.float32)
            r8[:6] = rh[:, roffs[s]:roffs[s + 1]]
            r8[6], r8[7] = np.float32(1e-4), np.inf
            tree = oracle.build_bvh(sp)
            hs = {k: v[roffs[s]:roffs[s + 1]] for k, v in hb.items()}
            bad, ties, _ = U.compare_closest(oracle, sp, None, tree, r8, hs, oracle.MODE_DEV)
            assert bad == 0, (width, s, bad, ties)


def test_ploc_has_no_karras_topology(ctx, soup):
    import fledge_gb300 as F
    pos, _, _ = soup
    b, _ = _ploc(ctx, pos[:3000], width=2)
    with pytest.raises(F.FlgError):
        b.topology(0, 1000)
