"""The oracle's treelet restructuring (Karras & Aila 2013 over the LBVH):
with no rounds it is the LBVH itself; after three rounds the tree is a valid
Karras-form tree over the depth-first leaf order (node bounds = union of
their range's triangles), its SAH cost is not above the LBVH's, and closest
hits are those of the LBVH (a tree changes only which of two exactly tied
triangles is found first)."""
import numpy as np
import pytest

import geometry as G


def _sah(t, tri):
    lo, hi = tri.min(1), tri.max(1)

    def ha(lo_, hi_):
        d = (hi_ - lo_).astype(np.float64)
        return d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 2] * d[..., 0]
    return 1.2 * ha(t["bounds"][:, :3], t["bounds"][:, 3:]).sum() + ha(lo[t["perm"]], hi[t["perm"]]).sum()


def _valid(t, tri):
    n = t["n"]
    lo, hi = tri.min(1), tri.max(1)
    assert np.array_equal(np.sort(t["perm"]), np.arange(n))
    seen = np.zeros(n, int)
    for i in range(n - 1):
        a, b = min(i, t["range_j"][i]), max(i, t["range_j"][i])
        assert a <= t["split"][i] < b
        ids = t["perm"][a:b + 1]
        assert np.array_equal(t["bounds"][i, :3], lo[ids].min(0)) and np.array_equal(t["bounds"][i, 3:], hi[ids].max(0))
        for side, c in ((0, t["split"][i]), (1, t["split"][i] + 1)):
            if t["leaf_flags"][i] >> side & 1:
                seen[c] += 1
                assert t["leaf_parent"][c] == i
            else:
                assert t["parent"][c] == i
    assert np.all(seen == 1)


def _cases():
    rng = np.random.default_rng(12)
    yield "soup", G.random_soup(20000, rng), None
    v, ind = G.meshed_sphere(60, 60, 1.0)
    yield "sphere", v, ind
    yield "clusters", G.geometric_clusters(24, 40, rng), None
    yield "duplicates", np.tile(G.random_soup(1, rng), (500, 1)), None
    yield "tiny", G.random_soup(9, rng), None


@pytest.mark.parametrize("name,pos,ind", list(_cases()), ids=[c[0] for c in _cases()])
def test_treelet_oracle_properties(oracle, name, pos, ind):
    tri = (pos[ind] if ind is not None else pos.reshape(-1, 3, 3)).astype(np.float32)
    lb = oracle.build_bvh(pos, ind)
    t0 = oracle.build_bvh_treelet(pos, ind, rounds=0)
    for k in ("perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds"):
        assert np.array_equal(np.asarray(t0[k]).reshape(np.asarray(lb[k]).shape), lb[k]), k
    t3 = oracle.build_bvh_treelet(pos, ind, rounds=3)
    _valid(t3, tri)
    assert _sah(t3, tri) <= _sah(t0, tri) * (1 + 1e-6)
    r8 = G.sphere_rays(4000, np.random.default_rng(5), center=tuple(tri.reshape(-1, 3).mean(0)))
    h0 = oracle.trace_closest(pos, ind, lb, r8, oracle.MODE_DEV)
    h3 = oracle.trace_closest(pos, ind, t3, r8, oracle.MODE_DEV)
    diff = h0["prim"] != h3["prim"]
    assert np.array_equal(h0["t"][~diff], h3["t"][~diff])
    assert np.all(h0["t"][diff] == h3["t"][diff])  # only exact ties may differ


def test_treelet_lowers_sah_cost_on_a_mesh(oracle):
    v, ind = G.meshed_sphere(100, 100, 1.0)
    tri = v[ind]
    c0 = _sah(oracle.build_bvh_treelet(v, ind, rounds=0), tri)
    c3 = _sah(oracle.build_bvh_treelet(v, ind, rounds=3), tri)
    assert c3 < 0.97 * c0


def test_treelet_rounds_keep_trees_valid_and_never_raise_cost(oracle):
    """Every round count the builder accepts (1..4) gives a valid tree, and a
    further round never raises the SAH cost: a round only replaces a treelet
    by one of least cost, and an unchanged treelet is among the candidates."""
    pos = G.random_soup(12000, np.random.default_rng(77))
    tri = pos.reshape(-1, 3, 3).astype(np.float32)
    costs = []
    for r in range(5):
        t = oracle.build_bvh_treelet(pos, rounds=r)
        _valid(t, tri)
        costs.append(_sah(t, tri))
    assert all(b <= a * (1 + 1e-6) for a, b in zip(costs, costs[1:])), costs
    assert costs[1] < costs[0]
