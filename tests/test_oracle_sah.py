"""The oracle's binned-SAH build (BasicBVHBuilder::recursiveBuilder with
EBVHPartitionMethod::ESAH, src/experimental/base_bvh.cpp:33-173) against a
second, independent restatement written here in numpy float32 scalars, on
small random, duplicate and planar inputs.  The reference builder needs
Embree and TBB and is not compiled here, so these two restatements pin each
other; the GPU builder is then compared bit-exactly with the oracle."""
import numpy as np
import pytest

import geometry as G

F32 = np.float32
FMAX = F32(np.finfo(np.float32).max)


def _area(lo, hi):
    ex, ey, ez = hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]
    return F32(2) * ((ex * ey + ex * ez) + ey * ez)


def _bucket(c, lo, hi):
    f = np.floor(((c - lo) / (hi - lo)) * F32(16))
    if f >= 0:
        return int(f) if f < 16 else 15
    return 0


def sah_py(pos):
    tri = pos.reshape(-1, 3, 3).astype(np.float32)
    n = tri.shape[0]
    tlo, thi = tri.min(axis=1), tri.max(axis=1)
    cen = ((tri[:, 0] + tri[:, 1]) + tri[:, 2]) / F32(3)
    order = list(range(n))
    m = max(n - 1, 0)
    out = {"split": np.zeros(m, np.int32), "leaf_flags": np.zeros(m, np.uint8), "range_j": np.zeros(m, np.int32),
           "parent": np.zeros(m, np.int32), "leaf_parent": np.zeros(n, np.int32),
           "bounds": np.zeros((m, 6), np.float32)}

    def union(ids):
        lo = np.full(3, FMAX, np.float32)
        hi = np.full(3, -FMAX, np.float32)
        for t in ids:
            lo = np.minimum(lo, tlo[t])
            hi = np.maximum(hi, thi[t])
        return lo, hi

    def node(f, cnt, depth, sah, slot):
        ids = order[f:f + cnt]
        blo, bhi = union(ids)
        h = -1
        if sah and not (cnt <= 8 or depth >= 26):
            a = depth % 3
            bk = [_bucket(cen[t, a], blo[a], bhi[a]) for t in ids]
            best, bi = FMAX, 0
            for i in range(1, 15):
                left = [t for t, b in zip(ids, bk) if b <= i]
                right = [t for t, b in zip(ids, bk) if b > i]
                q = (_area(*union(left)) * F32(len(left)) + _area(*union(right)) * F32(len(right))) / _area(blo, bhi)
                cost = F32(np.float64(0.125) + np.float64(q))
                if cost < best:
                    best, bi = cost, i
            if best < F32(cnt):
                left = [t for t, b in zip(ids, bk) if b <= bi]
                right = [t for t, b in zip(ids, bk) if b > bi]
                order[f:f + cnt] = left + right
                h = len(left)
        child_sah = sah and h >= 0
        if h < 0:
            h = cnt // 2
        mid = f + h
        llo, lhi = union(order[f:mid])
        rlo, rhi = union(order[mid:f + cnt])
        out["split"][slot] = mid - 1
        out["leaf_flags"][slot] = (1 if h == 1 else 0) | (2 if cnt - h == 1 else 0)
        out["range_j"][slot] = f + cnt - 1 if slot == f else f
        out["bounds"][slot] = np.concatenate([np.minimum(llo, rlo), np.maximum(lhi, rhi)])
        if h == 1:
            out["leaf_parent"][f] = slot
        else:
            out["parent"][mid - 1] = slot
        if cnt - h == 1:
            out["leaf_parent"][mid] = slot
        else:
            out["parent"][mid] = slot
        if h >= 2:
            node(f, h, depth + 1, child_sah, mid - 1)
        if cnt - h >= 2:
            node(mid, cnt - h, depth + 1, child_sah, mid)

    if n >= 2:
        node(0, n, 0, True, 0)
    elif n == 1:
        out["leaf_parent"][0] = -1
    out["perm"] = np.asarray(order, np.int32)
    return out


def _cases():
    rng = np.random.default_rng(41)
    yield "soup", G.random_soup(150, rng)
    yield "wide_soup", G.random_soup(60, rng, half=0.3)
    dup = np.tile(G.random_soup(1, rng), (40, 1))
    yield "duplicates", dup
    flat = G.random_soup(90, rng)
    flat.reshape(-1, 3)[:, 2] = 0.25
    yield "planar", flat
    yield "deep", G.geometric_clusters(60, 12, rng)  # reaches the depth limit of 26
    yield "nine", G.random_soup(9, rng)
    yield "two", G.random_soup(2, rng)
    yield "one", G.random_soup(1, rng)


@pytest.mark.parametrize("name,pos", list(_cases()), ids=[c[0] for c in _cases()])
def test_oracle_sah_matches_numpy_restatement(oracle, name, pos):
    with np.errstate(all="ignore"):
        ref = sah_py(pos)
    got = oracle.build_bvh_sah(pos)
    for k in ("perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds"):
        assert np.array_equal(got[k], ref[k].reshape(got[k].shape)), k


def test_oracle_sah_tree_is_a_partition(oracle):
    """Every position is one leaf of exactly one node; node bounds contain
    their triangles; the tree differs from the Morton-order LBVH."""
    pos = G.random_soup(3000, np.random.default_rng(9))
    t = oracle.build_bvh_sah(pos)
    n = 3000
    assert np.array_equal(np.sort(t["perm"]), np.arange(n))
    lp = t["leaf_parent"]
    assert np.all((lp >= 0) & (lp < n - 1))
    leaves = np.zeros(n, np.int32)
    for i in range(n - 1):
        for side in (0, 1):
            if t["leaf_flags"][i] & (1 << side):
                leaves[t["split"][i] + side] += 1
    assert np.all(leaves == 1)
    tri = pos.reshape(-1, 3, 3)[t["perm"]]
    root_lo, root_hi = t["bounds"][0, :3], t["bounds"][0, 3:]
    assert np.all(tri.min(axis=(0, 1)) == root_lo) and np.all(tri.max(axis=(0, 1)) == root_hi)
    lb = oracle.build_bvh(pos)
    assert not np.array_equal(lb["split"], t["split"])
