"""Helpers shared by the GPU parity tests: host<->device conversion through
torch, calls into libflg through the Python mirror, and the comparison rules
(bit-exact integers, recorded ties for closest-hit ids, 1e-5 relative vs the
FP64 oracle for hit values)."""
import numpy as np
import torch

import fledge_gb300 as F


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def rays_dev(r8):
    """[8, n] host rays -> Rays with per-ray tmin/tmax arrays."""
    t = dev(r8.astype(np.float32))
    return F.Rays(*[t[k] for k in range(8)]), t


def host(h):
    return {k: v.cpu().numpy() for k, v in h.items()}


def gpu_build(ctx, pos, ind=None, width=2, leaf=1):
    p = dev(pos.reshape(-1, 3).astype(np.float32))
    i = None if ind is None else dev(ind.reshape(-1, 3).astype(np.int32))
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=width, leaf_size=leaf)
    b.build()
    return b, (p, i)


TOPO_KEYS = ("morton", "perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds", "scene_bound")


def assert_same_topology(gpu, ref):
    for k in TOPO_KEYS:
        a, b = np.asarray(gpu[k]), np.asarray(ref[k])
        if k == "bounds":
            b = b.reshape(a.shape)
        assert a.shape == b.shape, k
        assert np.array_equal(a, b), f"{k}: {np.count_nonzero(a != b)} mismatches"


def compare_closest(oracle, pos, ind, tree, r8, hg, mode, allow_rel=0.0):
    """Returns (n_mismatch, n_ties).  A differing prim id is a tie when both
    triangles hit the ray and their t values agree to allow_rel (0: exactly,
    under the same arithmetic)."""
    ho = oracle.trace_closest(pos, ind, tree, r8, mode)
    diff = np.nonzero(hg["prim"] != ho["prim"])[0]
    ties = 0
    tri = (pos.reshape(-1, 3)[ind.reshape(-1, 3)] if ind is not None else pos.reshape(-1, 3, 3))
    for i in diff:
        pg, po = hg["prim"][i], ho["prim"][i]
        if pg < 0 or po < 0:
            continue
        # both triangles are hit, at the same fp32 distance of the test that
        # selects the closest one (reported t values are refined afterwards)
        okg, tg = oracle.pluecker(tri[pg, 0], tri[pg, 1], tri[pg, 2], r8[0:3, i], r8[3:6, i], mode)
        oko, to = oracle.pluecker(tri[po, 0], tri[po, 1], tri[po, 2], r8[0:3, i], r8[3:6, i], mode)
        if okg and oko and abs(float(tg[0]) - float(to[0])) <= allow_rel * abs(float(to[0])):
            ties += 1
    return len(diff) - ties, ties, ho


def check_t_fp64(oracle, pos, ind, n_tri, r8, hg, rel=1e-5):
    """Hit t, u, v of the GPU against the FP64 oracle on the same triangle:
    t within rel relative; u, v within rel of the barycentric scale (1)."""
    tuv, ok = oracle.hit_values64(pos, ind, n_tri, r8, hg["prim"])
    hit = hg["prim"] >= 0
    assert np.all(ok[hit])
    t64 = tuv[hit, 0]
    assert np.all(np.abs(hg["t"][hit] - t64) <= rel * np.abs(t64)), \
        np.max(np.abs(hg["t"][hit] - t64) / np.abs(t64))
    for k, col in (("u", 1), ("v", 2)):
        assert np.all(np.abs(hg[k][hit] - tuv[hit, col]) <= rel * np.maximum(1.0, np.abs(tuv[hit, col])))
