"""Generates tests/golden/golden.npz: seeded small workloads run through the CPU
oracle (oracle/oracle.cpp).  These are regression fixtures for the oracle and
small-size parity fixtures for the GPU path; the independent known answers
(Philox test vectors, the Karras paper tree, Morton bit patterns, exact
Pluecker hits, the watertight-mesh property) live in tests/test_oracle_kat.py.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import oracle as O  # noqa: E402
import geometry as G  # noqa: E402


class Med:
    sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0


def main():
    out = {}
    rng = np.random.default_rng(1)
    pos = G.random_soup(1000, rng)
    tree = O.build_bvh(pos)
    for k in ("morton", "perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds",
              "scene_bound", "codes_unsorted"):
        out["soup_" + k] = tree[k]
    out["soup_pos"] = pos
    rays = G.sphere_rays(2048, np.random.default_rng(2))
    out["soup_rays"] = rays
    for name, mode in (("ref", O.MODE_REF), ("dev", O.MODE_DEV)):
        h = O.trace_closest(pos, None, tree, rays, mode)
        for k in ("prim", "t", "u", "v"):
            out[f"soup_hit_{name}_{k}"] = h[k]
    short = rays.copy()
    short[7] = 1.8
    out["soup_rays_short"] = short
    out["soup_occ"] = O.trace_any(pos, None, tree, short, O.MODE_DEV)

    v, ind = G.meshed_sphere(16, 16, 1.0)
    stree = O.build_bvh(v, ind)
    srays = G.interior_rays(1000, np.random.default_rng(114514))
    sh = O.trace_closest(v, ind, stree, srays, O.MODE_DEV)
    out["sphere_pos"], out["sphere_ind"], out["sphere_rays"] = v, ind, srays
    for k in ("prim", "t", "u", "v"):
        out["sphere_hit_" + k] = sh[k]

    rho = G.value_noise_grid(16, np.random.default_rng(3))
    vr = G.sphere_rays(2048, np.random.default_rng(4))
    seed = 0xF1ED0002
    T, ck = O.volume_tr(rho, [0, 0, 0], [1, 1, 1], Med, vr, seed, want_ckpt=True)
    T64, nrr = O.volume_tr64(rho, [0, 0, 0], [1, 1, 1], Med, vr, seed)
    ok, p, w = O.volume_sample(rho, [0, 0, 0], [1, 1, 1], Med, vr, seed)
    out.update({"vol_rho": rho, "vol_rays": vr, "vol_T": T, "vol_ck_t": ck["t"], "vol_ck_k": ck["k"],
                "vol_ck_c": ck["c"], "vol_T64": T64, "vol_ok": ok, "vol_p": p, "vol_w": w,
                "vol_seed": np.uint64(seed)})
    dLdT = np.random.default_rng(5).random(2048).astype(np.float32)
    out["vol_dLdT"] = dLdT
    out["vol_grad"] = O.volume_tr_adjoint(rho, [0, 0, 0], [1, 1, 1], Med, vr, seed, dLdT)

    g = np.random.default_rng(6).standard_normal((3, 2048)).astype(np.float32)
    prim = out["soup_hit_dev_prim"]
    out["adj_g"] = g
    out["adj_grad"] = O.hit_adjoint64(pos, None, 1000, 3000, rays, prim, g[0], g[1], g[2])
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
