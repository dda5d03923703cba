"""Generates tests/golden/reference_lbvh.npz from the reference's own code:
RadixBVHBuilder (src/experimental/radix_bvh.cpp of the fledge project),
compiled unchanged into oracle/_ref/libfledge_ref.so (oracle/ref_driver.cpp,
`make -C oracle ref`).  The fixture carries its inputs, so the GPU tests can
compare the CUDA build with the reference's arrays on a machine without the
reference sources.

Scenes: a config-0 style soup of 2048 triangles (centroids U[0,1]^3, vertices
within +-0.01) with 2048 rays from the radius-2 sphere, and the reference's
MakeMeshedSphere(24, 24, 1) (indexed) with 2048 interior rays.  Stored per
scene: inputs, the builder's arrays (sorted Morton codes, leaf order as
original triangle ids, split, leaf flags, j - i + 1, direction, parents, node
bounds, scene bound) and RadixBVHBuilder::intersect's hit, tfar and hit_ng.

Run from the repository root, where the reference sources are present:
    python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import reference as R  # noqa: E402
import geometry as G  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_lbvh.npz")
FLT_MAX = np.finfo(np.float32).max


def scene(out, name, pos, ind, rays):
    r = R.RadixBVH(pos, ind)
    a = r.arrays()
    h = r.intersect(rays)
    r.close()
    out[name + "_pos"] = pos
    if ind is not None:
        out[name + "_ind"] = ind
    out[name + "_rays"] = rays
    for k, v in a.items():
        out[f"{name}_{k}"] = v
    for k in ("hit", "tfar", "ng"):
        out[f"{name}_ref_{k}"] = h[k]


def main():
    if not R.build():
        raise SystemExit("the reference sources are needed to build oracle/_ref")
    out = {}
    pos = G.random_soup(2048, np.random.default_rng(0xF1ED0000))
    rays = G.sphere_rays(2048, np.random.default_rng(0xF1ED0001), tmin=0.0, tmax=FLT_MAX)
    scene(out, "soup", pos, None, rays)
    v, ind = G.meshed_sphere(24, 24, 1.0)
    srays = G.interior_rays(2048, np.random.default_rng(114514))
    srays[7] = FLT_MAX
    scene(out, "sphere", v, ind, srays)
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
