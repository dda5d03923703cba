"""Wavefront path tracer (flg_pathtrace) against the oracle's restatement of
PathIntegrator::Li with the same Halton sample sequence: an icosphere with
value-noise displacement under a 0.2 x 0.2 area light (config 1 at small
size)."""
import numpy as np
import pytest

from fledge_gb300.scenes import icosphere, quad_light

pytestmark = pytest.mark.gpu


def _scene(level):
    v, f = icosphere(level)
    lv, lf = quad_light()
    pos = np.concatenate([v, lv], 0)
    ind = np.concatenate([f, lf + len(v)], 0)
    return pos, ind, len(f), 2


@pytest.mark.parametrize("width", [2, 4])
def test_pathtrace_matches_oracle(ctx, oracle, width):
    import fledge_gb300 as F
    import gpu_util as U
    pos, ind, lfirst, lcount = _scene(4)
    b, _ = U.gpu_build(ctx, pos, ind, width=width)
    cam = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)
    W, H, spp, depth = 96, 54, 4, 5
    img, stats = F.pathtrace(ctx, b, lfirst, lcount, width=W, height=H, spp=spp, max_depth=depth, **cam)
    ctx.sync()
    g = img.cpu().numpy()
    tree = oracle.build_bvh(pos, ind)
    ref, rays = oracle.pathtrace(pos, ind, tree, lfirst, lcount, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                                 cam["target"], cam["up"], cam["fov_deg"], W, H, spp, depth)
    assert stats["closest_rays"] == rays[0] and abs(stats["shadow_rays"] - rays[1]) <= rays[1] * 1e-3
    err = np.abs(g - ref)
    close = err <= 1e-4 * np.maximum(np.abs(ref), 1.0)
    # paths only diverge where a last-ulp difference of the bounce direction
    # (CUDA's vs libm's cos/sin) changes which triangle is hit
    assert close.mean() > 0.995, close.mean()
    assert abs(g.mean() - ref.mean()) <= 1e-3 * ref.mean()
    assert ref.mean() > 1e-4 and (ref > 0).mean() > 0.03


def _medium_grid(n=24):
    z, y, x = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    return (0.3 * (1.0 + 0.5 * np.sin(7 * x) * np.cos(5 * y) * np.sin(3 * z + 1))).astype(np.float32)


@pytest.mark.parametrize("g", [0.3, 0.0])
def test_volpath_matches_oracle(ctx, oracle, g):
    """Volumetric path tracing (VolPathIntegrator::Li): the medium fills a
    box around the sphere; delta tracking along every segment, HG
    scattering, ratio-tracked shadow rays, all on the oracle's Philox
    streams."""
    import torch
    import fledge_gb300 as F
    import gpu_util as U
    pos, ind, lfirst, lcount = _scene(4)
    b, _ = U.gpu_build(ctx, pos, ind, width=4)
    rho = _medium_grid()
    lo, hi = (-1.5, -1.5, -1.5), (1.5, 1.5, 1.5)
    vol = F.DenseGridVolume(torch.from_numpy(rho).cuda(), lo, hi, F.Medium(0.8, 0.2, g), ctx)
    cam = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)
    W, H, spp, depth, seed = 96, 54, 4, 5, 0xF1ED0001
    img, stats = F.pathtrace(ctx, b, lfirst, lcount, width=W, height=H, spp=spp, max_depth=depth, volume=vol,
                             seed=seed, **cam)
    ctx.sync()
    gi = img.cpu().numpy()
    tree = oracle.build_bvh(pos, ind)
    ref, rays = oracle.pathtrace(pos, ind, tree, lfirst, lcount, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                                 cam["target"], cam["up"], cam["fov_deg"], W, H, spp, depth,
                                 grid=(rho, lo, hi, oracle.Medium(0.8, 0.2, g, 0.1, 0.0)), seed=seed)
    assert abs(stats["closest_rays"] - rays[0]) <= rays[0] * 1e-3
    assert abs(stats["shadow_rays"] - rays[1]) <= rays[1] * 1e-3
    err = np.abs(gi - ref)
    close = err <= 1e-4 * np.maximum(np.abs(ref), 1.0)
    assert close.mean() > 0.99, close.mean()
    assert abs(gi.mean() - ref.mean()) <= 2e-3 * ref.mean()
    # the medium scatters light into pixels the surface-only image leaves dark
    surf, _ = oracle.pathtrace(pos, ind, tree, lfirst, lcount, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                               cam["target"], cam["up"], cam["fov_deg"], W, H, spp, depth)
    assert (ref > 0).mean() > (surf > 0).mean() + 0.02


def _mesh_medium_scene():
    from fledge_gb300.scenes import icosphere, quad_light
    v, f = icosphere(3)
    bv, bf = icosphere(2, radius=1.5, amplitude=0.0)  # the medium's boundary, outward normals
    lv, lf = quad_light()
    pos = np.concatenate([v, bv, lv], 0)
    ind = np.concatenate([f, bf + len(v), lf + len(v) + len(bv)], 0)
    return pos, ind, len(f), len(bf), len(f) + len(bf)


@pytest.mark.parametrize("g", [0.3, -0.5])
def test_volpath_mesh_medium_matches_oracle(ctx, oracle, g):
    """A homogeneous medium bounded by a closed mesh (the reference's HVolume
    attached to a mesh, scene.cpp:224-228): the sphere under the light sits
    inside a larger sphere whose triangles are material-less boundaries.
    Paths pass through them, scatter inside by HVolume::sample, and shadow
    rays attenuate through them as VolEstimateTr does; the image equals the
    oracle's restatement."""
    import fledge_gb300 as F
    import gpu_util as U
    pos, ind, first, count, lfirst = _mesh_medium_scene()
    b, _ = U.gpu_build(ctx, pos, ind, width=4)
    mm = dict(first=first, count=count, sigma_s=(0.5, 0.6, 0.7), sigma_a=(0.05, 0.05, 0.05), g=g, density=1.0)
    cam = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)
    W, H, spp, depth, seed = 96, 54, 4, 5, 0xF1ED0007
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=W, height=H, spp=spp, max_depth=depth, seed=seed,
                             mesh_medium=mm, **cam)
    ctx.sync()
    gi = img.cpu().numpy()
    tree = oracle.build_bvh(pos, ind)
    ref, rays = oracle.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                                 cam["target"], cam["up"], cam["fov_deg"], W, H, spp, depth, seed=seed,
                                 mesh_medium=(first, count, mm["sigma_s"], mm["sigma_a"], g, 1.0))
    assert abs(stats["closest_rays"] - rays[0]) <= rays[0] * 1e-3
    assert abs(stats["shadow_rays"] - rays[1]) <= rays[1] * 1e-3
    close = np.abs(gi - ref) <= 1e-4 * np.maximum(np.abs(ref), 1.0)
    assert close.mean() > 0.99, close.mean()
    assert np.all(np.abs(gi.mean(axis=(0, 1)) - ref.mean(axis=(0, 1))) <= 2e-3 * ref.mean(axis=(0, 1)))
    # light reaches the camera through the boundary, scattered by the medium
    assert (ref > 0).mean() > 0.3
    # the boundary is not opaque: with it as a plain surface almost nothing is lit
    opaque, _ = oracle.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                                 cam["target"], cam["up"], cam["fov_deg"], W, H, spp, depth)
    assert (ref > 0).mean() > (opaque > 0).mean() + 0.2
