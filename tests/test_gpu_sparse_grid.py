"""Sparse brick grid (flg_grid_create_sparse / flg_grid_sparsify, the
NanoVDBVolume declared in volume.hpp:72-92): the same densities behind a
brick table must give bit-identical transmittance, checkpoints, collisions
and adjoint gradients (on the stored voxels) as the dense grid, and the same
volumetric path-traced image."""
import numpy as np
import pytest
import torch

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu


def _masked_noise(ctx, n=61):
    import fledge_gb300 as F
    rho = F.gen_noise_grid(ctx, n, 0xF1ED0002)
    # empty out a checkerboard of 8^3 bricks (and a whole slab) so that the
    # table has holes; n = 61 leaves partial bricks at the far edges
    z, y, x = torch.meshgrid(*[torch.arange(n, device=rho.device) // 8] * 3, indexing="ij")
    rho[((x + y + z) % 2 == 0) | (z == 3)] = 0.0
    return rho


def test_sparsify_roundtrip_and_table(ctx):
    import fledge_gb300 as F
    rho = _masked_noise(ctx)
    sv = F.SparseGridVolume.from_dense(rho, ctx=ctx)
    bi = sv.brick_index.cpu().numpy()
    assert bi.shape == (8, 8, 8)
    occ = bi >= 0
    assert 0 < occ.sum() < bi.size
    # slots are dense and in brick order
    assert np.array_equal(np.sort(bi[occ]), np.arange(occ.sum()))
    assert np.array_equal(bi[occ], np.arange(occ.sum()))
    assert torch.equal(sv.to_dense(), rho)
    assert sv.majorant() == float(rho.max())


def test_sparse_tr_sample_bit_identical(ctx):
    import fledge_gb300 as F
    rho = _masked_noise(ctx)
    med = F.Medium(0.8, 0.2, 0.3)
    dv = F.DenseGridVolume(rho, (0, 0, 0), (1, 1, 1), med, ctx)
    sv = F.SparseGridVolume.from_dense(rho, (0, 0, 0), (1, 1, 1), med, ctx)
    r8 = G.sphere_rays(1 << 16, np.random.default_rng(7))
    rd, _ = U.rays_dev(r8)
    Td, ckd = dv.tr(rd, 11, checkpoint=True)
    Ts, cks = sv.tr(rd, 11, checkpoint=True)
    assert torch.equal(Td, Ts)
    for k in ("t", "k", "c"):
        assert torch.equal(ckd[k], cks[k])
    assert (Td < 1).float().mean() > 0.2  # the medium is not trivially thin
    okd, pd, wd = dv.sample(rd, 12)
    oks, ps, ws = sv.sample(rd, 12)
    assert torch.equal(okd, oks) and torch.equal(pd, ps) and torch.equal(wd, ws)


def test_sparse_adjoint_matches_dense_on_stored_voxels(ctx):
    import fledge_gb300 as F
    rho = _masked_noise(ctx)
    med = F.Medium(0.8, 0.2, 0.3)
    dv = F.DenseGridVolume(rho, (0, 0, 0), (1, 1, 1), med, ctx)
    sv = F.SparseGridVolume.from_dense(rho, (0, 0, 0), (1, 1, 1), med, ctx)
    r8 = G.sphere_rays(1 << 15, np.random.default_rng(8))
    rd, _ = U.rays_dev(r8)
    T, ck = dv.tr(rd, 21, checkpoint=True)
    g = torch.randn_like(T)
    gd = dv.tr_adjoint(rd, 21, g, T, ck)
    gs = sv.tr_adjoint(rd, 21, g, T, ck)
    assert gs.shape == sv.density.shape
    stored = sv.to_dense(torch.ones_like(sv.density)) > 0
    gsd = sv.to_dense(gs)
    # same atomics in a different memory layout: equal up to summation order
    assert torch.allclose(gsd[stored], gd[stored], rtol=1e-5, atol=1e-6)
    assert float(gd[stored].abs().sum()) > 0


def test_sparse_volpath_image_matches_dense(ctx):
    import fledge_gb300 as F
    from fledge_gb300.scenes import icosphere, quad_light
    v, f = icosphere(3)
    lv, lf = quad_light()
    pos = np.concatenate([v, lv], 0)
    ind = np.concatenate([f, lf + len(v)], 0)
    b, _ = U.gpu_build(ctx, pos, ind, width=4)
    rho = _masked_noise(ctx, 40) * 0.3
    med = F.Medium(0.8, 0.2, 0.3)
    lo, hi = (-1.5, -1.5, -1.5), (1.5, 1.5, 1.5)
    dv = F.DenseGridVolume(rho, lo, hi, med, ctx)
    sv = F.SparseGridVolume.from_dense(rho, lo, hi, med, ctx)
    cam = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)
    a, sa = F.pathtrace(ctx, b, len(f), 2, width=64, height=36, spp=2, max_depth=4, volume=dv, seed=5, **cam)
    c, sc = F.pathtrace(ctx, b, len(f), 2, width=64, height=36, spp=2, max_depth=4, volume=sv, seed=5, **cam)
    ctx.sync()
    assert sa == sc
    assert torch.allclose(a, c, rtol=1e-5, atol=1e-7)


class _Med:
    sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0


def test_sparse_matches_oracle(ctx, oracle):
    """The sparse grid against the oracle directly (on the dense values that
    its bricks hold): ratio-tracking T and checkpoints bit-equal, delta
    tracking collisions bit-equal, the adjoint within 1e-4 of the oracle's
    analytic gradient on every stored voxel."""
    import fledge_gb300 as F
    rho = _masked_noise(ctx)
    sv = F.SparseGridVolume.from_dense(rho, (0, 0, 0), (1, 1, 1), F.Medium(0.8, 0.2, 0.3), ctx)
    dense = sv.to_dense().cpu().numpy()
    r8 = G.sphere_rays(1 << 16, np.random.default_rng(17))
    rd, _ = U.rays_dev(r8)
    T, ck = sv.tr(rd, 31, checkpoint=True)
    ok, p, w = sv.sample(rd, 32)
    ctx.sync()
    To, cko = oracle.volume_tr(dense, [0, 0, 0], [1, 1, 1], _Med, r8, 31, want_ckpt=True)
    assert np.array_equal(T.cpu().numpy(), To)
    assert np.array_equal(ck["k"].cpu().numpy().view(np.uint32), cko["k"])
    assert np.array_equal(ck["t"].cpu().numpy(), cko["t"]) and np.array_equal(ck["c"].cpu().numpy(), cko["c"])
    oko, po, wo = oracle.volume_sample(dense, [0, 0, 0], [1, 1, 1], _Med, r8, 32)
    assert np.array_equal(ok.cpu().numpy(), oko)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(w.cpu().numpy(), wo)
    assert 0.1 < oko.mean() < 0.99 and (To < 1).mean() > 0.2
    m = 1 << 14
    dL = torch.rand(m, generator=torch.Generator().manual_seed(5)).cuda()
    rs, _ = U.rays_dev(r8[:, :m])
    Ts, cks = sv.tr(rs, 33, checkpoint=True)
    gs = sv.to_dense(sv.tr_adjoint(rs, 33, dL, Ts, cks)).cpu().numpy().astype(np.float64)
    go = oracle.volume_tr_adjoint(dense, [0, 0, 0], [1, 1, 1], _Med, r8[:, :m], 33, dL.cpu().numpy())
    stored = sv.to_dense(torch.ones_like(sv.density)).cpu().numpy() > 0
    scale = np.abs(go).max()
    assert scale > 0 and np.max(np.abs(gs[stored] - go[stored])) <= 1e-4 * scale
    # voxels of dropped bricks are not parameters: the oracle's gradient there
    # is what the dense grid would have received; the sparse grid has none
    assert np.all(gs[~stored] == 0)
