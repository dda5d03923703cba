"""GPU participating-media parity: ratio tracking (OpenVDBVolume::tr,
volume.cpp:75-107), delta tracking (OpenVDBVolume::sample, :109-148) and the
ratio-tracking adjoint.  Same Philox streams and the same fp32 arithmetic as
the oracle, so T, checkpoints and collisions are bit-equal; FP64 agreement is
1e-5 relative; gradients match FP64 finite differences to 1e-3."""
import os

import numpy as np
import pytest
import torch

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


class Med:
    sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0


def _vol(ctx, rho, med=Med):
    import fledge_gb300 as F
    m = F.Medium(med.sigma_s, med.sigma_a, med.g, med.rr_threshold, med.majorant)
    return F.DenseGridVolume(U.dev(rho), (0, 0, 0), (1, 1, 1), m, ctx)


def test_tr_golden_fixture(ctx):
    d = np.load(GOLDEN)
    v = _vol(ctx, d["vol_rho"])
    rd, _ = U.rays_dev(d["vol_rays"])
    T, ck = v.tr(rd, int(d["vol_seed"]), checkpoint=True)
    assert np.array_equal(T.cpu().numpy(), d["vol_T"])
    assert np.array_equal(ck["k"].cpu().numpy().view(np.uint32), d["vol_ck_k"])
    assert np.array_equal(ck["t"].cpu().numpy(), d["vol_ck_t"])
    ok, p, w = v.sample(rd, int(d["vol_seed"]))
    assert np.array_equal(ok.cpu().numpy(), d["vol_ok"]) and np.array_equal(p.cpu().numpy(), d["vol_p"])


@pytest.mark.parametrize("rr", [0.1, 0.0])
def test_tr_matches_oracle_and_fp64(ctx, oracle, rr):
    import fledge_gb300 as F
    rho = F.gen_noise_grid(ctx, 64, 0xF1ED0002).cpu().numpy()
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=rr, majorant=0.0))
    r8 = G.sphere_rays(1 << 17, np.random.default_rng(2))
    v = _vol(ctx, rho, med)
    rd, _ = U.rays_dev(r8)
    T, ck = v.tr(rd, 0xF1ED0002, checkpoint=True)
    To, cko = oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], med, r8, 0xF1ED0002, want_ckpt=True)
    assert np.array_equal(T.cpu().numpy(), To)
    assert np.array_equal(ck["k"].cpu().numpy().view(np.uint32), cko["k"])
    T64, _ = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], med, r8, 0xF1ED0002)
    Tg = T.cpu().numpy().astype(np.float64)
    close = np.abs(Tg - T64) <= 1e-5 * np.abs(T64) + 1e-7
    # rays whose roulette or exit decision flips between fp32 and fp64 are
    # counted, not hidden: they must be rare
    assert (~close).mean() < 2e-3, (~close).sum()


def test_sample_matches_oracle(ctx, oracle):
    import fledge_gb300 as F
    rho = F.gen_noise_grid(ctx, 48, 9).cpu().numpy()
    r8 = G.sphere_rays(1 << 16, np.random.default_rng(3))
    v = _vol(ctx, rho)
    rd, _ = U.rays_dev(r8)
    ok, p, w = v.sample(rd, 77)
    oko, po, wo = oracle.volume_sample(rho, [0, 0, 0], [1, 1, 1], Med, r8, 77)
    assert np.array_equal(ok.cpu().numpy(), oko)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(w.cpu().numpy(), wo)
    assert 0.1 < oko.mean() < 0.99


def test_volume_edge_rays_match_oracle(ctx, oracle):
    """Origins inside the box, tmax ending inside it, rays in and parallel
    to a face's plane (zero direction components), rays just outside a face,
    misses and NaN origins: T, checkpoints, collisions and the adjoint equal
    the oracle's."""
    rho = G.value_noise_grid(32, np.random.default_rng(3))
    r8 = G.volume_edge_rays(np.random.default_rng(4))
    v = _vol(ctx, rho)
    rd, _ = U.rays_dev(r8)
    T, ck = v.tr(rd, 123, checkpoint=True)
    To, cko = oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], Med, r8, 123, want_ckpt=True)
    assert np.array_equal(T.cpu().numpy(), To)
    assert np.array_equal(ck["k"].cpu().numpy().view(np.uint32), cko["k"])
    assert np.array_equal(ck["t"].cpu().numpy(), cko["t"])
    assert np.all(To[-66:] == 1.0)  # misses and NaN origins see no medium
    ok, p, w = v.sample(rd, 123)
    oko, po, wo = oracle.volume_sample(rho, [0, 0, 0], [1, 1, 1], Med, r8, 123)
    assert np.array_equal(ok.cpu().numpy(), oko)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(w.cpu().numpy(), wo)
    dLdT = torch.ones_like(T)
    g = v.tr_adjoint(rd, 123, dLdT, T, ck).cpu().numpy().astype(np.float64)
    go = oracle.volume_tr_adjoint(rho, [0, 0, 0], [1, 1, 1], Med, r8, 123, np.ones(r8.shape[1], np.float32))
    assert np.max(np.abs(g - go)) <= 1e-4 * np.abs(go).max()


def test_majorant_is_grid_max(ctx):
    import fledge_gb300 as F
    rho = F.gen_noise_grid(ctx, 40, 5)
    v = _vol(ctx, rho.cpu().numpy())
    assert v.majorant() == float(rho.max())


@pytest.mark.parametrize("use_ckpt", [True, False])
def test_adjoint_matches_oracle(ctx, oracle, use_ckpt):
    rho = G.value_noise_grid(24, np.random.default_rng(41))
    r8 = G.sphere_rays(1 << 15, np.random.default_rng(42))
    v = _vol(ctx, rho)
    rd, _ = U.rays_dev(r8)
    T, ck = v.tr(rd, 5, checkpoint=True)
    dLdT = torch.rand(r8.shape[1], generator=torch.Generator().manual_seed(3)).cuda()
    g = v.tr_adjoint(rd, 5, dLdT, T, ck if use_ckpt else None).cpu().numpy().astype(np.float64)
    go = oracle.volume_tr_adjoint(rho, [0, 0, 0], [1, 1, 1], Med, r8, 5, dLdT.cpu().numpy())
    scale = np.abs(go).max()
    assert np.max(np.abs(g - go)) <= 1e-4 * scale


def test_adjoint_fd64_random_voxels(ctx, oracle):
    """Gradient of summed T w.r.t. the grid vs FP64 central differences on 64
    seeded voxels (majorant fixed); rays whose roulette flips are excluded
    and counted."""
    res = 32
    rho = G.value_noise_grid(res, np.random.default_rng(51))
    maj = float(rho.max())
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=0.1, majorant=maj))
    r8 = G.sphere_rays(20000, np.random.default_rng(52))
    v = _vol(ctx, rho, med)
    rd, _ = U.rays_dev(r8)
    T, ck = v.tr(rd, 11, checkpoint=True)
    g = v.tr_adjoint(rd, 11, torch.ones_like(T), T, ck).cpu().numpy().reshape(-1)
    rng = np.random.default_rng(53)
    cand = np.nonzero(np.abs(g) > 1e-3 * np.abs(g).max())[0]
    picks = rng.choice(cand, 64, replace=False)
    flips = 0
    for vox in picks:
        x = float(rho.reshape(-1)[vox])
        if x > maj - 1e-3:
            continue
        h = 1e-4 * max(1.0, abs(x))
        rp, rm = rho.astype(np.float64).reshape(-1).copy(), rho.astype(np.float64).reshape(-1).copy()
        rp[vox] += h
        rm[vox] -= h
        Tp, np_ = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], med, r8, 11, rp.reshape(rho.shape))
        Tm, nm = oracle.volume_tr64(rho, [0, 0, 0], [1, 1, 1], med, r8, 11, rm.reshape(rho.shape))
        keep = np_ == nm
        flips += (~keep).sum()
        fd = (Tp[keep].sum() - Tm[keep].sum()) / (2 * h)
        assert abs(fd - g[vox]) <= 1e-3 * abs(fd) + 1e-5, (vox, fd, g[vox])
    assert flips <= 64 * 2


def test_adjoint_autograd_reference(ctx, oracle):
    """torch.autograd.Function around the C-ABI adjoint (test harness only),
    checked against the gradient of a plain differentiable forward: with
    roulette disabled the free-flight positions do not depend on the grid,
    so T = prod(1 - rho(p_i)/rho_max) is a torch expression of the grid."""
    res = 12
    rho = G.value_noise_grid(res, np.random.default_rng(61))
    maj = float(rho.max())
    med = type("M", (), dict(sigma_s=0.8, sigma_a=0.2, g=0.3, rr_threshold=0.0, majorant=maj))
    n = 256
    r8 = G.sphere_rays(n, np.random.default_rng(62))
    v = _vol(ctx, rho, med)
    rd, _ = U.rays_dev(r8)

    class Tr(torch.autograd.Function):
        @staticmethod
        def forward(c, grid):
            T, ck = v.tr(rd, 21, checkpoint=True)
            c.save_for_backward(T, ck["t"], ck["k"], ck["c"])
            return T

        @staticmethod
        def backward(c, gT):
            T, ct, ckk, cc = c.saved_tensors
            return v.tr_adjoint(rd, 21, gT.contiguous(), T, {"t": ct, "k": ckk, "c": cc})

    grid = U.dev(rho).requires_grad_(True)
    w = torch.rand(n, generator=torch.Generator().manual_seed(1)).cuda()
    (Tr.apply(grid) * w).sum().backward()
    g_gpu = grid.grad.cpu().numpy().astype(np.float64)

    # plain forward in float64 with autograd
    rg = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    L = torch.zeros((), dtype=torch.float64)
    sigma_t = np.float32(1.0)
    mu = float(np.float32(sigma_t * np.float32(maj)))
    for i in range(n):
        o, d = r8[0:3, i].astype(np.float64), r8[3:6, i].astype(np.float64)
        with np.errstate(divide="ignore"):
            inv = 1.0 / d
        t0 = np.maximum(np.minimum((0 - o) * inv, (1 - o) * inv), 0).max()
        t1 = np.minimum(np.maximum((0 - o) * inv, (1 - o) * inv), np.inf).min()
        if t0 > t1:
            continue
        u = oracle.stream_uniforms(21, i, 64).astype(np.float64)
        t, Ti = t0, torch.ones((), dtype=torch.float64)
        for k in range(64):
            t += -np.log(1.0 - u[k]) / mu
            if t >= t1:
                break
            gpos = (o + d * t) * (res - 1)
            b = np.floor(gpos).astype(int)
            f = gpos - b
            dens = torch.zeros((), dtype=torch.float64)
            for cidx in range(8):
                cx, cy, cz = cidx & 1, (cidx >> 1) & 1, cidx >> 2
                X, Y, Z = b[0] + cx, b[1] + cy, b[2] + cz
                if min(X, Y, Z) < 0 or max(X, Y, Z) >= res:
                    continue
                wgt = (f[0] if cx else 1 - f[0]) * (f[1] if cy else 1 - f[1]) * (f[2] if cz else 1 - f[2])
                dens = dens + wgt * rg[Z, Y, X]
            Ti = Ti * (1 - torch.clamp(dens / maj, min=0))
        L = L + float(w[i]) * Ti
    L.backward()
    g_ref = rg.grad.numpy()
    assert np.max(np.abs(g_gpu - g_ref)) <= 2e-3 * np.abs(g_ref).max()


def test_adjoint_cost_vs_forward(ctx):
    """Adjoint (with checkpoints) at most 3x the forward on a 256^3 grid."""
    import fledge_gb300 as F
    rho = F.gen_noise_grid(ctx, 256, 0xF1ED0002)
    v = F.DenseGridVolume(rho, medium=F.Medium(), ctx=ctx)
    soa = F.gen_rays(ctx, 1 << 22, 0xF1ED0002)
    rd = F.Rays.from_soa(soa)
    T, ck = v.tr(rd, 1, checkpoint=True)
    dL = torch.ones_like(T)
    grad = torch.zeros_like(rho)
    for _ in range(2):
        v.tr(rd, 1, checkpoint=True)
        v.tr_adjoint(rd, 1, dL, T, ck, grad)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    e[0].record()
    for _ in range(5):
        v.tr(rd, 1, checkpoint=True)
    e[1].record()
    e[2].record()
    for _ in range(5):
        grad.zero_()
        v.tr_adjoint(rd, 1, dL, T, ck, grad)
    e[3].record()
    torch.cuda.synchronize()
    fwd, adj = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    assert adj <= 3.0 * fwd, (fwd, adj)
