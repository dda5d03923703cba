"""Gradient of fixed hits' (t, u, v) with respect to vertex positions
(flg_hit_adjoint): against the FP64 oracle, FP64 finite differences, and the
autograd gradient of a plain torch forward."""
import numpy as np
import pytest
import torch

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu


def _hits(ctx, oracle, n_tri=20000, n_rays=1 << 16, seed=1, indexed=False):
    if indexed:
        v, ind = G.meshed_sphere(96, 96, 1.0)
        rays = G.interior_rays(n_rays, np.random.default_rng(seed))
        pos = v
    else:
        pos = G.random_soup(n_tri, np.random.default_rng(seed), half=0.03)
        ind = None
        rays = G.sphere_rays(n_rays, np.random.default_rng(seed + 1), tmin=0.0)
    b, (p, i) = U.gpu_build(ctx, pos, ind, width=4)
    rd, rt = U.rays_dev(rays)
    h = b.intersect(rd)
    return pos, ind, rays, b, p, i, rd, h


@pytest.mark.parametrize("indexed", [False, True])
def test_hit_adjoint_matches_fp64_oracle(ctx, oracle, indexed):
    import fledge_gb300 as F
    pos, ind, rays, b, p, i, rd, h = _hits(ctx, oracle, indexed=indexed)
    n = rays.shape[1]
    g = torch.randn((3, n), generator=torch.Generator().manual_seed(5)).cuda()
    mesh = F.InternalTriangleMesh(p, i)
    grad = F.hit_adjoint(ctx, mesh, rd, h, g[0].contiguous(), g[1].contiguous(), g[2].contiguous())
    gh = grad.cpu().numpy().astype(np.float64)
    prim = h["prim"].cpu().numpy()
    n_tri = ind.shape[0] if ind is not None else pos.shape[0] // 3
    go = oracle.hit_adjoint64(pos, ind, n_tri, pos.reshape(-1, 3).shape[0], rays, prim, *g.cpu().numpy())
    # fp32 adjoint vs FP64: gradients must agree to 1e-3 relative
    err = np.linalg.norm(gh - go) / np.linalg.norm(go)
    assert err < 1e-3, err


def test_hit_adjoint_fd64(ctx, oracle):
    import fledge_gb300 as F
    pos, ind, rays, b, p, i, rd, h = _hits(ctx, oracle, n_tri=2000, n_rays=20000, seed=11)
    prim = h["prim"].cpu().numpy()
    sel = np.nonzero(prim >= 0)[0]
    # keep rays whose triangle is hit by exactly one selected ray
    _, first, counts = np.unique(prim[sel], return_index=True, return_counts=True)
    sel = sel[first[counts == 1]][:64]
    assert sel.size >= 32
    n = rays.shape[1]
    gnp = np.zeros((3, n), np.float32)
    gnp[:, sel] = np.random.default_rng(12).standard_normal((3, sel.size))
    g = U.dev(gnp)
    grad = F.hit_adjoint(ctx, F.InternalTriangleMesh(p, i), rd, h, g[0], g[1], g[2]).cpu().numpy()
    P = pos.astype(np.float64).reshape(-1, 3)
    for r in sel:
        t = prim[r]
        o, d = rays[0:3, r].astype(np.float64), rays[3:6, r].astype(np.float64)

        def L(Q):
            a, bb, c = Q[3 * t], Q[3 * t + 1], Q[3 * t + 2]
            M = np.stack([d, -(bb - a), -(c - a)], 1)
            return float(gnp[:, r].astype(np.float64) @ np.linalg.solve(M, a - o))
        for vtx in range(3):
            for ax in range(3):
                e = 1e-6
                Qp, Qm = P.copy(), P.copy()
                Qp[3 * t + vtx, ax] += e
                Qm[3 * t + vtx, ax] -= e
                fd = (L(Qp) - L(Qm)) / (2 * e)
                assert abs(fd - grad[3 * t + vtx, ax]) <= 1e-3 * max(1.0, abs(fd)), (r, vtx, ax, fd)


def test_hit_adjoint_autograd_reference(ctx, oracle):
    """torch.autograd.Function around flg_hit_adjoint (test harness only) vs
    autograd through a plain float64 forward of (t, u, v)."""
    import fledge_gb300 as F
    pos, ind, rays, b, p, i, rd, h = _hits(ctx, oracle, n_tri=5000, n_rays=4096, seed=21)
    prim = h["prim"]
    mesh = F.InternalTriangleMesh(p, i)

    class TUV(torch.autograd.Function):
        @staticmethod
        def forward(c, verts):
            c.save_for_backward(verts)
            return torch.stack([h["t"], h["u"], h["v"]], 0)

        @staticmethod
        def backward(c, g):
            (verts,) = c.saved_tensors
            gg = torch.where((prim >= 0)[None, :], g, torch.zeros_like(g)).contiguous()
            return F.hit_adjoint(ctx, F.InternalTriangleMesh(verts, i), rd, h, gg[0], gg[1], gg[2])

    w = torch.randn((3, rays.shape[1]), generator=torch.Generator().manual_seed(2)).cuda()
    verts = p.clone().requires_grad_(True)
    (TUV.apply(verts) * w * (prim >= 0)).sum().backward()
    g_gpu = verts.grad.cpu().numpy().astype(np.float64)

    P = torch.tensor(pos.reshape(-1, 3), dtype=torch.float64, requires_grad=True)
    hit = (prim >= 0).cpu().numpy()
    pr = prim.cpu().numpy()[hit]
    tri = P.view(-1, 3, 3)[torch.from_numpy(pr).long()]
    o = torch.tensor(rays[0:3, hit].T, dtype=torch.float64)
    d = torch.tensor(rays[3:6, hit].T, dtype=torch.float64)
    M = torch.stack([d, -(tri[:, 1] - tri[:, 0]), -(tri[:, 2] - tri[:, 0])], 2)
    tuv = torch.linalg.solve(M, (tri[:, 0] - o).unsqueeze(-1)).squeeze(-1)
    (tuv * w.cpu().double().T[hit]).sum().backward()
    g_ref = P.grad.numpy()
    assert np.linalg.norm(g_gpu - g_ref) <= 1e-3 * np.linalg.norm(g_ref)
