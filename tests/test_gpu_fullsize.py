"""Parity at the benchmark workloads' full sizes (the other GPU tests run
reduced inputs).  The GPU runs each workload whole; the oracle checks a
seeded sample of it, where the oracle finishes in seconds.

  * batched scenes: 256 scenes, 34,597,655 triangles in one segmented build
    (4-wide, leaf ranges of 3).  The three largest scenes (about 1 M
    triangles each): Karras topology and bounds bit-exact; a seeded 1 M-ray
    sample of their 64 rays per triangle, traced by the persistent batched
    kernel: zero prim mismatches other than exact ties, t/u/v bit-equal to
    the oracle where ids agree, t/u/v within 1e-5 of FP64.
  * 8 M-triangle scene: topology bit-exact; a seeded 1 M sample of the
    3840x2160x4 camera rays as above; the shadow rays of that sample toward
    the point light: occlusion bits equal.
  * 256^3 grid, 4,194,304 rays: T and roulette checkpoints bit-equal on a
    65,536-ray subset; the adjoint's gradient at 64 seeded voxels equal to
    the oracle's analytic one over every ray that touches the voxel (1e-4),
    and that analytic gradient equal to FP64 central differences (1e-3),
    rays whose roulette decision flips between +h and -h counted and
    excluded (fewer than 1e-4 of the touching rays); once more with the
    roulette off, where nothing may flip.
  * path tracing of the level-8 icosphere at 1920x1080, 16 spp, depth 5:
    every 97th pixel against the oracle's PathIntegrator::Li restatement.
"""
import numpy as np
import pytest
import torch

import gpu_util as U

pytestmark = pytest.mark.gpu


def _free():
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def _check_sample(oracle, pos, ind, tree, r8, hg):
    bad, ties, ho = U.compare_closest(oracle, pos, ind, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = hg["prim"] == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    n_tri = tree["n"]
    U.check_t_fp64(oracle, pos, ind, n_tri, r8, hg)
    return ties


def test_batched_scenes_full_size(ctx, oracle):
    import fledge_gb300 as F
    from fledge_gb300 import scenes as S
    counts = S.batched_scene_counts()
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    n_tri = int(offs[-1])
    assert n_tri == 34597655
    pos = F.gen_triangles(ctx, n_tri, S.SEED_BATCH)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(pos), offs, ctx, node_width=4, leaf_size=3)
    bb.build()
    big = [int(s) for s in np.argsort(counts)[-3:]]
    # the rays of the three largest scenes, from the batch's own streams
    ray_counts = np.zeros(len(counts), np.int64)
    ray_counts[big] = counts[big] * S.RAYS_PER_TRI
    roffs = np.concatenate([[0], np.cumsum(ray_counts)]).astype(np.int64)
    full_roffs = offs * S.RAYS_PER_TRI
    soa = torch.cat([F.gen_rays(ctx, int(ray_counts[s]), S.SEED_BATCH + 1, first=int(full_roffs[s])) for s in big], 1)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = bb.intersect_batched(rays, roffs, persistent=2, refill_lanes=8, stack_depth=64)
    ctx.sync()
    rng = np.random.default_rng(0xF1ED0003)
    per = (1 << 20) // 3
    ph = None
    for s in big:
        a, b = int(offs[s]), int(offs[s + 1])
        sp = pos[3 * a:3 * b].cpu().numpy()
        tree = oracle.build_bvh(sp)
        U.assert_same_topology(bb.topology(scene=s), tree)
        idx = np.sort(rng.choice(int(ray_counts[s]), per, replace=False)) + int(roffs[s])
        it = torch.from_numpy(idx).cuda()
        r8 = np.zeros((8, per), np.float32)
        r8[:6] = soa[:, it].cpu().numpy()
        r8[6], r8[7] = np.float32(1e-4), np.inf
        hg = {k: v[it].cpu().numpy() for k, v in hits.items()}
        _check_sample(oracle, sp, None, tree, r8, hg)
        assert (hg["prim"] >= 0).mean() > 0.5
    bb.destroy()
    del pos, soa, rays, hits, ph
    _free()


def test_8m_triangles_camera_and_shadow_rays(ctx, oracle):
    import fledge_gb300 as F
    from fledge_gb300 import scenes as S
    n_tri = 8_000_000
    pos = F.gen_triangles(ctx, n_tri, S.SEED_BATCH + 40)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=4)
    b.build()
    ph = pos.cpu().numpy()
    tree = oracle.build_bvh(ph)
    U.assert_same_topology(b.topology(), tree)
    soa = S.camera_rays_4k(torch, pos.device)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = b.intersect(rays)
    # shadow rays toward the point light, as the benchmark forms them
    light = torch.tensor([0.5, 2.0, 0.5], device=pos.device)[:, None]
    hp = soa[0:3] + soa[3:6] * hits["t"][None, :]
    sd = light - hp
    dist = sd.norm(dim=0)
    sd = sd / dist
    hit = hits["prim"] >= 0
    sh = torch.cat([hp[:, hit], sd[:, hit], torch.full((1, int(hit.sum())), 1e-4, device=pos.device),
                    (dist[hit] * (1 - 1e-4))[None, :]], 0).contiguous()
    occ = b.intersectP(F.Rays(*[sh[k] for k in range(8)]), persistent=2, refill_lanes=16)
    ctx.sync()
    n = soa.shape[1]
    rng = np.random.default_rng(0xF1ED0004)
    idx = np.sort(rng.choice(n, 1 << 20, replace=False))
    it = torch.from_numpy(idx).cuda()
    r8 = np.zeros((8, idx.size), np.float32)
    r8[:6] = soa[:, it].cpu().numpy()
    r8[6], r8[7] = np.float32(1e-4), np.inf
    hg = {k: v[it].cpu().numpy() for k, v in hits.items()}
    _check_sample(oracle, ph, None, tree, r8, hg)
    # occlusion of the sample's shadow rays (shadow ray j belongs to the j-th hit)
    srank = torch.cumsum(hit.to(torch.int64), 0) - 1
    sel = it[hit[it]]
    sidx = srank[sel]
    s8 = sh[:, sidx].cpu().numpy()
    occ_o = oracle.trace_any(ph, None, tree, s8, oracle.MODE_DEV)
    assert np.array_equal(occ[sidx].cpu().numpy().astype(bool), occ_o.astype(bool))
    # the 8 M-triangle soup fills the unit box: almost every hit point is in
    # shadow (99.3 %); both outcomes still occur
    assert 0.5 < occ_o.mean() < 0.9999 and (occ_o == 0).sum() > 100
    b.destroy()
    del pos, soa, rays, hits, sh, occ
    _free()


class _Med:
    def __init__(self, rr, maj):
        self.sigma_s, self.sigma_a, self.g, self.rr_threshold, self.majorant = 0.8, 0.2, 0.3, rr, maj


def _touching(soa, res, vox):
    """Ids of the rays whose segment inside the unit box meets the trilinear
    support of lattice point vox (the 8 cells around it), with a margin."""
    z, rem = divmod(int(vox), res * res)
    y, x = divmod(rem, res)
    h = 1.0 / (res - 1)
    lo = torch.tensor([max(x - 1, 0) * h, max(y - 1, 0) * h, max(z - 1, 0) * h], device=soa.device) - 1e-5
    hi = torch.tensor([min(x + 1, res - 1) * h, min(y + 1, res - 1) * h, min(z + 1, res - 1) * h],
                      device=soa.device) + 1e-5
    o, d = soa[0:3], soa[3:6]
    inv = 1.0 / d
    ta, tb = (0.0 - o) * inv, (1.0 - o) * inv
    t0 = torch.clamp(torch.minimum(ta, tb).max(0).values, min=0.0)
    t1 = torch.maximum(ta, tb).min(0).values
    sa, sb = (lo[:, None] - o) * inv, (hi[:, None] - o) * inv
    s0 = torch.maximum(torch.minimum(sa, sb).max(0).values, t0)
    s1 = torch.minimum(torch.maximum(sa, sb).min(0).values, t1)
    return torch.nonzero(s0 <= s1).flatten()


@pytest.mark.parametrize("rr", [0.1, 0.0])
def test_volume_256_full_size(ctx, oracle, rr):
    import fledge_gb300 as F
    from fledge_gb300 import scenes as S
    res, n = 256, 1 << 22
    rho = F.gen_noise_grid(ctx, res, S.SEED_VOLUME)
    soa = F.gen_rays(ctx, n, S.SEED_VOLUME + 1)
    rays = F.Rays.from_soa(soa)
    rho_h = rho.cpu().numpy()
    seed = S.SEED_VOLUME
    # forward: T and checkpoints of the first 65,536 rays, bit-equal
    vol = F.DenseGridVolume(rho, medium=F.Medium(0.8, 0.2, 0.3, rr, 0.0), ctx=ctx)
    T, ck = vol.tr(rays, seed, checkpoint=True)
    ctx.sync()
    m = 1 << 16
    r8 = np.zeros((8, m), np.float32)
    r8[:6] = soa[:, :m].cpu().numpy()
    r8[7] = np.inf
    To, cko = oracle.volume_tr(rho_h, [0, 0, 0], [1, 1, 1], _Med(rr, 0.0), r8, seed, want_ckpt=True)
    assert np.array_equal(T[:m].cpu().numpy(), To)
    assert np.array_equal(ck["k"][:m].cpu().numpy().view(np.uint32), cko["k"])
    assert np.array_equal(ck["t"][:m].cpu().numpy(), cko["t"])
    assert np.array_equal(ck["c"][:m].cpu().numpy(), cko["c"])
    vol.destroy()
    # gradient of sum(T) at 64 voxels; the majorant sits just above the grid
    # maximum so that no perturbed voxel crosses it (it is held constant)
    maj = float(np.float32(rho_h.max() * (1.0 + 2.0 ** -10)))
    med = _Med(rr, maj)
    vol = F.DenseGridVolume(rho, medium=F.Medium(0.8, 0.2, 0.3, rr, maj), ctx=ctx)
    T, ck = vol.tr(rays, seed, checkpoint=True)
    g = vol.tr_adjoint(rays, seed, torch.ones_like(T), T, ck).reshape(-1)
    ctx.sync()
    gh = g.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(0xF1ED0005 + int(rr * 10))
    cand = np.nonzero(np.abs(gh) > 1e-3 * np.abs(gh).max())[0]
    picks = rng.choice(cand, 64, replace=False)
    flips = touching = worst = 0
    for vox in picks:
        ids_t = _touching(soa, res, vox)
        ids = ids_t.cpu().numpy()
        sub = np.zeros((8, ids.size), np.float32)
        sub[:6] = soa[:, ids_t].cpu().numpy()
        sub[7] = np.inf
        per_ray = oracle.volume_tr_adjoint_vox(rho_h, [0, 0, 0], [1, 1, 1], med, sub, ids, seed, int(vox))
        assert abs(gh[vox] - per_ray.sum()) <= 1e-4 * abs(per_ray.sum()) + 1e-7 * np.abs(gh).max(), vox
        x = float(rho_h.reshape(-1)[vox])
        hstep = 1e-4 * max(1.0, abs(x))
        Tp, np_ = oracle.volume_tr64_sub(rho_h, [0, 0, 0], [1, 1, 1], med, sub, ids, seed, int(vox), hstep)
        Tm, nm = oracle.volume_tr64_sub(rho_h, [0, 0, 0], [1, 1, 1], med, sub, ids, seed, int(vox), -hstep)
        keep = (np_ == nm) & ((Tp == 0) == (Tm == 0))
        flips += int((~keep).sum())
        worst = max(worst, int((~keep).sum()))
        touching += ids.size
        fd = (Tp[keep].sum() - Tm[keep].sum()) / (2 * hstep)
        an = per_ray[keep].sum()
        assert abs(fd - an) <= 1e-3 * abs(fd) + 1e-6 * np.abs(gh).max(), (vox, fd, an)
    assert touching > 64 * 100
    if rr == 0.0:
        assert flips == 0
    assert flips < 1e-4 * touching, (flips, touching, worst)
    vol.destroy()
    del rho, soa, rays, T, ck, g
    _free()


def test_path_tracing_full_size_pixel_subset(ctx, oracle):
    import fledge_gb300 as F
    from fledge_gb300 import scenes as S
    pos, ind, lfirst = S.path_tracing_scene(8)
    assert ind.shape[0] == 1310720 + 2
    b, _ = U.gpu_build(ctx, pos, ind, width=4, leaf=2)
    W, H, spp, depth = 1920, 1080, 16, 5
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=W, height=H, spp=spp, max_depth=depth,
                             **S.PATH_TRACING_CAMERA, persistent=2, refill_lanes=16)
    ctx.sync()
    g = img.cpu().numpy().reshape(-1, 3)
    tree = oracle.build_bvh(pos, ind)
    stride = 97
    cam = S.PATH_TRACING_CAMERA
    ref, _ = oracle.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"], cam["target"],
                              cam["up"], cam["fov_deg"], W, H, spp, depth, stride)
    ref = ref.reshape(-1, 3)[::stride]
    gs = g[::stride]
    close = np.abs(gs - ref) <= 1e-4 * np.maximum(np.abs(ref), 1.0)
    assert close.mean() > 0.995, close.mean()
    assert abs(gs.mean() - ref.mean()) <= 1e-3 * ref.mean()
    assert (ref > 0).mean() > 0.03
    b.destroy()
