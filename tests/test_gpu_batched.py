"""Batched scenes (one segmented build, one persistent trace), CUDA-graph
replay, and the error paths of the C ABI on the GPU."""
import ctypes as C

import numpy as np
import pytest
import torch

import geometry as G
import gpu_util as U

pytestmark = pytest.mark.gpu


def _batch(ctx, counts, rays_per_tri=8, seed=3, width=4):
    import fledge_gb300 as F
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    roffs = offs * rays_per_tri
    pos = F.gen_triangles(ctx, int(offs[-1]), seed)
    soa = F.gen_rays(ctx, int(roffs[-1]), seed + 1)
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(pos), offs, ctx, node_width=width)
    bb.build()
    return bb, pos, soa, offs, roffs


@pytest.mark.parametrize("opts", [{}, {"persistent": 1, "refill_lanes": 16}, {"persistent": 1, "refill_lanes": 1},
                                  {"persistent": 2, "refill_lanes": 16}])
def test_batched_trace_equals_per_scene(ctx, oracle, opts):
    import fledge_gb300 as F
    counts = [1, 2, 1000, 37, 20000, 5, 3000]
    bb, pos, soa, offs, roffs = _batch(ctx, counts)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hb = U.host(bb.intersect_batched(rays, roffs, **opts))
    ph, rh = pos.cpu().numpy(), soa.cpu().numpy()
    for s in range(len(counts)):
        sp = ph[3 * offs[s]:3 * offs[s + 1]]
        r8 = np.zeros((8, roffs[s + 1] - roffs[s]), np.float32)
        r8[:6] = rh[:, roffs[s]:roffs[s + 1]]
        r8[6], r8[7] = np.float32(1e-4), np.inf
        tree = oracle.build_bvh(sp)
        hs = {k: v[roffs[s]:roffs[s + 1]] for k, v in hb.items()}
        bad, ties, _ = U.compare_closest(oracle, sp, None, tree, r8, hs, oracle.MODE_DEV)
        assert bad == 0, (s, bad)


def test_batched_persistent_equals_plain(ctx):
    import fledge_gb300 as F
    rng = np.random.default_rng(8)
    counts = np.round(np.exp(rng.uniform(np.log(1e3), np.log(1e5), 24))).astype(np.int64)
    bb, pos, soa, offs, roffs = _batch(ctx, counts, rays_per_tri=4)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    a = U.host(bb.intersect_batched(rays, roffs))
    b = U.host(bb.intersect_batched(rays, roffs, persistent=1, refill_lanes=12))
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_back_to_back_traces_with_changing_offsets(ctx):
    """Batched traces enqueued one after another with different ray offsets
    and no synchronisation in between (each uploads its offsets on the
    context's stream): every call sees its own offsets, as when the calls
    run one at a time."""
    import fledge_gb300 as F
    counts = [500, 3000, 20, 7000, 1, 1200]
    bb, pos, soa, offs, roffs = _batch(ctx, counts, rays_per_tri=6, seed=11)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    n = int(roffs[-1])
    # the rays split into groups of scenes, each traced with its own offsets
    groups = [(0, 2), (2, 3), (3, 6)]
    ref = U.host(bb.intersect_batched(rays, roffs))
    ctx.sync()
    outs = []
    for rep in range(3):
        for (a, b) in groups:
            r0, r1 = int(roffs[a]), int(roffs[b])
            ro = np.zeros(len(counts) + 1, np.int64)
            ro[a + 1:b + 1] = roffs[a + 1:b + 1] - roffs[a]
            ro[b + 1:] = ro[b]
            sub = F.Rays(*[soa[k, r0:r1] for k in range(6)], tmin_const=1e-4)
            outs.append((r0, r1, bb.intersect_batched(sub, ro)))
    ctx.sync()
    for r0, r1, o in outs:
        h = U.host(o)
        for k in ref:
            assert np.array_equal(h[k], ref[k][r0:r1]), (r0, k)
    assert n == sum(r1 - r0 for r0, r1, _ in outs) // 3


def test_traces_on_two_contexts_share_a_handle(ctx):
    """One handle traced from two contexts (two streams) at once, groups of
    scenes alternating between them: the hits equal one trace of all rays."""
    import fledge_gb300 as F
    counts = [4000, 300, 9000, 1, 2500, 7000, 50]
    bb, pos, soa, offs, roffs = _batch(ctx, counts, rays_per_tri=6, seed=21)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    ref = U.host(bb.intersect_batched(rays, roffs))
    ctx.sync()
    side = torch.cuda.Stream()
    ctx2 = F.Context(0, side)
    built = torch.cuda.Event()
    built.record(ctx.stream)
    side.wait_event(built)
    outs = []
    for gi, (a, b) in enumerate([(0, 1), (1, 3), (3, 4), (4, 7)]):
        r0, r1 = int(roffs[a]), int(roffs[b])
        ro = np.zeros(len(counts) + 1, np.int64)
        ro[a + 1:b + 1] = roffs[a + 1:b + 1] - roffs[a]
        ro[b + 1:] = ro[b]
        sub = F.Rays(*[soa[k, r0:r1] for k in range(6)], tmin_const=1e-4)
        outs.append((r0, r1, bb.intersect_batched(sub, ro, ctx=(ctx, ctx2)[gi & 1])))
    ctx.sync()
    ctx2.sync()
    for r0, r1, o in outs:
        h = U.host(o)
        for k in ref:
            assert np.array_equal(h[k], ref[k][r0:r1]), (r0, k)
    ctx2.close()


def test_graph_capture_rebuild_and_trace(ctx, oracle):
    """Build + trace captured once, replayed after the vertices change in place."""
    import fledge_gb300 as F
    n = 50000
    pos = F.gen_triangles(ctx, n, 5)
    soa = F.gen_rays(ctx, 1 << 18, 6)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=4)
    b.build()
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    out = b.intersect(rays)  # allocates scratch before capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    ctx2 = F.Context(0, s)
    g = C.c_void_p()
    r0, h0, op0 = rays.struct(), F._hits_struct(out), F.FlgTraceOpts()
    # first trace on a context allocates its scratch: do it before capturing
    ctx2.check(ctx2.lib.flg_trace_closest(ctx2.h, b.h, C.byref(r0), rays.n, C.byref(op0), C.byref(h0)))
    ctx2.sync()
    with torch.cuda.stream(s):
        ctx2.check(ctx2.lib.flg_graph_begin(ctx2.h))
        ctx2.check(ctx2.lib.flg_bvh_rebuild(ctx2.h, b.h, C.c_void_p(pos.data_ptr())))
        r, hs, op = rays.struct(), F._hits_struct(out), F.FlgTraceOpts()
        ctx2.check(ctx2.lib.flg_trace_closest(ctx2.h, b.h, C.byref(r), rays.n, C.byref(op), C.byref(hs)))
        ctx2.check(ctx2.lib.flg_graph_end(ctx2.h, C.byref(g)))
    for trial in range(2):
        pos.copy_(F.gen_triangles(ctx, n, 100 + trial))
        torch.cuda.synchronize()
        ctx2.check(ctx2.lib.flg_graph_launch(ctx2.h, g))
        ctx2.sync()
        ph = pos.cpu().numpy()
        r8 = np.zeros((8, rays.n), np.float32)
        r8[:6] = soa.cpu().numpy()
        r8[6], r8[7] = np.float32(1e-4), np.inf
        tree = oracle.build_bvh(ph)
        bad, _, _ = U.compare_closest(oracle, ph, None, tree, r8, U.host(out), oracle.MODE_DEV)
        assert bad == 0
    ctx2.lib.flg_graph_destroy(g)
    ctx2.close()


def test_bounded_wait_times_out_and_context_survives(ctx):
    """A wait on a device flag that nothing sets returns FLG_ERR_TIMEOUT after
    its poll limit; the context keeps working afterwards."""
    from fledge_gb300 import _lib
    assert ctx.lib.flg_debug_wait_unset_flag(ctx.h, 2000) == _lib.FLG_ERR_TIMEOUT
    assert ctx.lib.flg_ctx_sync(ctx.h) == _lib.FLG_OK
    pos = G.random_soup(1000, np.random.default_rng(1))
    b, _ = U.gpu_build(ctx, pos)
    ctx.sync()


@pytest.mark.parametrize("batched", [False, True])
def test_spin_limit_on_real_waits_then_recovers(oracle, batched):
    """The bounded waits of real multi-tile builds cut to one poll each: the
    onesweep look-back (a timed-out tile still publishes a prefix), the
    climb's sibling hand-over (a climb that gives up marks the handle) and the
    collapse's grid barrier.  Each build returns FLG_OK or FLG_ERR_TIMEOUT,
    the context stays usable, and the next build with the default limit is
    bit-exact against the oracle: the marked handle's arrival counters and
    hand-over records are reset first."""
    import fledge_gb300 as F
    from fledge_gb300 import _lib
    c = F.Context(0)
    rng = np.random.default_rng(41)
    counts = [600000] if not batched else [200000, 0, 1, 3072, 150000, 250000]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pos = G.random_soup(int(offs[-1]), rng)
    if batched:
        b = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), offs, c, node_width=4, leaf_size=3)
    else:
        b = F.RadixBVHBuilder(F.InternalTriangleMesh(U.dev(pos)), c, node_width=4, leaf_size=3)
    b.build()
    c.sync()
    status = []
    c.check(c.lib.flg_ctx_set_spin_limit(c.h, 1))
    for _ in range(4):
        b.build()
        status.append(c.lib.flg_ctx_sync(c.h))
    c.check(c.lib.flg_ctx_set_spin_limit(c.h, 0))
    assert set(status) <= {_lib.FLG_OK, _lib.FLG_ERR_TIMEOUT}, status
    assert _lib.FLG_ERR_TIMEOUT in status, status
    b.build()
    c.sync()
    r8 = G.sphere_rays(1 << 16, np.random.default_rng(42))
    rd, _ = U.rays_dev(r8)
    for s, n in enumerate(counts):
        if n == 0:
            continue
        sp = pos[3 * offs[s]:3 * offs[s + 1]]
        tree = oracle.build_bvh(sp)
        U.assert_same_topology(b.topology(s) if batched else b.topology(), tree)
        if not batched:
            hg = U.host(b.intersect(rd, persistent=2, refill_lanes=8))
            bad, _, _ = U.compare_closest(oracle, sp, None, tree, r8, hg, oracle.MODE_DEV)
            assert bad == 0
    c.sync()
    b.destroy()
    c.close()


def test_argument_errors_launch_nothing(ctx):
    import fledge_gb300 as F
    from fledge_gb300 import _lib
    h = C.c_void_p()
    opts = F.FlgBuildOpts(3, 1, 1)
    p = torch.zeros((30, 3), device="cuda")
    assert ctx.lib.flg_bvh_build(ctx.h, C.c_void_p(p.data_ptr()), None, 10, 30, C.byref(opts),
                                 C.byref(h)) == _lib.FLG_ERR_ARG
    opts = F.FlgBuildOpts(4, 1, 1)
    assert ctx.lib.flg_bvh_build(ctx.h, C.c_void_p(p.data_ptr()), None, 10, 29, C.byref(opts),
                                 C.byref(h)) == _lib.FLG_ERR_ARG
    assert ctx.lib.flg_bvh_build(ctx.h, None, None, 10, 30, C.byref(opts), C.byref(h)) == _lib.FLG_ERR_ARG
    offs = (C.c_int64 * 3)(0, 5, 3)
    assert ctx.lib.flg_bvh_build_batched(ctx.h, C.c_void_p(p.data_ptr()), None, offs, 2, 15, C.byref(opts),
                                         C.byref(h)) == _lib.FLG_ERR_ARG
    b, _ = U.gpu_build(ctx, G.random_soup(10, np.random.default_rng(0)))
    r = F.FlgRays()
    hs = F.FlgHits()
    op = F.FlgTraceOpts(48, 0, 0, 0, 0)
    assert ctx.lib.flg_trace_closest(ctx.h, b.h, C.byref(r), 5, C.byref(op), C.byref(hs)) == _lib.FLG_ERR_ARG
    ctx.sync()


def test_batched_autotuner_record_and_parity(ctx, oracle):
    """fledge_gb300.autotune over a batch: every builder searched, the record
    lists the staged trials with medians, and the winning configuration
    traces like the oracle."""
    import fledge_gb300 as F
    from fledge_gb300 import autotune
    rng = np.random.default_rng(31)
    counts = np.round(np.exp(rng.uniform(np.log(500), np.log(60000), 12))).astype(np.int64)
    bb, pos, soa, offs, roffs = _batch(ctx, counts, rays_per_tri=4)
    bb.destroy()
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    rec = autotune.tune_batched(ctx, F.InternalTriangleMesh(pos), offs, rays, roffs, builders=("lbvh", "sah"),
                                reps=3, ray_fraction=0.25)
    assert rec["builder"] in ("lbvh", "sah") and set(rec["per_builder"]) == {"lbvh", "sah"}
    for name, p in rec["per_builder"].items():
        stages = {t["stage"] for t in p["search"]["trials"]}
        assert {"layout", "kernel", "block"} <= stages, name
        assert all(t["ms_min"] <= t["ms"] <= t["ms_max"] for t in p["search"]["trials"])
        assert p["search"]["best"]["node_width"] == p["node_width"] and p["search"]["reps"] == 3
    best = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(pos), offs, ctx, node_width=rec["node_width"],
                                    leaf_size=rec["leaf_size"], builder=rec["builder"])
    best.build()
    opts = {k: rec[k] for k in ("stack_depth", "block_threads", "persistent", "refill_lanes")}
    hb = U.host(best.intersect_batched(rays, roffs, **opts))
    ph, rh = pos.cpu().numpy(), soa.cpu().numpy()
    for s in (0, 5, 11):
        sp = ph[3 * offs[s]:3 * offs[s + 1]]
        r8 = np.zeros((8, roffs[s + 1] - roffs[s]), np.float32)
        r8[:6] = rh[:, roffs[s]:roffs[s + 1]]
        r8[6], r8[7] = np.float32(1e-4), np.inf
        tree = oracle.build_bvh_sah(sp) if rec["builder"] == "sah" else oracle.build_bvh(sp)
        hs = {k: v[roffs[s]:roffs[s + 1]] for k, v in hb.items()}
        bad, _, _ = U.compare_closest(oracle, sp, None, tree, r8, hs, oracle.MODE_DEV)
        assert bad == 0, s
    best.destroy()
