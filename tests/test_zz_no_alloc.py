"""flg_trace_closest_noalloc: closest hit for callers that cannot call
cudaMalloc when they trace (under an arena that owns all device memory, in a
frame loop where an allocation would stall the device).
Its traversal scratch is a fixed device array inside the library instead of
the context's lazily allocated buffers.

Checked through the C ABI against flg_trace_closest (same kernels, so the
bar is bit equality, as for the other traversal layouts), on two calls in a
row: the second call reuses the shared array the first one left behind, also
after a call whose rays overflow the short stack into the array's overflow
list.  A first call on a device made inside a stream capture is refused.
Kept in its own file, collected last."""
import ctypes as C

import numpy as np
import pytest

import fledge_gb300 as F
from fledge_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc(ctx, bvh, rays, n):
    import torch
    out = {"prim": torch.empty(n, dtype=torch.int32, device="cuda"),
           "t": torch.empty(n, dtype=torch.float32, device="cuda"),
           "u": torch.empty(n, dtype=torch.float32, device="cuda"),
           "v": torch.empty(n, dtype=torch.float32, device="cuda")}
    r, hs = rays.struct(), F._hits_struct(out)
    rc = ctx.lib.flg_trace_closest_noalloc(ctx.h, bvh.h, C.byref(r), n, C.byref(hs))
    return rc, out


@pytest.mark.parametrize("width", [2, 4, 8])
def test_noalloc_matches_allocating_entry_point(ctx, width):
    pos = F.gen_triangles(ctx, 60000, 0x5EED + width)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=width)
    b.build()
    results = []
    for call, (n, seed) in enumerate([(300000, 11), (1 << 20, 12)]):  # two calls in a row
        soa = F.gen_rays(ctx, n, seed)
        rays = F.Rays.from_soa(soa, tmin=1e-4)
        rc, got = _noalloc(ctx, b, rays, n)
        assert rc == _lib.FLG_OK, rc
        ctx.sync()
        ref = b.intersect(rays)
        ctx.sync()
        for k in ("prim", "t", "u", "v"):
            assert np.array_equal(got[k].cpu().numpy(), ref[k].cpu().numpy()), (call, k)
        results.append(float((got["prim"] >= 0).float().mean()))
    assert all(0.3 < h < 1.0 for h in results)


def test_noalloc_rejects_oversize(ctx):
    pos = F.gen_triangles(ctx, 1000, 3)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=4)
    b.build()
    r = F.FlgRays()
    hs = F.FlgHits()
    dummy = np.zeros(1, np.float32)
    p = dummy.ctypes.data
    r.ox = r.oy = r.oz = r.dx = r.dy = r.dz = p
    hs.prim = hs.t = hs.u = hs.v = p
    rc = ctx.lib.flg_trace_closest_noalloc(ctx.h, b.h, C.byref(r), (1 << 20) + 1, C.byref(hs))
    assert rc == _lib.FLG_ERR_ARG
    buf = C.create_string_buffer(512)
    ctx.lib.flg_ctx_last_error(ctx.h, buf, 512)
    assert b"maximum" in buf.value
    ctx.sync()


@pytest.mark.parametrize("width", [8])
def test_noalloc_deep_stack_scene_then_plain_scene(ctx, width):
    """Two calls in a row: first a scene that overflows the traversal stack
    (every ray crosses every box and hits only a target behind them all,
    tests/geometry.py sliver_comb with groups of 4096: at width 8, 7 pushes
    per level over a 39-level binary tree; a diagnostic read of the
    entry point's overflow count found all 4096 rays in the overflow list,
    served by the deep-stack retry from the shared array), then a plain
    scene.  Both bit-equal to flg_trace_closest; the context reports no error
    (no overflow left unserved, no stale overflow count carried into the
    second call)."""
    import geometry as G
    import gpu_util as U
    pos, r8 = G.sliver_comb(4096, np.random.default_rng(77))
    deep, _ = U.gpu_build(ctx, pos, width=width)
    rd, _ = U.rays_dev(r8)
    rc, got = _noalloc(ctx, deep, rd, rd.n)
    assert rc == _lib.FLG_OK, rc
    assert ctx.lib.flg_ctx_sync(ctx.h) == _lib.FLG_OK
    ref = deep.intersect(rd)
    ctx.sync()
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(got[k].cpu().numpy(), ref[k].cpu().numpy()), k
    assert np.all(got["prim"].cpu().numpy() == pos.shape[0] // 3 - 1)  # every ray reaches the target
    plain = F.RadixBVHBuilder(F.InternalTriangleMesh(F.gen_triangles(ctx, 50000, 91)), ctx, node_width=width)
    plain.build()
    soa = F.gen_rays(ctx, 200000, 92)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    rc, got2 = _noalloc(ctx, plain, rays, rays.n)
    assert rc == _lib.FLG_OK, rc
    assert ctx.lib.flg_ctx_sync(ctx.h) == _lib.FLG_OK
    ref2 = plain.intersect(rays)
    ctx.sync()
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(got2[k].cpu().numpy(), ref2[k].cpu().numpy()), k


def test_noalloc_first_call_inside_a_capture_is_refused():
    """In a fresh process, a first call inside a capture (before the scratch
    has been looked up on the device) returns FLG_ERR_STATE and records
    nothing; the capture still ends cleanly."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = r"""
import ctypes as C, sys, torch
sys.path.insert(0, %r)
import fledge_gb300 as F
from fledge_gb300 import _lib
ctx0 = F.Context(0)
pos = F.gen_triangles(ctx0, 2000, 3)
b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx0, node_width=4)
b.build()
rays = F.Rays.from_soa(F.gen_rays(ctx0, 1024, 4), tmin=1e-4)
out = {k: torch.empty(1024, dtype=torch.int32 if k == "prim" else torch.float32, device="cuda") for k in "ptuv"}
out = {"prim": out["p"], "t": out["t"], "u": out["u"], "v": out["v"]}
ctx0.sync()
s = torch.cuda.Stream()
ctx = F.Context(0, s)
r, hs = rays.struct(), F._hits_struct(out)
g = C.c_void_p()
torch.cuda.synchronize()
with torch.cuda.stream(s):
    ctx.check(ctx.lib.flg_graph_begin(ctx.h))
    rc = ctx.lib.flg_trace_closest_noalloc(ctx.h, b.h, C.byref(r), 1024, C.byref(hs))
    rc_end = ctx.lib.flg_graph_end(ctx.h, C.byref(g))
buf = C.create_string_buffer(512)
ctx.lib.flg_ctx_last_error(ctx.h, buf, 512)
ctx.lib.flg_graph_destroy(g)
print(rc, rc_end, int(b"capture" in buf.value))
""" % root
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    rc, rc_end, msg = (int(x) for x in p.stdout.split())
    assert rc == _lib.FLG_ERR_STATE and rc_end == _lib.FLG_OK and msg == 1
