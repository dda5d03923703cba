"""flg_trace_closest_noalloc: closest hit for callers that cannot call
cudaMalloc when they trace (inside a CUDA stream capture, under an arena that
owns all device memory, in a frame loop where an allocation would stall).
Its traversal scratch is a fixed device array inside the library instead of
the context's lazily allocated buffers.

Checked through the C ABI against flg_trace_closest (same kernels, so the
bar is bit equality, as for the other traversal layouts), on two calls in a
row: the second call reuses the shared array the first one left behind.
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
