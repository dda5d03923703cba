"""fledge_gb300 — GB300-native acceleration-structure and participating-media
path of the fledge renderer, behind a C ABI (include/flg.h, libflg.so).

Python mirror of the reference's interfaces for this path (paths relative to
the fledge project root):

  * ``InternalTriangleMesh``   experimental/base_bvh.hpp:26-31
  * ``RadixBVHBuilder``        BVHBuilderBase / RadixBVHBuilder
                               (base_bvh.hpp:105-117, radix_bvh.hpp:32-84):
                               ``build()``, ``getBound()``, ``intersect()``
                               (closest hit, batched) and ``intersectP()``
  * ``DenseGridVolume``        Volume / OpenVDBVolume (volume.hpp:16-70):
                               ``tr()``, ``sample()`` and the adjoint
                               ``tr_adjoint()``

Device memory is plain torch CUDA tensors; every computation runs in the CUDA
kernels of libflg.so.  There is no CPU fallback: without the built library or
a GPU these classes raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (FlgBuildOpts, FlgBvhInfo, FlgBvhTopology, FlgError, FlgHits, FlgMedium, FlgRays,
                   FlgTraceOpts, FlgTrCkpt, check, load)

__all__ = ["Context", "InternalTriangleMesh", "RadixBVHBuilder", "BatchedRadixBVHBuilder", "Rays",
           "DenseGridVolume", "SparseGridVolume", "Medium", "hit_adjoint", "gen_triangles", "gen_rays", "gen_noise_grid", "read_ply",
           "FlgError", "load"]


def _torch():
    import torch
    return torch


def _ptr(t) -> Optional[int]:
    return None if t is None else int(t.data_ptr())


class Context:
    """A device + stream + error word (flg_ctx).  By default it issues work on
    torch's current CUDA stream so that torch and the library stay ordered."""

    def __init__(self, device: int = 0, stream=None):
        torch = _torch()
        self.lib = load()
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        sp = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        if not sp:
            sp = 1  # cudaStreamLegacy: torch's default stream
        h = C.c_void_p()
        check(self.lib.flg_ctx_create(device, C.c_void_p(sp), C.byref(h)))
        self.h = h
        self.device = device

    def sync(self) -> None:
        check(self.lib.flg_ctx_sync(self.h), self.h)

    def check(self, code: int) -> None:
        check(code, self.h)

    def set_stage_timing(self, on: bool = True) -> None:
        """Records an event at the end of every build / trace stage."""
        check(self.lib.flg_ctx_set_stage_timing(self.h, 1 if on else 0), self.h)

    def stage_times(self) -> dict:
        """{stage: {"ms": summed milliseconds, "n": count}} since the last read."""
        import json
        buf = C.create_string_buffer(1 << 16)
        check(self.lib.flg_ctx_stage_times(self.h, buf, len(buf)), self.h)
        return json.loads(buf.value.decode() or "{}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.flg_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclass
class Rays:
    """Structure-of-arrays rays (device float32 tensors of length n)."""
    ox: object
    oy: object
    oz: object
    dx: object
    dy: object
    dz: object
    tmin: object = None
    tmax: object = None
    tmin_const: float = 0.0
    tmax_const: float = float("inf")

    @property
    def n(self) -> int:
        return int(self.ox.numel())

    @staticmethod
    def from_soa(soa, tmin: float = 0.0, tmax: float = float("inf")) -> "Rays":
        """soa: [6, n] or [8, n] float32 tensor (ox oy oz dx dy dz [tmin tmax])."""
        if soa.shape[0] == 8:
            return Rays(*[soa[k] for k in range(8)])
        return Rays(*[soa[k] for k in range(6)], tmin_const=tmin, tmax_const=tmax)

    def struct(self) -> FlgRays:
        return FlgRays(_ptr(self.ox), _ptr(self.oy), _ptr(self.oz), _ptr(self.dx), _ptr(self.dy),
                       _ptr(self.dz), _ptr(self.tmin), _ptr(self.tmax), self.tmin_const, self.tmax_const)


@dataclass
class InternalTriangleMesh:
    """Indexed mesh (experimental/base_bvh.hpp:26-31): p = [nVert, 3] float32,
    ind = [nTri, 3] int32 or None for a triangle soup."""
    p: object
    ind: object = None

    @property
    def n_tri(self) -> int:
        return int(self.ind.shape[0]) if self.ind is not None else int(self.p.shape[0]) // 3

    @property
    def n_vert(self) -> int:
        return int(self.p.shape[0])


def _hits_struct(h) -> FlgHits:
    return FlgHits(_ptr(h["prim"]), _ptr(h["t"]), _ptr(h["u"]), _ptr(h["v"]))


def _alloc_hits(n: int, device):
    torch = _torch()
    return {"prim": torch.empty(n, dtype=torch.int32, device=device),
            "t": torch.empty(n, dtype=torch.float32, device=device),
            "u": torch.empty(n, dtype=torch.float32, device=device),
            "v": torch.empty(n, dtype=torch.float32, device=device)}


def _trace_opts(stack_depth=0, block_threads=0, persistent=0, refill_lanes=0, ray_sort=0,
                tri_test=0) -> FlgTraceOpts:
    """tri_test: 0 watertight Pluecker, 1 the live renderer's Moller-Trumbore."""
    return FlgTraceOpts(stack_depth, block_threads, persistent, refill_lanes, ray_sort, tri_test)


def _builder_id(name: str) -> int:
    """'lbvh' (the Karras radix tree), 'ploc' (locally-ordered clustering),
    'sah' (BasicBVHBuilder's binned-SAH build) or 'treelet' (the LBVH refined
    by treelet restructuring)."""
    ids = {"lbvh": _lib.FLG_BUILDER_LBVH, "ploc": _lib.FLG_BUILDER_PLOC, "sah": _lib.FLG_BUILDER_SAH,
           "treelet": _lib.FLG_BUILDER_TREELET}
    if name not in ids:
        raise ValueError(f"builder must be one of {sorted(ids)}")
    return ids[name]


class RadixBVHBuilder:
    """GPU Karras LBVH with the BVHBuilderBase interface (base_bvh.hpp:105-117)."""

    def __init__(self, mesh: InternalTriangleMesh, ctx: Optional[Context] = None, node_width: int = 4,
                 leaf_size: int = 1, builder: str = "lbvh", treelet_rounds: int = 0):
        self.mesh = mesh
        self.ctx = ctx or Context(mesh.p.device.index or 0)
        self.node_width = node_width
        self.leaf_size = leaf_size
        self.builder = _builder_id(builder)
        self.treelet_rounds = treelet_rounds  # builder 'treelet': passes, 1..4 (0 = 3)
        self.h = None

    def _opts(self) -> FlgBuildOpts:
        return FlgBuildOpts(self.node_width, self.leaf_size, 1, self.builder, self.treelet_rounds)

    def build(self) -> None:
        lib = self.ctx.lib
        if self.h is not None:
            self.ctx.check(lib.flg_bvh_rebuild(self.ctx.h, self.h, C.c_void_p(_ptr(self.mesh.p))))
            return
        h = C.c_void_p()
        opts = self._opts()
        self.ctx.check(lib.flg_bvh_build(self.ctx.h, C.c_void_p(_ptr(self.mesh.p)),
                                         C.c_void_p(_ptr(self.mesh.ind)), self.mesh.n_tri,
                                         self.mesh.n_vert, C.byref(opts), C.byref(h)))
        self.h = h

    def getBound(self):
        info = FlgBvhInfo()
        self.ctx.check(self.ctx.lib.flg_bvh_info_get(self.h, C.byref(info)))
        b = np.array(info.bound[:], dtype=np.float32)
        return b[:3], b[3:]

    def info(self) -> FlgBvhInfo:
        info = FlgBvhInfo()
        self.ctx.check(self.ctx.lib.flg_bvh_info_get(self.h, C.byref(info)))
        return info

    def set_width(self, node_width: int, leaf_size: int = 1) -> None:
        self.ctx.check(self.ctx.lib.flg_bvh_set_width(self.ctx.h, self.h, node_width, leaf_size))
        self.node_width, self.leaf_size = node_width, leaf_size

    def intersect(self, rays: Rays, out=None, **opts):
        """Closest hit for a batch of rays: dict of prim (-1 = miss), t, u, v."""
        n = rays.n
        out = out or _alloc_hits(n, rays.ox.device)
        r, hs, op = rays.struct(), _hits_struct(out), _trace_opts(**opts)
        self.ctx.check(self.ctx.lib.flg_trace_closest(self.ctx.h, self.h, C.byref(r), n, C.byref(op),
                                                      C.byref(hs)))
        return out

    def hit_normals(self, rays: Rays, prim, kind: str = "pluecker", out=None):
        """Normals of fixed hits, [n, 3]: "pluecker" (BVHRayHit::hit_ng of the
        experimental path) or "geometric" (SInteraction::m_ng of the live
        renderer's triangle test)."""
        torch = _torch()
        k = {"pluecker": 0, "geometric": 1}[kind]
        out = out if out is not None else torch.empty((rays.n, 3), dtype=torch.float32, device=prim.device)
        r = rays.struct()
        self.ctx.check(self.ctx.lib.flg_hit_normals(self.ctx.h, self.h, C.byref(r), rays.n, C.c_void_p(_ptr(prim)),
                                                    k, C.c_void_p(_ptr(out))))
        return out

    def intersectP(self, rays: Rays, out=None, **opts):
        """Any hit (occlusion) for a batch of rays: uint8 tensor."""
        torch = _torch()
        n = rays.n
        out = out if out is not None else torch.empty(n, dtype=torch.uint8, device=rays.ox.device)
        r, op = rays.struct(), _trace_opts(**opts)
        self.ctx.check(self.ctx.lib.flg_trace_any(self.ctx.h, self.h, C.byref(r), n, C.byref(op),
                                                  C.c_void_p(_ptr(out))))
        return out

    def topology(self, scene: int = 0, n: Optional[int] = None) -> dict:
        """Karras arrays of one scene (host numpy), for parity checks."""
        n = self.mesh.n_tri if n is None else n
        m = max(n - 1, 0)
        t = {"morton": np.zeros(n, np.uint32), "perm": np.zeros(n, np.int32), "split": np.zeros(m, np.int32),
             "leaf_flags": np.zeros(m, np.uint8), "range_j": np.zeros(m, np.int32),
             "parent": np.zeros(m, np.int32), "leaf_parent": np.zeros(n, np.int32),
             "bounds": np.zeros((m, 6), np.float32), "scene_bound": np.zeros(6, np.float32)}
        s = FlgBvhTopology(*[t[k].ctypes.data for k in ("morton", "perm", "split", "leaf_flags", "range_j",
                                                        "parent", "leaf_parent", "bounds", "scene_bound")])
        self.ctx.check(self.ctx.lib.flg_bvh_download(self.h, scene, C.byref(s)))
        return t

    def destroy(self) -> None:
        if self.h is not None:
            self.ctx.lib.flg_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class BatchedRadixBVHBuilder(RadixBVHBuilder):
    """Many scenes built in one segmented launch and traced in one launch."""

    def __init__(self, mesh: InternalTriangleMesh, tri_offsets: Sequence[int], ctx: Optional[Context] = None,
                 node_width: int = 4, leaf_size: int = 1, builder: str = "lbvh", treelet_rounds: int = 0):
        super().__init__(mesh, ctx, node_width, leaf_size, builder, treelet_rounds)
        self.tri_offsets = np.ascontiguousarray(np.asarray(tri_offsets, dtype=np.int64))

    def build(self) -> None:
        lib = self.ctx.lib
        if self.h is not None:
            self.ctx.check(lib.flg_bvh_rebuild(self.ctx.h, self.h, C.c_void_p(_ptr(self.mesh.p))))
            return
        h = C.c_void_p()
        opts = self._opts()
        offs = self.tri_offsets.ctypes.data_as(C.POINTER(C.c_int64))
        self.ctx.check(lib.flg_bvh_build_batched(self.ctx.h, C.c_void_p(_ptr(self.mesh.p)),
                                                 C.c_void_p(_ptr(self.mesh.ind)), offs,
                                                 len(self.tri_offsets) - 1, self.mesh.n_vert, C.byref(opts),
                                                 C.byref(h)))
        self.h = h

    def intersect_batched(self, rays: Rays, ray_offsets: Sequence[int], out=None, ctx: Optional[Context] = None,
                          **opts):
        """Closest hits of every scene's rays in one launch.  ``ctx``: trace
        on another context (its stream and scratch) than the one that built
        the handle; traces only read the handle, so traces on several
        contexts may run at once, but not beside a rebuild."""
        c = ctx or self.ctx
        ro = np.ascontiguousarray(np.asarray(ray_offsets, dtype=np.int64))
        n = int(ro[-1])
        out = out or _alloc_hits(n, rays.ox.device)
        r, hs, op = rays.struct(), _hits_struct(out), _trace_opts(**opts)
        c.check(c.lib.flg_trace_closest_batched(
            c.h, self.h, C.byref(r), ro.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(op), C.byref(hs)))
        return out

    def topology(self, scene: int = 0, n: Optional[int] = None) -> dict:
        n = int(self.tri_offsets[scene + 1] - self.tri_offsets[scene]) if n is None else n
        return super().topology(scene, n)


@dataclass
class Medium:
    sigma_s: float = 0.8
    sigma_a: float = 0.2
    g: float = 0.3
    rr_threshold: float = 0.1
    majorant: float = 0.0

    def struct(self) -> FlgMedium:
        return FlgMedium(self.sigma_s, self.sigma_a, self.g, self.rr_threshold, self.majorant)


class DenseGridVolume:
    """Heterogeneous medium on a dense lattice with the Volume interface
    (volume.hpp:16-30): ``tr`` (ratio tracking), ``sample`` (delta tracking)
    and the adjoint ``tr_adjoint``."""

    def __init__(self, density, box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0), medium: Medium = Medium(),
                 ctx: Optional[Context] = None):
        self.ctx = ctx or Context(density.device.index or 0)
        self.density = density  # [nz, ny, nx] float32, x fastest
        nz, ny, nx = density.shape
        lo = (C.c_float * 3)(*box_lo)
        hi = (C.c_float * 3)(*box_hi)
        m = medium.struct()
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.flg_grid_create(self.ctx.h, C.c_void_p(_ptr(density)), nx, ny, nz, lo, hi,
                                                    C.byref(m), C.byref(h)))
        self.h = h
        self.medium = medium

    def majorant(self) -> float:
        v = C.c_float()
        self.ctx.check(self.ctx.lib.flg_grid_majorant(self.h, C.byref(v)))
        return float(v.value)

    def tr(self, rays: Rays, seed: int, checkpoint: bool = False):
        torch = _torch()
        n = rays.n
        dev = rays.ox.device
        T = torch.empty(n, dtype=torch.float32, device=dev)
        ck = None
        ckp = None
        if checkpoint:
            ck = {"t": torch.empty(n, dtype=torch.float32, device=dev),
                  "k": torch.empty(n, dtype=torch.int32, device=dev),
                  "c": torch.empty(n, dtype=torch.float32, device=dev)}
            ckp = C.byref(FlgTrCkpt(_ptr(ck["t"]), _ptr(ck["k"]), _ptr(ck["c"])))
        r = rays.struct()
        self.ctx.check(self.ctx.lib.flg_volume_tr(self.ctx.h, self.h, C.byref(r), n, seed, C.c_void_p(_ptr(T)),
                                                  ckp))
        return (T, ck) if checkpoint else T

    def tr_adjoint(self, rays: Rays, seed: int, dLdT, T, ckpt=None, grad=None):
        torch = _torch()
        if grad is None:
            grad = torch.zeros_like(self.density)
        ckp = None if ckpt is None else C.byref(FlgTrCkpt(_ptr(ckpt["t"]), _ptr(ckpt["k"]), _ptr(ckpt["c"])))
        r = rays.struct()
        self.ctx.check(self.ctx.lib.flg_volume_tr_adjoint(self.ctx.h, self.h, C.byref(r), rays.n, seed,
                                                          C.c_void_p(_ptr(dLdT)), C.c_void_p(_ptr(T)), ckp,
                                                          C.c_void_p(_ptr(grad))))
        return grad

    def sample(self, rays: Rays, seed: int):
        torch = _torch()
        n = rays.n
        dev = rays.ox.device
        ok = torch.empty(n, dtype=torch.uint8, device=dev)
        p = torch.empty((n, 3), dtype=torch.float32, device=dev)
        w = torch.empty(n, dtype=torch.float32, device=dev)
        r = rays.struct()
        self.ctx.check(self.ctx.lib.flg_volume_sample(self.ctx.h, self.h, C.byref(r), n, seed,
                                                      C.c_void_p(_ptr(ok)), C.c_void_p(_ptr(p)),
                                                      C.c_void_p(_ptr(w))))
        return ok, p, w

    def destroy(self) -> None:
        if getattr(self, "h", None) is not None:
            self.ctx.lib.flg_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class SparseGridVolume(DenseGridVolume):
    """The same medium on a sparse grid of 8^3 bricks (the NanoVDBVolume that
    volume.hpp:72-92 declares): ``from_dense`` keeps the bricks with a
    non-zero voxel.  ``density`` is the [n_bricks, 8, 8, 8] brick array;
    ``tr_adjoint`` gradients have that shape."""

    BRICK = 8

    def __init__(self, brick_index, bricks, shape, box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0),
                 medium: Medium = Medium(), ctx: Optional[Context] = None):
        self.ctx = ctx or Context(brick_index.device.index or 0)
        self.brick_index = brick_index  # [bnz, bny, bnx] int32, slot or -1
        self.density = bricks           # [n_bricks, 8, 8, 8] float32
        self.shape = tuple(shape)       # (nz, ny, nx) of the lattice
        nz, ny, nx = self.shape
        lo = (C.c_float * 3)(*box_lo)
        hi = (C.c_float * 3)(*box_hi)
        m = medium.struct()
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.flg_grid_create_sparse(
            self.ctx.h, C.c_void_p(_ptr(brick_index)), C.c_void_p(_ptr(bricks) if bricks.numel() else None),
            int(bricks.shape[0]), nx, ny, nz, lo, hi, C.byref(m), C.byref(h)))
        self.h = h
        self.medium = medium

    @classmethod
    def from_dense(cls, density, box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0), medium: Medium = Medium(),
                   ctx: Optional[Context] = None) -> "SparseGridVolume":
        torch = _torch()
        ctx = ctx or Context(density.device.index or 0)
        nz, ny, nx = density.shape
        b = cls.BRICK
        bidx = torch.empty(((nz + b - 1) // b, (ny + b - 1) // b, (nx + b - 1) // b), dtype=torch.int32,
                           device=density.device)
        cnt = C.c_int64()
        lib = ctx.lib
        ctx.check(lib.flg_grid_sparsify(ctx.h, C.c_void_p(_ptr(density)), nx, ny, nz, C.c_void_p(_ptr(bidx)), None,
                                        0, C.byref(cnt)))
        bricks = torch.empty((cnt.value, b, b, b), dtype=torch.float32, device=density.device)
        if cnt.value:
            ctx.check(lib.flg_grid_sparsify(ctx.h, C.c_void_p(_ptr(density)), nx, ny, nz, C.c_void_p(_ptr(bidx)),
                                            C.c_void_p(_ptr(bricks)), cnt.value, C.byref(cnt)))
        return cls(bidx, bricks, (nz, ny, nx), box_lo, box_hi, medium, ctx)

    def to_dense(self, values=None):
        """Scatters brick-layout values (the densities, or an adjoint
        gradient) back to the dense [nz, ny, nx] lattice (zeros elsewhere)."""
        torch = _torch()
        vals = self.density if values is None else values
        nz, ny, nx = self.shape
        b = self.BRICK
        bz, by, bx = self.brick_index.shape
        out = torch.zeros((bz * b, by * b, bx * b), dtype=vals.dtype, device=vals.device)
        full = torch.zeros((bz, by, bx, b, b, b), dtype=vals.dtype, device=vals.device)
        occ = self.brick_index >= 0
        full[occ] = vals.reshape(-1, b, b, b)[self.brick_index[occ].long()]
        out = full.permute(0, 3, 1, 4, 2, 5).reshape(bz * b, by * b, bx * b)
        return out[:nz, :ny, :nx].contiguous()


def hit_adjoint(ctx: Context, mesh: InternalTriangleMesh, rays: Rays, hits, dLdt=None, dLdu=None, dLdv=None,
                grad=None):
    """dL/dpos for fixed hits (fp32 atomics into a [nVert, 3] tensor)."""
    torch = _torch()
    if grad is None:
        grad = torch.zeros_like(mesh.p)
    r, hs = rays.struct(), _hits_struct(hits)
    ctx.check(ctx.lib.flg_hit_adjoint(ctx.h, C.c_void_p(_ptr(mesh.p)), C.c_void_p(_ptr(mesh.ind)), mesh.n_tri,
                                      mesh.n_vert, C.byref(r), rays.n, C.byref(hs), C.c_void_p(_ptr(dLdt)),
                                      C.c_void_p(_ptr(dLdu)), C.c_void_p(_ptr(dLdv)), C.c_void_p(_ptr(grad))))
    return grad


def pathtrace(ctx: Context, bvh: RadixBVHBuilder, light_first: int, light_count: int, light_le=(10.0, 10.0, 10.0),
              albedo=(0.7, 0.7, 0.7), eye=(0.0, 0.5, 4.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
              fov_deg: float = 40.0, width: int = 1920, height: int = 1080, spp: int = 16, max_depth: int = 5,
              volume: Optional["DenseGridVolume"] = None, seed: int = 0, mesh_medium: Optional[dict] = None,
              **opts):
    """Wavefront path tracing of the mesh of `bvh` (PathIntegrator::Li with
    next-event estimation; with `volume`, VolPathIntegrator::Li with the
    grid's medium filling its box; with `mesh_medium` = dict(first, count,
    sigma_s, sigma_a, g, density), VolPathIntegrator::Li with a homogeneous
    medium bounded by triangles [first, first + count)).  Returns
    (radiance [height, width, 3], stats)."""
    torch = _torch()
    mesh = bvh.mesh
    sc = _lib.FlgPtScene(_ptr(mesh.p), _ptr(mesh.ind), mesh.n_tri, mesh.n_vert, light_first, light_count,
                         (C.c_float * 3)(*light_le), (C.c_float * 3)(*albedo))
    cam = _lib.FlgPtCamera((C.c_float * 3)(*eye), (C.c_float * 3)(*target), (C.c_float * 3)(*up), fov_deg,
                           width, height)
    out = torch.empty((height, width, 3), dtype=torch.float32, device=mesh.p.device)
    st = _lib.FlgPtStats()
    op = _trace_opts(**opts)
    if mesh_medium is not None:
        m = mesh_medium
        mm = _lib.FlgMeshMedium(m["first"], m["count"], (C.c_float * 3)(*m["sigma_s"]),
                                (C.c_float * 3)(*m["sigma_a"]), m["g"], m.get("density", 1.0))
        ctx.check(ctx.lib.flg_volpath_mesh(ctx.h, bvh.h, C.byref(mm), seed, C.byref(sc), C.byref(cam), spp,
                                           max_depth, C.byref(op), C.c_void_p(_ptr(out)), C.byref(st)))
    elif volume is None:
        ctx.check(ctx.lib.flg_pathtrace(ctx.h, bvh.h, C.byref(sc), C.byref(cam), spp, max_depth, C.byref(op),
                                        C.c_void_p(_ptr(out)), C.byref(st)))
    else:
        ctx.check(ctx.lib.flg_volpath(ctx.h, bvh.h, volume.h, seed, C.byref(sc), C.byref(cam), spp, max_depth,
                                      C.byref(op), C.c_void_p(_ptr(out)), C.byref(st)))
    return out, {"closest_rays": st.closest_rays, "shadow_rays": st.shadow_rays}


# ------------------------------ mesh ingestion -------------------------------

def read_ply(path: str) -> dict:
    """Reads a PLY triangle mesh (MakeTriangleMesh, plymesh.cpp:19-86) on the
    host: dict of pos [n_vert, 3] float32, idx [n_tri, 3] int32, and normal
    [n_vert, 3] / uv [n_vert, 2] float32 or None."""
    lib = load()
    m = _lib.FlgHostMesh()
    err = C.create_string_buffer(256)
    code = lib.flg_ply_read(path.encode(), C.byref(m), err, 256)
    if code != _lib.FLG_OK:
        raise FlgError(code, err.value.decode() or lib.flg_status_string(code).decode())
    try:
        nv, nt = int(m.n_vert), int(m.n_tri)

        def arr(ptr, n, dt, cols):
            if not ptr or n == 0:
                return None if not ptr else np.zeros((0, cols), dt)
            return np.ctypeslib.as_array(ptr, shape=(n * cols,)).astype(dt, copy=True).reshape(n, cols)

        return {"pos": arr(m.pos, nv, np.float32, 3), "idx": arr(m.idx, nt, np.int32, 3),
                "normal": arr(m.normal, nv, np.float32, 3), "uv": arr(m.uv, nv, np.float32, 2)}
    finally:
        lib.flg_host_mesh_free(C.byref(m))


# --------------------------- synthetic workloads -----------------------------

def gen_triangles(ctx: Context, n: int, seed: int, first: int = 0, half_extent: float = 0.01):
    torch = _torch()
    pos = torch.empty((3 * n, 3), dtype=torch.float32, device=f"cuda:{ctx.device}")
    ctx.check(ctx.lib.flg_gen_triangles(ctx.h, seed, first, n, half_extent, C.c_void_p(_ptr(pos))))
    return pos


def gen_rays(ctx: Context, n: int, seed: int, first: int = 0, center=(0.5, 0.5, 0.5), radius: float = 2.0):
    """[6, n] float32 SoA: origins on a sphere, directions toward U[0,1]^3."""
    torch = _torch()
    soa = torch.empty((6, n), dtype=torch.float32, device=f"cuda:{ctx.device}")
    c = (C.c_float * 3)(*center)
    ps = [C.c_void_p(_ptr(soa[k])) for k in range(6)]
    ctx.check(ctx.lib.flg_gen_rays(ctx.h, seed, first, n, c, radius, *ps))
    return soa


def gen_noise_grid(ctx: Context, res: int, seed: int, scale: float = 4.0):
    torch = _torch()
    rho = torch.empty((res, res, res), dtype=torch.float32, device=f"cuda:{ctx.device}")
    ctx.check(ctx.lib.flg_gen_noise_grid(ctx.h, seed, res, res, res, scale, C.c_void_p(_ptr(rho))))
    return rho
