"""Autotuner of the batched build + trace step (no counterpart in the
reference): picks the tree builder, the node width and leaf size, and the
traversal kernel options of a batched workload, and persists the choice as a
JSON record that the benchmark loads.

For every builder (the Karras LBVH, PLOC, the binned-SAH rule, the LBVH
refined by three rounds of treelet restructuring, "treelet1" by one round)
the batch is
built, the build is timed (median of `reps`), and flg_autotune_trace_batched
runs its staged search (layout, kernel, block size; each trial the median of
`reps` launches) on a fraction of every scene's rays.  The builder whose
build + full trace is fastest wins; the record keeps every trial.

    python -m fledge_gb300.autotune [--out PATH] [--reps 5] [--ray-fraction 0.125]

tunes the 256-scene batch (config 3) on cuda:0 and writes the record.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import time

import numpy as np

from . import (BatchedRadixBVHBuilder, Context, FlgTraceOpts, InternalTriangleMesh, Rays, _torch, check)
from . import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_RECORD = os.path.join(HERE, "tuned", "batched_config3.json")


def _median_ms(torch, fn, reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return statistics.median(out)


def subsample_offsets(ray_offsets, fraction: float):
    """The first `fraction` of every scene's rays (at least one where the
    scene has any): returns (indices of the kept rays' ranges, new offsets)."""
    ro = np.asarray(ray_offsets, np.int64)
    cnt = np.diff(ro)
    keep = np.where(cnt > 0, np.maximum(1, np.floor(cnt * fraction)), 0).astype(np.int64)
    return keep, np.concatenate([[0], np.cumsum(keep)]).astype(np.int64)


BUILDERS = ("lbvh", "ploc", "sah", "treelet", "treelet1")


def builder_args(name: str) -> dict:
    """Builder keyword arguments of a candidate name: 'treelet<r>' is the
    treelet builder with r restructuring rounds."""
    if name.startswith("treelet") and name[7:].isdigit():
        return {"builder": "treelet", "treelet_rounds": int(name[7:])}
    return {"builder": name}


def tune_batched(ctx: Context, mesh: InternalTriangleMesh, tri_offsets, rays: Rays, ray_offsets,
                 builders=BUILDERS, reps: int = 5, ray_fraction: float = 0.125) -> dict:
    """Returns the tuning record (see the module docstring)."""
    torch = _torch()
    ro = np.asarray(ray_offsets, np.int64)
    keep, sub_off = subsample_offsets(ro, ray_fraction)
    # the sampled rays, contiguous per scene
    idx = np.concatenate([np.arange(ro[s], ro[s] + keep[s]) for s in range(len(keep)) if keep[s] > 0])
    it = torch.from_numpy(idx).to(rays.ox.device)
    cols = [rays.ox, rays.oy, rays.oz, rays.dx, rays.dy, rays.dz]
    if rays.tmin is not None and rays.tmax is not None:
        cols += [rays.tmin, rays.tmax]
    soa = torch.stack([c[it] for c in cols], 0).contiguous()
    sub = (Rays(*[soa[k] for k in range(8)]) if len(cols) == 8 else
           Rays(*[soa[k] for k in range(6)], tmin_const=rays.tmin_const, tmax_const=rays.tmax_const))
    n_full = int(ro[-1])
    per = {}
    for name in builders:
        bb = BatchedRadixBVHBuilder(mesh, tri_offsets, ctx, node_width=4, leaf_size=1, **builder_args(name))
        bb.build()
        build_ms = _median_ms(torch, bb.build, reps)
        best = FlgTraceOpts()
        w, leaf = C.c_int32(), C.c_int32()
        buf = C.create_string_buffer(1 << 20)
        r = sub.struct()
        offs = np.ascontiguousarray(sub_off)
        t0 = time.perf_counter()
        check(ctx.lib.flg_autotune_trace_batched(ctx.h, bb.h, C.byref(r), offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                                 reps, C.byref(best), C.byref(w), C.byref(leaf), buf, len(buf)),
              ctx.h)
        tune_s = time.perf_counter() - t0
        search = json.loads(buf.value.decode())
        bb.set_width(w.value, leaf.value)
        opts = dict(stack_depth=best.stack_depth, block_threads=best.block_threads, persistent=best.persistent,
                    refill_lanes=best.refill_lanes)
        trace_ms = _median_ms(torch, lambda: bb.intersect_batched(rays, ro, **opts), max(3, reps // 2))
        per[name] = {"build_ms": round(build_ms, 4), "trace_ms": round(trace_ms, 3),
                     "step_ms": round(build_ms + trace_ms, 3),
                     "mrays_s": round(n_full / ((build_ms + trace_ms) * 1e-3) / 1e6, 2),
                     "node_width": w.value, "leaf_size": leaf.value, "trace_opts": opts,
                     "search_seconds": round(tune_s, 1), "search": search}
        bb.destroy()
    win = min(per, key=lambda k: per[k]["step_ms"])
    w = per[win]
    return {"workload": {"scenes": len(tri_offsets) - 1, "triangles": int(tri_offsets[-1]), "rays": n_full,
                         "search_rays": int(sub_off[-1]), "ray_fraction": ray_fraction},
            "reps": reps, "builder": win, "node_width": w["node_width"], "leaf_size": w["leaf_size"],
            **w["trace_opts"], "step_ms": w["step_ms"], "per_builder": per,
            "device": torch.cuda.get_device_name(0), "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}


def tune_config3(out: str = DEFAULT_RECORD, reps: int = 5, ray_fraction: float = 0.125,
                 builders=BUILDERS) -> dict:
    """Tunes the 256-scene batch with the benchmark's seeds and writes the record."""
    torch = _torch()
    from . import gen_rays, gen_triangles
    ctx = Context(0)
    counts = S.batched_scene_counts()
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    roffs = offs * S.RAYS_PER_TRI
    pos = gen_triangles(ctx, int(offs[-1]), S.SEED_BATCH)
    n = int(roffs[-1])
    soa = torch.empty((6, n), dtype=torch.float32, device="cuda")
    chunk = 1 << 28
    for c0 in range(0, n, chunk):
        m = min(chunk, n - c0)
        soa[:, c0:c0 + m] = gen_rays(ctx, m, S.SEED_BATCH + 1, first=c0)
    rays = Rays.from_soa(soa, tmin=1e-4)
    rec = tune_batched(ctx, InternalTriangleMesh(pos), offs, rays, roffs, builders, reps, ray_fraction)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        json.dump(rec, f, indent=1)
    ctx.close()
    return rec


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_RECORD)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--ray-fraction", type=float, default=0.125)
    ap.add_argument("--builders", default=",".join(BUILDERS))
    a = ap.parse_args()
    rec = tune_config3(a.out, a.reps, a.ray_fraction, tuple(a.builders.split(",")))
    print(json.dumps({k: v for k, v in rec.items() if k != "per_builder"}))
    print(json.dumps({k: {kk: vv for kk, vv in v.items() if kk != "search"} for k, v in rec["per_builder"].items()}))


if __name__ == "__main__":
    main()
