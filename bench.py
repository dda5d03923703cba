#!/usr/bin/env python3
"""Benchmark of the GB300 LBVH / traversal / transmittance path.

Headline workload (one step): 256 independent random-triangle scenes with
triangle counts log-uniform in [1e3, 1e6] (about 37 M triangles), 64 rays per
triangle (about 2.4 G rays), built by one segmented LBVH build and traced by
one persistent closest-hit launch.  Metric: aggregate Mrays/s of the step
(build + trace), with the build time reported beside it, the plain
one-scene-per-launch path measured on the same inputs, and the volume
transmittance forward/adjoint pass on a 256^3 grid with 4,194,304 rays.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  All inputs are seeded synthetic data
generated on the device (Philox streams); inputs exceed the 129 MB L2, so no
flush is needed between steps.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s & LBVH ms, batched+adjoint vs plain on 1 GB300, t rel err ≤1e-5"
N_SCENES = 256
RAYS_PER_TRI = 64
SEED_C0, SEED_C2, SEED_C3 = 0xF1ED0000, 0xF1ED0002, 0xF1ED0003
# Algorithmic bytes (compulsory DRAM traffic): per ray 6 floats in + prim, t,
# u, v out; per triangle of a batched build: bounds 36 + Morton 44 + sort of
# (scene, code) keys (histogram 8 + 5 passes x 24) + Karras 20 + refit 100.
BYTES_PER_RAY = 24 + 16
BYTES_PER_TRI_BATCHED = 36 + 44 + (8 + 5 * 24) + 20 + 100
# DRAM bytes per ray of the trace kernel from the committed ncu capture
# (profiles/k_trace_ww_w4_config3_8scenes.md: dram__bytes_read.sum +
# dram__bytes_write.sum of one launch over the first 8 scenes, divided by its
# 41,186,368 rays); scaled by rays to a full launch.
TRACE_DRAM_BYTES_PER_RAY_NCU = (1.259081e9 + 0.378162e9) / 41186368


_T0 = time.perf_counter()
_VERBOSE = False


def log(msg: str) -> None:
    if _VERBOSE:
        sys.stderr.write(f"[bench {time.perf_counter() - _T0:8.2f}s] {msg}\n")
        sys.stderr.flush()


def scene_counts(seed: int = SEED_C3, n: int = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = np.round(np.exp(rng.uniform(math.log(1e3), math.log(1e6), N_SCENES))).astype(np.int64)
    return c if n is None else c[:n]


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={device}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows if len(r) >= 9 for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU reference arm (the oracle restates the reference; run on all host cores)
# ---------------------------------------------------------------------------

def sah_cpu(O, scenes, n_tri_gpu: int, gpu_build_ms: float) -> dict:
    """The oracle's binned-SAH build (one thread, recursive) on the largest
    scene of the CPU sample, beside the GPU's batched SAH build rate."""
    pos = max((p for p, _ in scenes), key=lambda p: p.shape[0])
    n = pos.shape[0] // 3
    t0 = time.perf_counter()
    O.build_bvh_sah(pos)
    dt = time.perf_counter() - t0
    return {"cpu_mtris_s": round(n / dt / 1e6, 3), "gpu_mtris_s": round(n_tri_gpu / (gpu_build_ms * 1e-3) / 1e6, 1),
            "cpu_sample": f"oracle SAH build of one {n}-triangle scene, 1 thread ({dt:.2f} s)"}


def cpu_sample(max_tris: int = 1_500_000, rays_cap: int = 2_000_000):
    """Bounded sample of the headline workload for the CPU: the first scenes
    of the batch up to max_tris triangles, 64 rays per triangle capped at
    rays_cap rays, generated with numpy (same distributions)."""
    counts = scene_counts()
    keep, tot = [], 0
    for c in counts:
        if tot + c > max_tris:
            break
        keep.append(int(c))
        tot += int(c)
    rng = np.random.default_rng(7)
    scenes = []
    rays_left = rays_cap
    for c in keep:
        cent = rng.random((c, 1, 3), dtype=np.float32)
        pos = (cent + (2 * rng.random((c, 3, 3), dtype=np.float32) - 1) * np.float32(0.01)).reshape(-1, 3)
        nr = min(c * RAYS_PER_TRI, max(rays_left, 0))
        rays_left -= nr
        u = rng.random((nr, 5))
        z = 1 - 2 * u[:, 0]
        ph = 2 * np.pi * u[:, 1]
        s = np.sqrt(np.maximum(0, 1 - z * z))
        o = np.stack([0.5 + 2 * s * np.cos(ph), 0.5 + 2 * s * np.sin(ph), 0.5 + 2 * z])
        d = u[:, 2:5].T - o
        d /= np.linalg.norm(d, axis=0, keepdims=True)
        r8 = np.zeros((8, nr), np.float32)
        r8[0:3], r8[3:6], r8[6], r8[7] = o, d, 1e-4, np.inf
        scenes.append((pos.astype(np.float32), r8))
    return scenes


def cpu_step(O, scenes):
    t0 = time.perf_counter()
    n_rays = 0
    for pos, r8 in scenes:
        n = pos.shape[0] // 3
        tree = O.build_timed(pos, None, n)
        tree["n"] = n
        if r8.shape[1]:
            O.trace_closest(pos, None, tree, r8, O.MODE_REF)
        n_rays += r8.shape[1]
    return n_rays, time.perf_counter() - t0


def run_reference(args, rank: int) -> None:
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    scenes = cpu_sample()
    for _ in range(max(args.warmup, 0) and 1):
        cpu_step(O, scenes[:2])
    rates = []
    for _ in range(args.steps):
        nr, dt = cpu_step(O, scenes)
        rates.append(nr / dt / 1e6)
    v = statistics.median(rates)
    ntri = sum(p.shape[0] // 3 for p, _ in scenes)
    nrays = sum(r.shape[1] for _, r in scenes)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(nrays / v / 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy, same distributions as the GPU workload)",
            "config": {"workload": "batched random-triangle scenes (config 3 generator), CPU sample",
                       "scenes": len(scenes), "triangles": ntri, "rays": nrays},
            "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": f"{len(scenes)} scenes / {ntri} triangles / {nrays} rays per step: "
                                       "oracle build (parallel bounds, Morton, 32-byte-record sort, Karras, "
                                       "atomic refit) + recursive closest hit"},
            "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args, rank: int, world: int, local_rank: int) -> None:
    import torch
    import fledge_gb300 as F
    dist = world > 1
    if dist:
        import torch.distributed as tdist

    def barrier():
        if dist:
            tdist.barrier()

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = F.Context(local_rank)
    lib = ctx.lib
    launches0 = lib.flg_ctx_launch_count(ctx.h)

    # ---- inputs (device-resident, generated by Philox) ----
    counts = scene_counts()
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    roffs = offs * RAYS_PER_TRI
    n_tri, n_rays = int(offs[-1]), int(roffs[-1])
    log(f'generating {n_tri} triangles, {n_rays} rays')
    pos = F.gen_triangles(ctx, n_tri, SEED_C3)
    soa = torch.empty((6, n_rays), dtype=torch.float32, device=dev)
    chunk = 1 << 28
    for c0 in range(0, n_rays, chunk):
        m = min(chunk, n_rays - c0)
        ps = [C.c_void_p(soa[k, c0:].data_ptr()) for k in range(6)]
        cen = (C.c_float * 3)(0.5, 0.5, 0.5)
        ctx.check(lib.flg_gen_rays(ctx.h, SEED_C3 + 1, c0, m, cen, 2.0, *ps))
    if args.presort_rays:
        log("presorting rays (diagnostics)")
        presort_rays(torch, soa, roffs)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = {"prim": torch.empty(n_rays, dtype=torch.int32, device=dev),
            "t": torch.empty(n_rays, dtype=torch.float32, device=dev),
            "u": torch.empty(n_rays, dtype=torch.float32, device=dev),
            "v": torch.empty(n_rays, dtype=torch.float32, device=dev)}
    mesh = F.InternalTriangleMesh(pos)
    width, leaf = args.width, args.leaf
    bb = F.BatchedRadixBVHBuilder(mesh, offs, ctx, node_width=width, leaf_size=leaf)
    log('first build')
    bb.build()
    topts = dict(persistent=args.persistent, refill_lanes=args.refill, stack_depth=args.stack)
    ctx.sync()

    stream = torch.cuda.current_stream(dev)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        bb.build()
        if ev:
            ev[1].record(stream)
        bb.intersect_batched(rays, roffs, out=hits, **topts)
        if ev:
            ev[2].record(stream)

    log('warm-up steps')
    for _ in range(args.warmup):
        step()
    ctx.sync()
    barrier()
    torch.cuda.synchronize()
    log('timed steps')
    clk = ClockSampler(local_rank)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    l0 = lib.flg_ctx_launch_count(ctx.h)
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    launches = lib.flg_ctx_launch_count(ctx.h) - l0
    ctx.sync()
    total_ms = t_start.elapsed_time(t_end)
    build_ms = [e[0].elapsed_time(e[1]) for e in evs]
    trace_ms = [e[1].elapsed_time(e[2]) for e in evs]
    if dist:
        t = torch.tensor([total_ms], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = world * n_rays / (ms_step * 1e-3) / 1e6
    hit_rate = float((hits["prim"] >= 0).float().mean().item())

    pk = peaks()
    trace_bytes = n_rays * BYTES_PER_RAY + int(bb.info().device_bytes)
    tr_ms = statistics.median(trace_ms)
    roof = {"bound": "hbm", "achieved": round(trace_bytes / (tr_ms * 1e-3) / 1e9, 1), "peak": pk["hbm_gbs"],
            "unit": "GB/s", "frac": None,
            "traffic": (round(n_rays * TRACE_DRAM_BYTES_PER_RAY_NCU) if width == 4 and args.persistent == 2
                        else None),
            "traffic_source": "ncu capture of 8 scenes scaled by rays (lower bound at full size)",
            "kernel": ("k_trace_bvh2<false>" if width == 2 else
                       f"k_trace_ww<{width},false,{args.stack}>" if args.persistent == 2 else
                       f"k_trace_persistent<{width},false,{args.stack}>" if args.persistent else
                       f"k_trace_wide<{width},false,{args.stack}>"),
            "peak_source": pk["source"],
            # what bounds it instead of HBM (the committed ncu capture of the same kernel)
            "limiter": ("L1 data pipe: 98.5 % of L1 wavefronts busy, DRAM 0.7 %, L2 hit rate 98 % "
                        "(profiles/k_trace_ww_w4_config3_8scenes.md)") if width == 4 and args.persistent == 2 else None}
    roof["frac"] = round(roof["achieved"] / roof["peak"], 4)
    b_ms = statistics.median(build_ms)
    build_roof = {"achieved": round(n_tri * BYTES_PER_TRI_BATCHED / (b_ms * 1e-3) / 1e9, 1),
                  "frac": round(n_tri * BYTES_PER_TRI_BATCHED / (b_ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                  "bytes_per_tri": BYTES_PER_TRI_BATCHED}

    # ---- plain path: one build + one trace launch per scene (BVH2 kernel) ----
    log(f'timed: {total_ms / args.steps:.1f} ms/step, build {statistics.median(build_ms):.2f} ms')
    plain = None
    if not args.skip_plain:
        handles = []
        for s in range(N_SCENES):
            sub = F.InternalTriangleMesh(pos[3 * offs[s]:3 * offs[s + 1]])
            h = F.RadixBVHBuilder(sub, ctx, node_width=2)
            h.build()
            handles.append(h)
        sub_rays = [F.Rays(*[soa[k, roffs[s]:roffs[s + 1]] for k in range(6)], tmin_const=1e-4)
                    for s in range(N_SCENES)]
        sub_hits = [{k: v[roffs[s]:roffs[s + 1]] for k, v in hits.items()} for s in range(N_SCENES)]

        def plain_step():
            for s in range(N_SCENES):
                handles[s].build()
                handles[s].intersect(sub_rays[s], out=sub_hits[s])
        plain_step()
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.plain_steps):
            plain_step()
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1) / args.plain_steps
        plain = {"ms_per_step": round(pms, 3), "mrays_s": round(n_rays / (pms * 1e-3) / 1e6, 2),
                 "speedup_batched_vs_plain": round(pms / ms_step, 3)}
        for h in handles:
            h.destroy()
        del handles

    # ---- high-quality builders (PLOC, binned SAH) on the same scenes and rays ----
    log('plain path done' if plain else 'plain skipped')
    hq = sah = None
    if not args.skip_hq:
        res = {}
        for name in ("ploc", "sah"):
            hb = F.BatchedRadixBVHBuilder(mesh, offs, ctx, node_width=width, leaf_size=leaf, builder=name)
            hb.build()
            hb.intersect_batched(rays, roffs, out=hits, **topts)  # warm-up
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record(stream)
            hb.build()
            ev[1].record(stream)
            hb.intersect_batched(rays, roffs, out=hits, **topts)
            ev[2].record(stream)
            torch.cuda.synchronize()
            hb_ms, ht_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
            res[name] = {"builder": "ploc (radius 16)" if name == "ploc" else "binned SAH (16 buckets, reference rule)",
                         "build_ms": round(hb_ms, 3), "trace_ms": round(ht_ms, 2),
                         "mrays_s": round(n_rays / (ht_ms * 1e-3) / 1e6, 1),
                         "trace_speedup_vs_lbvh": round(statistics.median(trace_ms) / ht_ms, 3),
                         "step_ms": round(hb_ms + ht_ms, 2)}
            hb.destroy()
            log(f'{name} builder done')
        hq, sah = res["ploc"], res["sah"]

    # ---- e2e: host (pinned) inputs, copies inside the timed region ----
    e2e = None
    if not args.skip_e2e:
        e2e = run_e2e(args, ctx, torch, F, pos, soa, offs, roffs, n_tri, n_rays, width, leaf, topts, dev, world)

    # ---- volume: config 2 forward + adjoint ----
    log('e2e done')
    vol = run_volume(ctx, torch, F, dev) if not args.skip_volume else None
    log("config 0")
    c0 = run_c0(ctx, torch, F, dev, pk) if not args.skip_c0 else None
    log("config 4")
    c4 = run_c4(ctx, torch, F, dev, pk) if not args.skip_c4 else None
    log("config 1")
    c1 = run_c1(ctx, torch, F, dev, rank == 0 and not args.skip_cpu) if not args.skip_c1 else None
    log("config 1 with a medium")
    c1v = run_c1_volume(ctx, torch, F, dev, rank == 0 and not args.skip_cpu) if not args.skip_c1 else None

    # ---- CPU baseline (rank 0) ----
    log('volume done')
    cpu = None
    if rank == 0 and not args.skip_cpu:
        from oracle import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        O.set_threads(cores)
        scenes = cpu_sample(max_tris=600_000, rays_cap=1_000_000)
        nr, dt = cpu_step(O, scenes)
        ntri = sum(p.shape[0] // 3 for p, _ in scenes)
        cpu = {"value": round(nr / dt / 1e6, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
               "sample": f"{len(scenes)} scenes, {ntri} triangles, {nr} rays: oracle build + closest hit "
                         f"({dt:.1f} s)"}
        if sah is not None:
            sah.update(sah_cpu(O, scenes, n_tri, sah["build_ms"]))

    total_launches = lib.flg_ctx_launch_count(ctx.h) - launches0
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded Philox on device)",
                "config": {"workload": "config 3: 256 batched random-triangle scenes, log-uniform [1e3,1e6] "
                                       "triangles, 64 rays/triangle; segmented LBVH build + persistent trace",
                           "triangles": n_tri, "rays": n_rays, "node_width": width, "leaf_size": leaf,
                           "refill_lanes": args.refill, "l2": "inputs larger than L2 (no flush)",
                           "parallelism": f"replicas x{world}"},
                "build_ms": round(b_ms, 3), "trace_ms": round(tr_ms, 3), "hit_rate": round(hit_rate, 4),
                "build_roofline": build_roof, "roofline": roof, "plain": plain, "volume": vol,
                "hq_builder": hq, "sah_builder": sah, "config0": c0, "config1": c1, "config1_volume": c1v, "config4": c4,
                "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches),
                "gpu_launches_total": int(total_launches)}
        print(json.dumps(line), flush=True)
    ctx.close()


def run_e2e(args, ctx, torch, F, pos, soa, offs, roffs, n_tri, n_rays, width, leaf, topts, dev, world):
    """Same step through the public API with host buffers: H2D of triangles
    and rays from pinned memory, build, trace, D2H of the hits, all timed.
    Rays move in chunks of scenes on a copy stream, overlapped with tracing."""
    need = n_tri * 36 + n_rays * (24 + 16)
    avail = 0
    with open("/proc/meminfo") as f:
        for line in f:
            if line.startswith("MemAvailable:"):
                avail = int(line.split()[1]) * 1024
    if need > 0.6 * avail:
        return {"value": None, "unit": "Mrays/s", "skipped": f"needs {need / 1e9:.0f} GB pinned host memory, "
                                                             f"{avail / 1e9:.0f} GB available"}
    h_pos = torch.empty(pos.shape, dtype=torch.float32, pin_memory=True)
    h_pos.copy_(pos)
    h_rays = torch.empty(soa.shape, dtype=torch.float32, pin_memory=True)
    h_rays.copy_(soa)
    h_out = {k: torch.empty(n_rays, dtype=torch.int32 if k == "prim" else torch.float32, pin_memory=True)
             for k in ("prim", "t", "u", "v")}
    d_pos = torch.empty_like(pos)
    d_rays = torch.empty_like(soa)
    d_out = {k: torch.empty(n_rays, dtype=v.dtype, device=dev) for k, v in h_out.items()}
    bb = F.BatchedRadixBVHBuilder(F.InternalTriangleMesh(d_pos), offs, ctx, node_width=width, leaf_size=leaf)
    d_pos.copy_(h_pos)
    bb.build()
    main = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(dev)
    # scene groups of about 256 M rays
    groups, g0 = [], 0
    for s in range(N_SCENES):
        if roffs[s + 1] - roffs[g0] >= (1 << 28) or s == N_SCENES - 1:
            groups.append((g0, s + 1))
            g0 = s + 1

    def e2e_step():
        d_pos.copy_(h_pos, non_blocking=True)
        bb.build()
        evs = []
        for (a, b) in groups:
            r0, r1 = int(roffs[a]), int(roffs[b])
            with torch.cuda.stream(copy):
                d_rays[:, r0:r1].copy_(h_rays[:, r0:r1], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy)
            main.wait_event(ev)
            ro = np.zeros(N_SCENES + 1, np.int64)
            ro[a + 1:b + 1] = roffs[a + 1:b + 1] - roffs[a]
            ro[b + 1:] = ro[b]
            sub_rays = F.Rays(*[d_rays[k, r0:r1] for k in range(6)], tmin_const=1e-4)
            sub_out = {k: v[r0:r1] for k, v in d_out.items()}
            bb.intersect_batched(sub_rays, ro, out=sub_out, **topts)
            done = torch.cuda.Event()
            done.record(main)
            evs.append((done, r0, r1))
        for done, r0, r1 in evs:
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                for k in h_out:
                    h_out[k][r0:r1].copy_(d_out[k][r0:r1], non_blocking=True)
        main.wait_stream(copy)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    ok = bool(torch.equal(h_out["prim"][:1 << 20].to(dev), d_out["prim"][:1 << 20]))
    bb.destroy()
    return {"value": round(world * n_rays / dt / 1e6, 2), "unit": "Mrays/s",
            "h2d_bytes_per_step": int(n_tri * 36 + n_rays * 24), "d2h_bytes_per_step": int(n_rays * 16),
            "ms_per_step": round(dt * 1e3, 3), "host_readback_consistent": ok}


BYTES_PER_TRI_SINGLE = 36 + 44 + (4 + 4 * 16) + 20 + 100


def presort_rays(torch, soa, roffs):
    """Diagnostics: reorder every scene's rays by a 6-D Morton key of origin
    and direction (4 bits per coordinate) to measure what ray coherence buys."""
    def spread(x):  # 4 bits -> every 6th bit
        out = torch.zeros_like(x)
        for b in range(4):
            out |= ((x >> b) & 1) << (6 * b)
        return out
    for s in range(len(roffs) - 1):
        a, b = int(roffs[s]), int(roffs[s + 1])
        if b - a < 2:
            continue
        seg = soa[:, a:b]
        key = torch.zeros(b - a, dtype=torch.int64, device=soa.device)
        for k in range(6):
            lo, hi = (-1.6, 2.6) if k < 3 else (-1.0, 1.0)
            q = ((seg[k] - lo) / (hi - lo) * 16).clamp(0, 15).to(torch.int64)
            key |= spread(q) << k
        order = torch.argsort(key)
        soa[:, a:b] = seg[:, order]


def _time(torch, fn, reps, stream):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_c0(ctx, torch, F, dev, pk):
    """Config 0: 65,536 triangles, 1,048,576 rays: build ms and closest-hit
    Mrays/s for the plain BVH2 kernel and the 4-wide kernel."""
    s = torch.cuda.current_stream(dev)
    pos = F.gen_triangles(ctx, 65536, SEED_C0)
    rays = F.Rays.from_soa(F.gen_rays(ctx, 1 << 20, SEED_C0 + 1), tmin=1e-4)
    out = {}
    for w in (2, 4):
        b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=w)
        b.build()
        # 4-wide: the persistent while-while kernel (816 against 627 Mrays/s for one thread per ray)
        topts = dict(persistent=2, refill_lanes=8) if w == 4 else {}
        hits = b.intersect(rays, **topts)
        bms = _time(torch, b.build, 20, s)
        tms = _time(torch, lambda: b.intersect(rays, out=hits, **topts), 20, s)
        out[f"w{w}"] = {"build_ms": round(bms, 4), "trace_ms": round(tms, 4),
                        "mrays_s": round((1 << 20) / (tms * 1e-3) / 1e6, 1)}
        b.destroy()
    out["build_roofline_frac"] = round(65536 * BYTES_PER_TRI_SINGLE / (out["w2"]["build_ms"] * 1e-3) / 1e9
                                       / pk["hbm_gbs"], 4)
    return out


C1_CAMERA = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)
# Trace options of the path-tracing legs: the persistent while-while kernel, refilled once 16 lanes
# are idle (19.5 ms against 21.5 ms for one thread per ray on config 1).
C1_TRACE = dict(persistent=2, refill_lanes=16)


def c1_scene():
    from fledge_gb300.scenes import icosphere, quad_light
    v, f = icosphere(8)
    lv, lf = quad_light()
    return np.concatenate([v, lv], 0), np.concatenate([f, lf + len(v)], 0), len(f)


def run_c1(ctx, torch, F, dev, with_cpu: bool):
    """Config 1: wavefront path tracing of the level-8 displaced icosphere
    (1,310,720 triangles) under a 0.2 x 0.2 light, 1920x1080 at 16 spp,
    depth 5: Mrays/s over all closest-hit and shadow rays."""
    pos, ind, lfirst = c1_scene()
    p, i = torch.from_numpy(pos).to(dev), torch.from_numpy(ind).to(dev)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=4, leaf_size=2)
    b.build()
    F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=1, max_depth=5, **C1_CAMERA, **C1_TRACE)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=16, max_depth=5, **C1_CAMERA,
                             **C1_TRACE)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    n = stats["closest_rays"] + stats["shadow_rays"]
    res = {"workload": "config 1: 1,310,720-triangle displaced icosphere, 1920x1080x16 spp, depth 5",
           "ms": round(dt * 1e3, 2), "mrays_s": round(n / dt / 1e6, 1), "closest_rays": stats["closest_rays"],
           "shadow_rays": stats["shadow_rays"], "mean_radiance": round(float(img.mean()), 6)}
    if with_cpu:
        from oracle import oracle as O
        O.build()
        O.set_threads(os.cpu_count() or 1)
        tree = O.build_bvh(pos, ind)
        stride = 5
        t0 = time.perf_counter()
        _, rays = O.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), C1_CAMERA["eye"],
                              C1_CAMERA["target"], C1_CAMERA["up"], C1_CAMERA["fov_deg"], 1920, 1080, 16, 5, stride)
        cdt = time.perf_counter() - t0
        res["cpu_mrays_s"] = round(sum(rays) / cdt / 1e6, 3)
        res["cpu_sample"] = f"every {stride}th pixel ({sum(rays)} rays, {cdt:.1f} s, {os.cpu_count()} threads)"
    b.destroy()
    return res


def run_c1_volume(ctx, torch, F, dev, with_cpu: bool):
    """Volumetric path tracing (VolPathIntegrator::Li) of the config-1 scene
    with a 128^3 noise medium (densities in [0, 0.8], sigma_s 0.8, sigma_a 0.2,
    g 0.3) filling the box [-1.5, 1.5]^3 around the sphere: 1920x1080 at
    4 spp, depth 5.  Mrays/s over closest-hit and shadow rays (the free-flight
    and ratio-tracking steps are extra work per ray)."""
    pos, ind, lfirst = c1_scene()
    p, i = torch.from_numpy(pos).to(dev), torch.from_numpy(ind).to(dev)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=4, leaf_size=2)
    b.build()
    rho = F.gen_noise_grid(ctx, 128, SEED_C2 + 16, scale=0.8)
    lo, hi = (-1.5, -1.5, -1.5), (1.5, 1.5, 1.5)
    vol = F.DenseGridVolume(rho, lo, hi, F.Medium(0.8, 0.2, 0.3), ctx)
    seed = SEED_C2 + 17
    F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=1, max_depth=5, volume=vol, seed=seed,
                **C1_CAMERA, **C1_TRACE)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=4, max_depth=5, volume=vol, seed=seed,
                             **C1_CAMERA, **C1_TRACE)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    n = stats["closest_rays"] + stats["shadow_rays"]
    res = {"workload": "config 1 + 128^3 medium around the sphere, 1920x1080x4 spp, depth 5",
           "ms": round(dt * 1e3, 2), "mrays_s": round(n / dt / 1e6, 1), "closest_rays": stats["closest_rays"],
           "shadow_rays": stats["shadow_rays"], "mean_radiance": round(float(img.mean()), 6)}
    if with_cpu:
        from oracle import oracle as O
        O.build()
        O.set_threads(os.cpu_count() or 1)
        tree = O.build_bvh(pos, ind)
        stride = 23
        grid = (rho.cpu().numpy(), lo, hi, O.Medium(0.8, 0.2, 0.3, 0.1, 0.0))
        t0 = time.perf_counter()
        _, rays = O.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), C1_CAMERA["eye"],
                              C1_CAMERA["target"], C1_CAMERA["up"], C1_CAMERA["fov_deg"], 1920, 1080, 4, 5, stride,
                              grid=grid, seed=seed)
        cdt = time.perf_counter() - t0
        res["cpu_mrays_s"] = round(sum(rays) / cdt / 1e6, 3)
        res["cpu_sample"] = f"every {stride}th pixel ({sum(rays)} rays, {cdt:.1f} s, {os.cpu_count()} threads)"
    b.destroy()
    return res


def run_c4(ctx, torch, F, dev, pk):
    """Config 4: an 8 M-triangle random soup inside a 512^3 noise volume;
    3840x2160x4 camera rays (closest hit), one shadow ray per hit toward a
    point light (any hit), transmittance of the camera rays through the volume
    with its adjoint (checkpointed), and the hit adjoint w.r.t. vertices."""
    s = torch.cuda.current_stream(dev)
    n_tri = 8_000_000
    pos = F.gen_triangles(ctx, n_tri, SEED_C3 + 40)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=4)
    b.build()
    bms = _time(torch, b.build, 5, s)
    W, H, spp = 3840, 2160, 4
    n = W * H * spp
    g = torch.Generator(device=dev).manual_seed(SEED_C3 + 41)
    pix = torch.arange(n, device=dev)
    px = (pix // spp) % W
    py = (pix // spp) // W
    jx = torch.rand(n, device=dev, generator=g)
    jy = torch.rand(n, device=dev, generator=g)
    tan = math.tan(math.radians(22.5))
    sx = ((px.float() + jx) / W * 2 - 1) * tan * (W / H)
    sy = (1 - (py.float() + jy) / H * 2) * tan
    d = torch.stack([sx, sy, torch.ones_like(sx)], 0)
    d = d / d.norm(dim=0, keepdim=True)
    o = torch.tensor([0.5, 0.5, -1.5], device=dev)[:, None].expand(3, n)
    soa = torch.cat([o, d], 0).contiguous()
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = b.intersect(rays)
    tms = _time(torch, lambda: b.intersect(rays, out=hits), 3, s)
    # shadow rays toward a point light
    light = torch.tensor([0.5, 2.0, 0.5], device=dev)[:, None]
    hp = o + d * hits["t"][None, :]
    sd = light - hp
    dist = sd.norm(dim=0)
    sd = sd / dist
    hit = hits["prim"] >= 0
    n_sh = int(hit.sum())
    sh = torch.cat([hp[:, hit], sd[:, hit], torch.full((1, n_sh), 1e-4, device=dev),
                    (dist[hit] * (1 - 1e-4))[None, :]], 0).contiguous()
    srays = F.Rays(*[sh[k] for k in range(8)])
    # Coherent camera rays keep one thread per ray (4271 against 3627 Mrays/s persistent); the
    # scattered shadow rays take the persistent while-while kernel (2765 against 2354 Mrays/s).
    sopts = dict(persistent=2, refill_lanes=16)
    occ = b.intersectP(srays, **sopts)
    sms = _time(torch, lambda: b.intersectP(srays, out=occ, **sopts), 3, s)
    # volume over the same box
    rho = F.gen_noise_grid(ctx, 512, SEED_C2 + 40)
    vol = F.DenseGridVolume(rho, medium=F.Medium(0.8, 0.2, 0.3, 0.1, 0.0), ctx=ctx)
    T, ck = vol.tr(rays, 5, checkpoint=True)
    grad = torch.zeros_like(rho)
    dL = torch.ones_like(T)
    fwd = _time(torch, lambda: vol.tr(rays, 5, checkpoint=True), 3, s)
    adj = _time(torch, lambda: vol.tr_adjoint(rays, 5, dL, T, ck, grad), 3, s)
    gpos = torch.zeros_like(pos)
    ones = torch.ones(n, device=dev)
    hadj = _time(torch, lambda: F.hit_adjoint(ctx, F.InternalTriangleMesh(pos), rays, hits, ones, None, None, gpos),
                 3, s)
    ctx.sync()
    res = {"workload": "config 4: 8M triangles, 512^3 grid, 3840x2160x4 camera + shadow rays",
           "build_ms": round(bms, 3),
           "build_roofline_frac": round(n_tri * BYTES_PER_TRI_SINGLE / (bms * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
           "primary_mrays_s": round(n / (tms * 1e-3) / 1e6, 1), "hit_rate": round(float(hit.float().mean()), 4),
           "shadow_mrays_s": round(n_sh / (sms * 1e-3) / 1e6, 1), "occluded": round(float(occ.float().mean()), 4),
           "tr_fwd_ms": round(fwd, 3), "tr_adj_ms": round(adj, 3), "adj_over_fwd": round(adj / fwd, 3),
           "hit_adjoint_ms": round(hadj, 3)}
    vol.destroy()
    b.destroy()
    return res


def run_volume(ctx, torch, F, dev):
    """Config 2: 256^3 value-noise grid in [0,4], 4,194,304 rays, ratio
    tracking forward (with checkpoints) and adjoint."""
    rho = F.gen_noise_grid(ctx, 256, SEED_C2)
    vol = F.DenseGridVolume(rho, medium=F.Medium(0.8, 0.2, 0.3, 0.1, 0.0), ctx=ctx)
    soa = F.gen_rays(ctx, 1 << 22, SEED_C2 + 1)
    rays = F.Rays.from_soa(soa)
    T, ck = vol.tr(rays, SEED_C2, checkpoint=True)
    dL = torch.ones_like(T)
    grad = torch.zeros_like(rho)
    for _ in range(3):
        vol.tr(rays, SEED_C2, checkpoint=True)
        vol.tr_adjoint(rays, SEED_C2, dL, T, ck, grad)
    s = torch.cuda.current_stream(dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    reps = 10
    torch.cuda.synchronize()
    e[0].record(s)
    for _ in range(reps):
        vol.tr(rays, SEED_C2, checkpoint=True)
    e[1].record(s)
    for _ in range(reps):
        grad.zero_()
        vol.tr_adjoint(rays, SEED_C2, dL, T, ck, grad)
    e[2].record(s)
    for _ in range(reps):
        vol.tr_adjoint(rays, SEED_C2, dL, T, None, grad)
    e[3].record(s)
    torch.cuda.synchronize()
    fwd = e[0].elapsed_time(e[1]) / reps
    adj = e[1].elapsed_time(e[2]) / reps
    adj_replay = e[2].elapsed_time(e[3]) / reps
    vol.destroy()
    return {"workload": "config 2: 256^3 grid, 4,194,304 rays", "fwd_ms": round(fwd, 4),
            "adj_ms": round(adj, 4), "adj_replay_ms": round(adj_replay, 4),
            "adj_over_fwd": round(adj / fwd, 3), "fwd_mrays_s": round((1 << 22) / (fwd * 1e-3) / 1e6, 1)}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=4)
    # defaults: the fastest setting of the sweep over node width, leaf size,
    # kernel kind and refill threshold on the first 32 scenes
    # leaf ranges of up to 3 triangles: 1244 Mrays/s against 1166 for 2, 1017 for 1 and 1232 for 4
    ap.add_argument("--leaf", type=int, default=3)
    ap.add_argument("--refill", type=int, default=8)
    ap.add_argument("--persistent", type=int, default=2)
    ap.add_argument("--stack", type=int, default=64)
    ap.add_argument("--presort-rays", action="store_true",
                    help="diagnostics only: reorder each scene's rays by a 6-D Morton key before timing")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-volume", action="store_true")
    ap.add_argument("--skip-c0", action="store_true")
    ap.add_argument("--skip-c4", action="store_true")
    ap.add_argument("--skip-c1", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-hq", action="store_true", help="skip the PLOC and SAH builder comparisons")
    ap.add_argument("--scenes", type=int, default=256, help="diagnostics only: first N scenes")
    ap.add_argument("--verbose", action="store_true", help="progress on stderr")
    args = ap.parse_args()
    global N_SCENES, _VERBOSE
    N_SCENES = args.scenes
    _VERBOSE = args.verbose
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
