#!/usr/bin/env python3
"""Benchmark of the GB300 LBVH / traversal / transmittance path.

Headline workload (one step): 256 independent random-triangle scenes with
triangle counts log-uniform in [1e3, 1e6] (34,597,655 triangles), 64 rays per
triangle (2,214,249,920 rays), built by one segmented LBVH build and traced by
one persistent closest-hit launch.  Metric: aggregate Mrays/s of the step
(build + trace), with the build time and its per-stage roofline beside it,
the one-scene-per-launch paths on the same inputs, the end-to-end rate
through host buffers, the other workloads (65,536-triangle scene, path
tracing, 256^3 volume forward/adjoint, 8 M-triangle scene), a parity leg that
checks seeded samples of every workload against the CPU oracle after the
timed region, and the CPU baseline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  All inputs are seeded synthetic data
generated on the device (Philox streams); inputs exceed the 129 MB L2, so no
flush is needed between steps.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
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

from fledge_gb300 import scenes as S  # noqa: E402  (numpy only; no GPU)

METRIC = "Mrays/s & LBVH ms, batched+adjoint vs plain on 1 GB300, t rel err ≤1e-5"
N_SCENES = S.N_SCENES
RAYS_PER_TRI = S.RAYS_PER_TRI
SEED_C0, SEED_C2, SEED_C3 = S.SEED_SOUP, S.SEED_VOLUME, S.SEED_BATCH
# Algorithmic bytes (compulsory DRAM traffic).  Per ray: 6 floats in, prim,
# t, u, v out.  Per triangle of an LBVH build, by stage: bounds (read the
# triangle) 36, Morton (read 36, write code + index 8, digit histograms 4) 48,
# four 8-bit sort passes of (code, index) pairs 4 x 16, Karras topology 20 and
# refit 100 (both in the climb); 268 in all.  A batched build adds its
# per-scene digit histograms and bucket offsets (written, scanned, read).
BYTES_PER_RAY = 24 + 16
STAGE_BYTES_PER_TRI = {"bounds": 36, "morton": 48, "sort_pass": 16, "climb": 120}
BYTES_PER_TRI = 268
TRACE_PROFILE = os.path.join(ROOT, "profiles", "k_trace_ww_config3.json")
TRACE_SOURCES = ["fledge_gb300/csrc/trace.cu", "fledge_gb300/csrc/common.cuh", "fledge_gb300/csrc/internal.h"]
TUNED = os.path.join(ROOT, "fledge_gb300", "tuned", "batched_config3.json")

_T0 = time.perf_counter()
_VERBOSE = False


def log(msg: str) -> None:
    if _VERBOSE:
        sys.stderr.write(f"[bench {time.perf_counter() - _T0:8.2f}s] {msg}\n")
        sys.stderr.flush()


def scene_counts(n: int = None) -> np.ndarray:
    return S.batched_scene_counts(N_SCENES if n is None else n)


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def source_hash(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(os.path.join(ROOT, p), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def trace_profile() -> dict:
    """The committed ncu summary of the trace kernel (machine-readable), and
    whether the kernel's sources still hash to what was captured."""
    if not os.path.exists(TRACE_PROFILE):
        return {}
    d = json.load(open(TRACE_PROFILE))
    d["stale"] = d.get("source_sha16") != source_hash(TRACE_SOURCES)
    return d


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
# CPU reference arm: the oracle restates the reference's build and traversal
# (the reference itself needs TBB/Embree/OpenVDB); run on all host cores.
# ---------------------------------------------------------------------------

def soup_np(n: int, rng) -> np.ndarray:
    cent = rng.random((n, 1, 3), dtype=np.float32)
    return (cent + (2 * rng.random((n, 3, 3), dtype=np.float32) - 1) * np.float32(0.01)).reshape(-1, 3)


def sphere_rays_np(n: int, rng) -> np.ndarray:
    u = rng.random((n, 5))
    z = 1 - 2 * u[:, 0]
    ph = 2 * np.pi * u[:, 1]
    s = np.sqrt(np.maximum(0, 1 - z * z))
    o = np.stack([0.5 + 2 * s * np.cos(ph), 0.5 + 2 * s * np.sin(ph), 0.5 + 2 * z])
    d = u[:, 2:5].T - o
    d /= np.linalg.norm(d, axis=0, keepdims=True)
    r8 = np.zeros((8, n), np.float32)
    r8[0:3], r8[3:6], r8[6], r8[7] = o, d, 1e-4, np.inf
    return r8


CPU_QUANTILES = (0.0, 0.2, 0.4, 0.6, 0.8, 1.0)
CPU_RAYS_CAP = 250_000


def cpu_sample():
    """Scenes of the batch at six quantiles of its size distribution (the
    smallest, the largest and four between, 1.33 M triangles), each with its
    64 rays per triangle capped at 250,000, generated with numpy (same
    distributions as the device generators)."""
    counts = scene_counts()
    order = np.argsort(counts, kind="stable")
    picks = [int(order[int(round(q * (len(order) - 1)))]) for q in CPU_QUANTILES]
    rng = np.random.default_rng(7)
    out = []
    for s in picks:
        n = int(counts[s])
        out.append((n, soup_np(n, rng), sphere_rays_np(min(n * RAYS_PER_TRI, CPU_RAYS_CAP), rng)))
    return out


def cpu_step(O, sample):
    """One timed pass over the sample: per scene the oracle's build
    (reference-performance mode: parallel bounds / Morton, parallel sort of
    32-byte records, parallel Karras and atomic refit) and its recursive
    closest-hit traversal, timed separately.  Returns the config-3-equivalent
    Mrays/s and the per-scene costs: seconds per triangle of build and per ray
    of trace at each sampled size, interpolated in log(size) to all 256
    scenes, give the time of the whole batch, total rays / (sum over scenes of
    n_tri x s/tri + n_rays x s/ray)."""
    sizes, b_cost, r_cost = [], [], []
    for n, pos, r8 in sample:
        t0 = time.perf_counter()
        tree = O.build_timed(pos, None, n)
        t1 = time.perf_counter()
        tree["n"] = n
        O.trace_closest(pos, None, tree, r8, O.MODE_REF)
        t2 = time.perf_counter()
        sizes.append(math.log(n))
        b_cost.append((t1 - t0) / n)
        r_cost.append((t2 - t1) / r8.shape[1])
    counts = scene_counts().astype(np.float64)
    lc = np.log(counts)
    bt = np.interp(lc, sizes, b_cost)
    rt = np.interp(lc, sizes, r_cost)
    t_batch = float(np.sum(counts * bt + RAYS_PER_TRI * counts * rt))
    rays = float(np.sum(counts) * RAYS_PER_TRI)
    return rays / t_batch / 1e6, {"sizes": [int(round(math.exp(x))) for x in sizes],
                                  "build_ns_per_tri": [round(x * 1e9, 2) for x in b_cost],
                                  "trace_ns_per_ray": [round(x * 1e9, 2) for x in r_cost],
                                  "batch_seconds": round(t_batch, 2)}


def cpu_sample_desc(sample, cores: int) -> str:
    ntri = sum(n for n, _, _ in sample)
    nr = sum(r.shape[1] for _, _, r in sample)
    return (f"{len(sample)} scenes of the batch at size quantiles {CPU_QUANTILES} ({ntri} triangles, {nr} rays, "
            f"64 rays/triangle capped at {CPU_RAYS_CAP}); oracle build and recursive closest hit timed per scene "
            f"on {cores} threads; cost per triangle and per ray interpolated in log(size) over all 256 scenes: "
            "config-3-equivalent Mrays/s = total rays / (sum n_tri s/tri + n_rays s/ray)")


def run_reference(args, rank: int) -> None:
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    sample = cpu_sample()
    for _ in range(min(max(args.warmup, 0), 1)):
        cpu_step(O, sample[:3])
    rates, wall = [], []
    detail = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        v, detail = cpu_step(O, sample)
        wall.append(time.perf_counter() - t0)
        rates.append(v)
    v = statistics.median(rates)
    n_rays = int(np.sum(scene_counts()) * RAYS_PER_TRI)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(n_rays / v / 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy, same distributions as the GPU workload)",
            "config": {"workload": "config 3: 256 batched random-triangle scenes, log-uniform [1e3,1e6] "
                                   "triangles, 64 rays/triangle; build + closest hit per scene",
                       "triangles": int(np.sum(scene_counts())), "rays": n_rays},
            "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": cpu_sample_desc(sample, cores), "model": detail,
                             "sample_seconds_per_step": round(statistics.median(wall), 2)},
            "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Parity leg (after the timed region): seeded samples against the oracle.
# ---------------------------------------------------------------------------

def compare_closest(O, pos, tree, r8, hg):
    """Prim mismatches other than exact ties, ties, t/u/v mismatches where the
    ids agree, and the largest relative t error against FP64."""
    ho = O.trace_closest(pos, None, tree, r8, O.MODE_DEV)
    diff = np.nonzero(hg["prim"] != ho["prim"])[0]
    tri = pos.reshape(-1, 3, 3)
    ties = 0
    for i in diff:
        a, b = int(hg["prim"][i]), int(ho["prim"][i])
        if a < 0 or b < 0:
            continue
        oka, ta = O.pluecker(tri[a, 0], tri[a, 1], tri[a, 2], r8[0:3, i], r8[3:6, i], O.MODE_DEV)
        okb, tb = O.pluecker(tri[b, 0], tri[b, 1], tri[b, 2], r8[0:3, i], r8[3:6, i], O.MODE_DEV)
        if oka and okb and ta[0] == tb[0]:
            ties += 1
    same = hg["prim"] == ho["prim"]
    tuv_bad = int(sum(np.count_nonzero(hg[k][same] != ho[k][same]) for k in ("t", "u", "v")))
    hit = hg["prim"] >= 0
    tuv64, ok = O.hit_values64(pos, None, tree["n"], r8, hg["prim"])
    rel = np.abs(hg["t"][hit].astype(np.float64) - tuv64[hit, 0]) / np.abs(tuv64[hit, 0])
    return {"rays": int(r8.shape[1]), "prim_mismatch": int(len(diff) - ties), "ties": int(ties),
            "tuv_mismatch": tuv_bad, "t_fp64_max_rel": float(rel.max()) if rel.size else 0.0,
            "hit_rate": round(float(hit.mean()), 4)}


def topology_mismatch(gpu: dict, ref: dict) -> int:
    bad = 0
    for k in ("morton", "perm", "split", "leaf_flags", "range_j", "parent", "leaf_parent", "bounds", "scene_bound"):
        a, b = np.asarray(gpu[k]), np.asarray(ref[k]).reshape(np.asarray(gpu[k]).shape)
        bad += int(np.count_nonzero(a != b))
    return bad


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def load_tuned() -> dict:
    """The LBVH entry of the committed autotuner record (fledge_gb300/autotune.py):
    node width, leaf size and trace options, plus what the tuner found for
    the other builders."""
    if not os.path.exists(TUNED):
        return {}
    rec = json.load(open(TUNED))
    lb = rec["per_builder"]["lbvh"]
    return {"node_width": lb["node_width"], "leaf_size": lb["leaf_size"], **lb["trace_opts"],
            "record": {"fastest_builder": rec["builder"],
                       "headline_builder": "lbvh: the timed step builds the plain LBVH, the build the metric "
                                           "names; the other builders are measured beside it",
                       "reps": rec["reps"], "when": rec["when"],
                       "search_rays": rec["workload"]["search_rays"],
                       "step_ms": {k: v["step_ms"] for k, v in rec["per_builder"].items()}}}


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
    pk = peaks()

    # ---- inputs (device-resident, generated by Philox) ----
    # Scenes are independent: with N ranks, rank r builds and traces scenes
    # r, r + N, ... of a batch of N x 256 scenes (replicas of the 256-scene
    # generator with rank-offset streams), so per-rank work stays fixed.
    counts = scene_counts()
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    roffs = offs * RAYS_PER_TRI
    n_tri, n_rays = int(offs[-1]), int(roffs[-1])
    seed = SEED_C3 + 0x100 * rank
    log(f'generating {n_tri} triangles, {n_rays} rays')
    pos = F.gen_triangles(ctx, n_tri, seed)
    soa = torch.empty((6, n_rays), dtype=torch.float32, device=dev)
    chunk = 1 << 28
    for c0 in range(0, n_rays, chunk):
        m = min(chunk, n_rays - c0)
        ps = [C.c_void_p(soa[k, c0:].data_ptr()) for k in range(6)]
        cen = (C.c_float * 3)(0.5, 0.5, 0.5)
        ctx.check(lib.flg_gen_rays(ctx.h, seed + 1, c0, m, cen, 2.0, *ps))
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = {"prim": torch.empty(n_rays, dtype=torch.int32, device=dev),
            "t": torch.empty(n_rays, dtype=torch.float32, device=dev),
            "u": torch.empty(n_rays, dtype=torch.float32, device=dev),
            "v": torch.empty(n_rays, dtype=torch.float32, device=dev)}
    mesh = F.InternalTriangleMesh(pos)
    tuned = load_tuned() if not args.no_tuned else {}
    width = args.width or tuned.get("node_width", 4)
    leaf = args.leaf or tuned.get("leaf_size", 3)
    topts = dict(persistent=args.persistent if args.persistent is not None else tuned.get("persistent", 2),
                 refill_lanes=args.refill or tuned.get("refill_lanes", 8),
                 stack_depth=args.stack or tuned.get("stack_depth", 64),
                 block_threads=tuned.get("block_threads", 256))
    bb = F.BatchedRadixBVHBuilder(mesh, offs, ctx, node_width=width, leaf_size=leaf)
    log('first build')
    bb.build()
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
    ctx.set_stage_timing(True)
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
    stages = ctx.stage_times()
    ctx.set_stage_timing(False)
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
    info = bb.info()

    # ---- roofline of the dominant kernel (the traversal launch) ----
    K = args.steps
    kern_ms = stages.get("trace", {}).get("ms", float("nan")) / K
    trace_bytes = n_rays * BYTES_PER_RAY + int(info.device_bytes)
    prof = trace_profile()
    kname = (f"k_trace_ww<{width},false,{topts['stack_depth']}>" if topts["persistent"] == 2 else
             f"k_trace_persistent<{width},false,{topts['stack_depth']}>" if topts["persistent"] else
             f"k_trace_wide<{width},false,{topts['stack_depth']}>") if width > 2 else "k_trace_bvh2<false>"
    prof_ok = bool(prof) and not prof["stale"] and prof.get("kernel") == kname
    roof = {"bound": "hbm", "achieved": round(trace_bytes / (kern_ms * 1e-3) / 1e9, 1), "peak": pk["hbm_gbs"],
            "unit": "GB/s", "frac": None,
            "traffic": round(n_rays * prof["dram_bytes_per_ray"]) if prof_ok else None,
            "kernel": kname, "kernel_ms": round(kern_ms, 3), "peak_source": pk["source"],
            "algorithmic_bytes": trace_bytes,
            "traffic_source": (f"{TRACE_PROFILE[len(ROOT) + 1:]}: ncu DRAM bytes per ray of one launch "
                               f"({prof.get('workload')}), scaled by rays" if prof_ok else
                               "none: no committed capture of this kernel's current source"),
            "limiter": prof.get("limiter") if prof_ok else None,
            # the kernel's own roof: the L1 data pipe (fraction of its wavefronts busy, ncu)
            "l1_wavefront_frac": round(prof["l1tex_data_pipe_wavefronts_pct"] / 100.0, 4) if prof_ok else None,
            "profile_source_sha16": prof.get("source_sha16"), "source_sha16": source_hash(TRACE_SOURCES)}
    roof["frac"] = round(roof["achieved"] / roof["peak"], 4)
    b_ms = statistics.median(build_ms)
    seg_bytes = 3 * 4 * 256 * 4 * N_SCENES
    build_roof = {"achieved": round((n_tri * BYTES_PER_TRI + seg_bytes) / (b_ms * 1e-3) / 1e9, 1),
                  "frac": round((n_tri * BYTES_PER_TRI + seg_bytes) / (b_ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                  "bytes_per_tri": BYTES_PER_TRI, "segment_table_bytes": seg_bytes, "stages": {}}
    for name, v in stages.items():
        if name.startswith("trace"):
            continue
        ms = v["ms"] / K
        e = {"ms": round(ms, 4), "launches_per_build": v["n"] // K, "share": round(ms / b_ms, 4)}
        if name in STAGE_BYTES_PER_TRI:
            by = STAGE_BYTES_PER_TRI[name] * n_tri * (v["n"] // K)
            e["frac"] = round(by / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4)
        if name == "collapse":
            # reads every BVH2 node record (64 B) once, writes the wide nodes
            by = 64 * n_tri + (112 if width == 4 else 224) * int(info.n_wide_nodes)
            e["bytes"] = by
            e["frac"] = round(by / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4)
        build_roof["stages"][name] = e
    trace_stages = {k: round(v["ms"] / K, 3) for k, v in stages.items() if k.startswith("trace")}
    log(f'timed: {ms_step:.1f} ms/step, build {b_ms:.2f} ms')

    # ---- parity sample of the headline workload (oracle runs later) ----
    par3 = None
    if not args.skip_parity:
        big = [int(s) for s in np.argsort(counts)[-3:]]
        rng = np.random.default_rng(0xF1ED0003)
        par3 = []
        for s in big:
            idx = np.sort(rng.choice(int(roffs[s + 1] - roffs[s]), (1 << 20) // 3, replace=False)) + int(roffs[s])
            it = torch.from_numpy(idx).to(dev)
            r8 = np.zeros((8, idx.size), np.float32)
            r8[:6] = soa[:, it].cpu().numpy()
            r8[6], r8[7] = np.float32(1e-4), np.inf
            par3.append((s, pos[3 * int(offs[s]):3 * int(offs[s + 1])].cpu().numpy(), bb.topology(scene=s), r8,
                         {k: v[it].cpu().numpy() for k, v in hits.items()}))

    # ---- e2e: host (pinned) inputs, copies inside the timed region (right
    # after the device-resident step, before the legs that build many handles) ----
    e2e = None
    if not args.skip_e2e:
        e2e = run_e2e(args, ctx, torch, F, pos, soa, offs, roffs, n_tri, n_rays, width, leaf, topts, dev, world)
    log('e2e done')

    # ---- one-scene-per-launch paths on the same inputs ----
    plain = None
    if not args.skip_plain:
        plain = {}
        sub_rays = [F.Rays(*[soa[k, roffs[s]:roffs[s + 1]] for k in range(6)], tmin_const=1e-4)
                    for s in range(N_SCENES)]
        sub_hits = [{k: v[roffs[s]:roffs[s + 1]] for k, v in hits.items()} for s in range(N_SCENES)]
        arms = [("bvh2", dict(node_width=2), {}),
                ("same_kernel", dict(node_width=width, leaf_size=leaf), topts)]
        for name, bopts, op in arms:
            handles = []
            for s in range(N_SCENES):
                h = F.RadixBVHBuilder(F.InternalTriangleMesh(pos[3 * offs[s]:3 * offs[s + 1]]), ctx, **bopts)
                h.build()
                handles.append(h)

            def plain_step():
                for s in range(N_SCENES):
                    handles[s].build()
                    handles[s].intersect(sub_rays[s], out=sub_hits[s], **op)
            plain_step()
            ctx.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.plain_steps):
                plain_step()
            e1.record(stream)
            torch.cuda.synchronize()
            pms = e0.elapsed_time(e1) / args.plain_steps
            plain[name] = {"ms_per_step": round(pms, 3), "mrays_s": round(n_rays / (pms * 1e-3) / 1e6, 2),
                           "speedup_batched_vs_plain": round(pms / ms_step, 3), "steps": args.plain_steps,
                           "kernel": "k_trace_bvh2<false>, one thread per ray" if name == "bvh2" else kname,
                           "layout": bopts, "trace_opts": op}
            for h in handles:
                h.destroy()
            del handles
            log(f'plain {name} done')
        plain["speedup_batched_vs_plain_same_kernel"] = plain["same_kernel"]["speedup_batched_vs_plain"]
        plain["speedup_batched_vs_plain_bvh2"] = plain["bvh2"]["speedup_batched_vs_plain"]

    # ---- higher-quality builders (PLOC, binned SAH, treelet-restructured LBVH) on the same scenes and rays ----
    hq = sah = tl = None
    if not args.skip_hq:
        res = {}
        for name, rounds in (("ploc", 0), ("sah", 0), ("treelet", 3), ("treelet1", 1)):
            hb = F.BatchedRadixBVHBuilder(mesh, offs, ctx, node_width=width, leaf_size=leaf,
                                          builder=name.rstrip("1"), treelet_rounds=rounds)
            hb.build()
            hb.intersect_batched(rays, roffs, out=hits, **topts)  # warm-up
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ctx.set_stage_timing(True)
            ev[0].record(stream)
            hb.build()
            ev[1].record(stream)
            torch.cuda.synchronize()
            bst = ctx.stage_times()
            ctx.set_stage_timing(False)
            hb_ms = ev[0].elapsed_time(ev[1])
            ctx.sync()
            ev[1].record(stream)
            hb.intersect_batched(rays, roffs, out=hits, **topts)
            ev[2].record(stream)
            torch.cuda.synchronize()
            ht_ms = ev[1].elapsed_time(ev[2])
            res[name] = {"builder": {"ploc": "ploc (radius 16)", "sah": "binned SAH (16 buckets, reference rule)",
                                     "treelet": "LBVH + 3 rounds of 7-leaf treelet restructuring",
                                     "treelet1": "LBVH + 1 round of 7-leaf treelet restructuring"}[name],
                         "build_ms": round(hb_ms, 3), "trace_ms": round(ht_ms, 2),
                         "mrays_s": round(n_rays / (ht_ms * 1e-3) / 1e6, 1),
                         "trace_speedup_vs_lbvh": round(statistics.median(trace_ms) / ht_ms, 3),
                         "step_ms": round(hb_ms + ht_ms, 2),
                         "build_stages_ms": {k: round(v["ms"], 3) for k, v in bst.items()}}
            hb.destroy()
            log(f'{name} builder done')
        hq, sah, tl = res["ploc"], res["sah"], res["treelet"]
        tl["one_round"] = res["treelet1"]


    # ---- the other workloads ----
    vol = run_volume(ctx, torch, F, dev, pk) if not args.skip_volume else None
    log("config 0")
    c0 = run_c0(ctx, torch, F, dev, pk) if not args.skip_c0 else None
    log("config 4")
    c4 = run_c4(ctx, torch, F, dev, pk) if not args.skip_c4 else None
    log("config 1")
    c1 = run_c1(ctx, torch, F, dev, rank == 0) if not args.skip_c1 else None
    log("config 1 with a medium")
    c1v = run_c1_volume(ctx, torch, F, dev, rank == 0 and not args.skip_cpu) if not args.skip_c1 else None
    total_launches = lib.flg_ctx_launch_count(ctx.h) - launches0
    bb.destroy()
    del pos, soa, rays, hits
    ctx.close()

    # ---- CPU legs (rank 0): parity against the oracle, CPU baseline ----
    parity = cpu = None
    if rank == 0 and not (args.skip_cpu and args.skip_parity):
        from oracle import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        O.set_threads(cores)
        if not args.skip_parity:
            log("parity leg")
            parity = {}
            if par3:
                p3 = {"scenes": [], "topology_mismatch": 0}
                for s, sp, topo, r8, hg in par3:
                    tree = O.build_bvh(sp)
                    p3["topology_mismatch"] += topology_mismatch(topo, tree)
                    p3["scenes"].append(dict(scene=s, triangles=int(tree["n"]), **compare_closest(O, sp, tree, r8, hg)))
                p3["prim_mismatch"] = sum(x["prim_mismatch"] for x in p3["scenes"])
                p3["tuv_mismatch"] = sum(x["tuv_mismatch"] for x in p3["scenes"])
                p3["t_fp64_max_rel"] = max(x["t_fp64_max_rel"] for x in p3["scenes"])
                parity["config3_largest_scenes"] = p3
            for key, leg in (("config0", c0), ("config4", c4), ("config2", vol), ("config1", c1)):
                chk = leg.pop("_parity", None) if leg else None
                if chk is not None:
                    parity[key] = chk(O)
            parity["mismatch_total"] = int(sum(v.get("prim_mismatch", 0) + v.get("tuv_mismatch", 0) +
                                               v.get("topology_mismatch", 0) + v.get("occlusion_mismatch", 0) +
                                               v.get("T_mismatch", 0) + v.get("pixel_mismatch", 0)
                                               for v in parity.values() if isinstance(v, dict)))
        if not args.skip_cpu:
            log("CPU baseline")
            sample = cpu_sample()
            v, detail = cpu_step(O, sample)
            cpu = {"value": round(v, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                   "sample": cpu_sample_desc(sample, cores), "model": detail}
            if sah is not None:
                n, sp, _ = sample[-1]
                t0 = time.perf_counter()
                O.build_bvh_sah(sp)
                dt = time.perf_counter() - t0
                sah.update({"cpu_mtris_s": round(n / dt / 1e6, 3),
                            "gpu_mtris_s": round(n_tri / (sah["build_ms"] * 1e-3) / 1e6, 1),
                            "cpu_sample": f"oracle SAH build of one {n}-triangle scene, 1 thread ({dt:.2f} s)"})
    for leg in (c0, c4, vol, c1):
        if leg:
            leg.pop("_parity", None)

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded Philox on device)",
                "config": {"workload": "config 3: 256 batched random-triangle scenes, log-uniform [1e3,1e6] "
                                       "triangles, 64 rays/triangle; segmented LBVH build + persistent trace",
                           "triangles": n_tri, "rays": n_rays, "node_width": width, "leaf_size": leaf,
                           "trace_opts": topts, "tuned_from": (TUNED[len(ROOT) + 1:] if tuned else None),
                           "autotuner": tuned.get("record"),
                           "l2": "inputs larger than L2 (no flush)", "parallelism": f"scene shards x{world}"},
                "build_ms": round(b_ms, 3), "trace_ms": round(statistics.median(trace_ms), 3),
                "trace_stages_ms": trace_stages, "hit_rate": round(hit_rate, 4),
                "build_roofline": build_roof, "roofline": roof, "plain": plain, "volume": vol,
                "hq_builder": hq, "sah_builder": sah, "treelet_builder": tl, "config0": c0, "config1": c1, "config1_volume": c1v,
                "config4": c4, "parity": parity, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
                "gpu_launches": int(launches), "gpu_launches_total": int(total_launches)}
        print(json.dumps(line), flush=True)


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
    # every rank of this node pins its own copy; all ranks decide together
    ranks_here = int(os.environ.get("LOCAL_WORLD_SIZE", "1"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
    fits = torch.tensor([1 if need * ranks_here <= 0.6 * avail else 0], device=dev)
    if dist:
        tdist.all_reduce(fits, op=tdist.ReduceOp.MIN)
    if int(fits.item()) == 0:
        return {"value": None, "unit": "Mrays/s",
                "skipped": f"needs {need * ranks_here / 1e9:.0f} GB pinned host memory for {ranks_here} rank(s), "
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
    # Groups are traced on two contexts (two streams) in turn, so that a
    # group's persistent kernel fills the SMs that the previous group's last
    # rays leave idle.
    side = torch.cuda.Stream(dev)
    ctx2 = F.Context(dev.index or 0, side)
    tstreams, tctx = (main, side), (ctx, ctx2)
    # scene groups of about 64 M rays: the first trace waits for one group's
    # upload and the last download follows the last trace
    groups, g0 = [], 0
    for s in range(N_SCENES):
        if roffs[s + 1] - roffs[g0] >= (1 << 26) or s == N_SCENES - 1:
            groups.append((g0, s + 1))
            g0 = s + 1

    # One copy stream carries every copy in order (triangles, all ray groups,
    # then each group's hits once its trace is done): on this system a
    # host-to-device and a device-to-host copy running at once each drop to
    # ~60 GB/s, against ~200 GB/s alone.
    # Busy time of the copy stream inside the timed steps: events around
    # every copy batch (each recorded after the batch's wait, so it spans the
    # copies alone).  The copies are hidden behind the traces while the host
    # keeps up; on a shared host their rate varies from run to run.
    spans, timing = [], [False]

    def timed_copy(fn, kind):
        if not timing[0]:
            fn()
            return
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(copy)
        fn()
        e1.record(copy)
        spans.append((kind, e0, e1))

    def e2e_step():
        with torch.cuda.stream(copy):
            timed_copy(lambda: d_pos.copy_(h_pos, non_blocking=True), "h2d")
            pos_ev = torch.cuda.Event()
            pos_ev.record(copy)
        main.wait_event(pos_ev)
        bb.build()
        built = torch.cuda.Event()
        built.record(main)
        side.wait_event(built)
        up = []
        with torch.cuda.stream(copy):
            for (a, b) in groups:
                r0, r1 = int(roffs[a]), int(roffs[b])
                # one contiguous copy per ray column: a strided [6, m] slice
                # would go through a pageable host temporary (~55 GB/s)
                timed_copy(lambda: [d_rays[k, r0:r1].copy_(h_rays[k, r0:r1], non_blocking=True)
                                    for k in range(6)], "h2d")
                ev = torch.cuda.Event()
                ev.record(copy)
                up.append(ev)
        for gi, (a, b) in enumerate(groups):
            r0, r1 = int(roffs[a]), int(roffs[b])
            ts = tstreams[gi & 1]
            ts.wait_event(up[gi])
            ro = np.zeros(N_SCENES + 1, np.int64)
            ro[a + 1:b + 1] = roffs[a + 1:b + 1] - roffs[a]
            ro[b + 1:] = ro[b]
            sub_rays = F.Rays(*[d_rays[k, r0:r1] for k in range(6)], tmin_const=1e-4)
            sub_out = {k: v[r0:r1] for k, v in d_out.items()}
            bb.intersect_batched(sub_rays, ro, out=sub_out, ctx=tctx[gi & 1], **topts)
            done = torch.cuda.Event()
            done.record(ts)
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                timed_copy(lambda: [h_out[k][r0:r1].copy_(d_out[k][r0:r1], non_blocking=True)
                                    for k in h_out], "d2h")
        main.wait_stream(side)
        main.wait_stream(copy)

    # Copy rates of this machine, each direction alone (one column of rays in,
    # one hit array out; outside the timed region): the e2e step hides its
    # copies behind the traces except the first group in and the last out.
    def rate(dst, src):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(main)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record(main)
        torch.cuda.synchronize()
        return round(3 * src.numel() * src.element_size() / (e0.elapsed_time(e1) * 1e6), 1)

    m = min(n_rays, 1 << 28)
    h2d_gbs = rate(d_rays[0, :m], h_rays[0, :m])
    h2d_last_gbs = rate(d_rays[5, n_rays - m:], h_rays[5, n_rays - m:])
    d2h_gbs = rate(h_out["t"][:m], d_out["t"][:m])
    d2h_last_gbs = rate(h_out["v"][n_rays - m:], d_out["v"][n_rays - m:])

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    timing[0] = True
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    timing[0] = False
    busy = {"h2d": 0.0, "d2h": 0.0}
    for kind, e0, e1 in spans:
        busy[kind] += e0.elapsed_time(e1) / args.steps
    h2d_b, d2h_b = n_tri * 36 + n_rays * 24, n_rays * 16
    if dist:  # the whole job's step: the slowest rank
        t = torch.tensor([dt], device=dev, dtype=torch.float64)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        dt = float(t.item())
    ok = bool(torch.equal(h_out["prim"][:1 << 20].to(dev), d_out["prim"][:1 << 20]))
    bb.destroy()
    ctx2.close()
    return {"value": round(world * n_rays / dt / 1e6, 2), "unit": "Mrays/s",
            "h2d_bytes_per_step": int(n_tri * 36 + n_rays * 24), "d2h_bytes_per_step": int(n_rays * 16),
            "ms_per_step": round(dt * 1e3, 3), "host_readback_consistent": ok,
            "copy_stream_in_step": {"h2d_ms": round(busy["h2d"], 1), "d2h_ms": round(busy["d2h"], 1),
                                    "h2d_gbs": round(h2d_b / (busy["h2d"] * 1e6), 1) if busy["h2d"] else None,
                                    "d2h_gbs": round(d2h_b / (busy["d2h"] * 1e6), 1) if busy["d2h"] else None},
            "copy_gbs_alone": {"h2d_first_gb": h2d_gbs, "h2d_last_gb": h2d_last_gbs, "d2h_first_gb": d2h_gbs,
                               "d2h_last_gb": d2h_last_gbs}, "ray_groups": len(groups)}


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


def _graph_step(torch, F, ctx, b, pos, rays, hits, topts, dev):
    """A rebuild + trace step captured once into a CUDA graph
    (flg_graph_begin / end) and replayed, against the same step issued as
    plain launches: on a small workload the launches are a visible part of
    the step."""
    side = torch.cuda.Stream(dev)
    ctx2 = F.Context(dev.index or 0, side)
    r, hs, op = rays.struct(), F._hits_struct(hits), F._trace_opts(**topts)
    # the first trace on a context allocates its scratch: before the capture
    ctx2.check(ctx2.lib.flg_trace_closest(ctx2.h, b.h, C.byref(r), rays.n, C.byref(op), C.byref(hs)))
    ctx2.sync()
    g = C.c_void_p()
    with torch.cuda.stream(side):
        ctx2.check(ctx2.lib.flg_graph_begin(ctx2.h))
        ctx2.check(ctx2.lib.flg_bvh_rebuild(ctx2.h, b.h, C.c_void_p(pos.data_ptr())))
        ctx2.check(ctx2.lib.flg_trace_closest(ctx2.h, b.h, C.byref(r), rays.n, C.byref(op), C.byref(hs)))
        ctx2.check(ctx2.lib.flg_graph_end(ctx2.h, C.byref(g)))

    def plain():
        ctx2.check(ctx2.lib.flg_bvh_rebuild(ctx2.h, b.h, C.c_void_p(pos.data_ptr())))
        ctx2.check(ctx2.lib.flg_trace_closest(ctx2.h, b.h, C.byref(r), rays.n, C.byref(op), C.byref(hs)))

    res = {}
    for name, fn in (("graph", lambda: ctx2.check(ctx2.lib.flg_graph_launch(ctx2.h, g))), ("plain", plain)):
        fn()
        torch.cuda.synchronize()
        res[name + "_step_ms"] = round(_time(torch, fn, 50, side), 4)
    ctx2.sync()
    ctx2.lib.flg_graph_destroy(g)
    ctx2.close()
    res["launches_per_step"] = "build (about 14 kernels) + trace (3), one graph launch when replayed"
    return res


def run_c0(ctx, torch, F, dev, pk):
    """Config 0: 65,536 triangles, 1,048,576 rays: build ms and closest-hit
    Mrays/s for the plain BVH2 kernel and the 4-wide kernel."""
    s = torch.cuda.current_stream(dev)
    pos = F.gen_triangles(ctx, 65536, SEED_C0)
    soa = F.gen_rays(ctx, 1 << 20, SEED_C0 + 1)
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    out = {}
    keep = {}
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
        keep[w] = (b.topology(), {k: v.cpu().numpy() for k, v in hits.items()})
        if w == 4:
            out["w4_graph"] = _graph_step(torch, F, ctx, b, pos, rays, hits, topts, dev)
        b.destroy()
    out["build_roofline_frac"] = round(65536 * BYTES_PER_TRI / (out["w2"]["build_ms"] * 1e-3) / 1e9
                                       / pk["hbm_gbs"], 4)
    ph = pos.cpu().numpy()
    r8 = np.zeros((8, 1 << 20), np.float32)
    r8[:6] = soa.cpu().numpy()
    r8[6], r8[7] = np.float32(1e-4), np.inf

    def check(O):
        tree = O.build_bvh(ph)
        res = {"topology_mismatch": topology_mismatch(keep[2][0], tree)}
        for w in (2, 4):
            c = compare_closest(O, ph, tree, r8, keep[w][1])
            res[f"w{w}"] = c
        res["prim_mismatch"] = res["w2"]["prim_mismatch"] + res["w4"]["prim_mismatch"]
        res["tuv_mismatch"] = res["w2"]["tuv_mismatch"] + res["w4"]["tuv_mismatch"]
        return res
    out["_parity"] = check
    return out


def run_c1(ctx, torch, F, dev, with_cpu: bool):
    """Config 1: wavefront path tracing of the level-8 displaced icosphere
    (1,310,720 triangles) under a 0.2 x 0.2 light, 1920x1080 at 16 spp,
    depth 5: Mrays/s over all closest-hit and shadow rays."""
    pos, ind, lfirst = S.path_tracing_scene(8)
    cam = S.PATH_TRACING_CAMERA
    topts = dict(persistent=2, refill_lanes=16)
    p, i = torch.from_numpy(pos).to(dev), torch.from_numpy(ind).to(dev)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=4, leaf_size=2)
    b.build()
    F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=1, max_depth=5, **cam, **topts)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=16, max_depth=5, **cam, **topts)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    n = stats["closest_rays"] + stats["shadow_rays"]
    res = {"workload": "config 1: 1,310,720-triangle displaced icosphere, 1920x1080x16 spp, depth 5",
           "ms": round(dt * 1e3, 2), "mrays_s": round(n / dt / 1e6, 1), "closest_rays": stats["closest_rays"],
           "shadow_rays": stats["shadow_rays"], "mean_radiance": round(float(img.mean()), 6)}
    gimg = img.cpu().numpy().reshape(-1, 3)
    b.destroy()
    stride = 5

    def check(O):
        """The oracle's PathIntegrator::Li restatement on every 5th pixel:
        parity of those pixels and the CPU path-tracing rate."""
        tree = O.build_bvh(pos, ind)
        t0 = time.perf_counter()
        ref, rays = O.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"], cam["target"],
                                cam["up"], cam["fov_deg"], 1920, 1080, 16, 5, stride)
        cdt = time.perf_counter() - t0
        res["cpu_mrays_s"] = round(sum(rays) / cdt / 1e6, 3)
        res["cpu_sample"] = f"every {stride}th pixel ({sum(rays)} rays, {cdt:.1f} s, {os.cpu_count()} threads)"
        ref = ref.reshape(-1, 3)[::stride]
        g = gimg[::stride]
        close = np.all(np.abs(g - ref) <= 1e-4 * np.maximum(np.abs(ref), 1.0), axis=1)
        return {"pixels": int(ref.shape[0]), "pixel_mismatch_frac": round(float(1 - close.mean()), 6),
                "mean_rel_diff": float(abs(g.mean() - ref.mean()) / ref.mean()),
                "note": "pixels whose paths diverge on a last-ulp difference of a bounce direction (CUDA's vs libm's "
                        "cos/sin) are counted, not failed; the GPU tests bound them at 0.5 %"}
    if with_cpu:
        res["_parity"] = check
    return res


def run_c1_volume(ctx, torch, F, dev, with_cpu: bool):
    """Volumetric path tracing (VolPathIntegrator::Li) of the config-1 scene
    with a 128^3 noise medium (densities in [0, 0.8], sigma_s 0.8, sigma_a 0.2,
    g 0.3) filling the box [-1.5, 1.5]^3 around the sphere: 1920x1080 at
    4 spp, depth 5.  Mrays/s over closest-hit and shadow rays (the free-flight
    and ratio-tracking steps are extra work per ray)."""
    pos, ind, lfirst = S.path_tracing_scene(8)
    cam = S.PATH_TRACING_CAMERA
    topts = dict(persistent=2, refill_lanes=16)
    p, i = torch.from_numpy(pos).to(dev), torch.from_numpy(ind).to(dev)
    b = F.RadixBVHBuilder(F.InternalTriangleMesh(p, i), ctx, node_width=4, leaf_size=2)
    b.build()
    rho = F.gen_noise_grid(ctx, 128, SEED_C2 + 16, scale=0.8)
    lo, hi = (-1.5, -1.5, -1.5), (1.5, 1.5, 1.5)
    vol = F.DenseGridVolume(rho, lo, hi, F.Medium(0.8, 0.2, 0.3), ctx)
    seed = SEED_C2 + 17
    F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=1, max_depth=5, volume=vol, seed=seed,
                **cam, **topts)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img, stats = F.pathtrace(ctx, b, lfirst, 2, width=1920, height=1080, spp=4, max_depth=5, volume=vol, seed=seed,
                             **cam, **topts)
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
        _, rays = O.pathtrace(pos, ind, tree, lfirst, 2, (10, 10, 10), (0.7, 0.7, 0.7), cam["eye"],
                              cam["target"], cam["up"], cam["fov_deg"], 1920, 1080, 4, 5, stride,
                              grid=grid, seed=seed)
        cdt = time.perf_counter() - t0
        res["cpu_mrays_s"] = round(sum(rays) / cdt / 1e6, 3)
        res["cpu_sample"] = f"every {stride}th pixel ({sum(rays)} rays, {cdt:.1f} s, {os.cpu_count()} threads)"
    vol.destroy()
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
    ctx.set_stage_timing(True)
    bms = _time(torch, b.build, 5, s)
    stages = ctx.stage_times()
    ctx.set_stage_timing(False)
    soa = S.camera_rays_4k(torch, dev)
    n = soa.shape[1]
    rays = F.Rays.from_soa(soa, tmin=1e-4)
    hits = b.intersect(rays)
    tms = _time(torch, lambda: b.intersect(rays, out=hits), 3, s)
    # shadow rays toward a point light
    light = torch.tensor([0.5, 2.0, 0.5], device=dev)[:, None]
    hp = soa[0:3] + soa[3:6] * hits["t"][None, :]
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
    # The plain path on the same rays: BVH2 nodes, one thread per ray (k_trace_bvh2)
    b2 = F.RadixBVHBuilder(F.InternalTriangleMesh(pos), ctx, node_width=2)
    b2.build()
    hits2 = b2.intersect(rays)
    tms2 = _time(torch, lambda: b2.intersect(rays, out=hits2), 3, s)
    occ2 = b2.intersectP(srays)
    sms2 = _time(torch, lambda: b2.intersectP(srays, out=occ2), 3, s)
    same_occ = bool(torch.equal(occ2, occ))
    del hits2, occ2
    b2.destroy()
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
           "build_roofline_frac": round(n_tri * BYTES_PER_TRI / (bms * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
           "build_stages_ms": {k: round(v["ms"] / 5, 4) for k, v in stages.items()},
           "primary_mrays_s": round(n / (tms * 1e-3) / 1e6, 1), "hit_rate": round(float(hit.float().mean()), 4),
           "shadow_mrays_s": round(n_sh / (sms * 1e-3) / 1e6, 1), "occluded": round(float(occ.float().mean()), 4),
           "plain_bvh2": {"kernel": "k_trace_bvh2, one thread per ray, BVH2 nodes",
                          "primary_mrays_s": round(n / (tms2 * 1e-3) / 1e6, 1),
                          "shadow_mrays_s": round(n_sh / (sms2 * 1e-3) / 1e6, 1),
                          "primary_speedup": round(tms2 / tms, 3), "shadow_speedup": round(sms2 / sms, 3),
                          "same_occlusion": same_occ},
           "tr_fwd_ms": round(fwd, 3), "tr_adj_ms": round(adj, 3), "adj_over_fwd": round(adj / fwd, 3),
           "hit_adjoint_ms": round(hadj, 3)}
    # parity sample: 1 M camera rays and the shadow rays of their hits
    rng = np.random.default_rng(0xF1ED0004)
    idx = np.sort(rng.choice(n, 1 << 20, replace=False))
    it = torch.from_numpy(idx).to(dev)
    r8 = np.zeros((8, idx.size), np.float32)
    r8[:6] = soa[:, it].cpu().numpy()
    r8[6], r8[7] = np.float32(1e-4), np.inf
    hg = {k: v[it].cpu().numpy() for k, v in hits.items()}
    srank = torch.cumsum(hit.to(torch.int64), 0) - 1
    sidx = srank[it[hit[it]]]
    s8 = sh[:, sidx].cpu().numpy()
    occ_g = occ[sidx].cpu().numpy().astype(bool)
    topo = b.topology()
    ph = pos.cpu().numpy()

    def check(O):
        tree = O.build_bvh(ph)
        r = compare_closest(O, ph, tree, r8, hg)
        r["topology_mismatch"] = topology_mismatch(topo, tree)
        occ_o = O.trace_any(ph, None, tree, s8, O.MODE_DEV).astype(bool)
        r["shadow_rays"] = int(s8.shape[1])
        r["occlusion_mismatch"] = int(np.count_nonzero(occ_o != occ_g))
        return r
    res["_parity"] = check
    vol.destroy()
    b.destroy()
    return res


def run_volume(ctx, torch, F, dev, pk):
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
    m = 1 << 16
    r8 = np.zeros((8, m), np.float32)
    r8[:6] = soa[:, :m].cpu().numpy()
    r8[7] = np.inf
    Tg = T[:m].cpu().numpy()
    ckg = {k: v[:m].cpu().numpy() for k, v in ck.items()}
    rho_h = rho.cpu().numpy()
    vol.destroy()

    class Med:
        sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0

    def check(O):
        To, cko = O.volume_tr(rho_h, [0, 0, 0], [1, 1, 1], Med, r8, SEED_C2, want_ckpt=True)
        bad = int(np.count_nonzero(To != Tg))
        bad_ck = int(np.count_nonzero(cko["k"] != ckg["k"].view(np.uint32)) + np.count_nonzero(cko["t"] != ckg["t"]) +
                     np.count_nonzero(cko["c"] != ckg["c"]))
        return {"rays": m, "T_mismatch": bad, "checkpoint_mismatch": bad_ck,
                "note": "finite differences of the adjoint at this size run in tests/test_gpu_fullsize.py"}
    return {"workload": "config 2: 256^3 grid, 4,194,304 rays", "fwd_ms": round(fwd, 4),
            "adj_ms": round(adj, 4), "adj_replay_ms": round(adj_replay, 4),
            "adj_over_fwd": round(adj / fwd, 3), "fwd_mrays_s": round((1 << 22) / (fwd * 1e-3) / 1e6, 1),
            "_parity": check}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # layout and trace options: the tuned record (fledge_gb300/tuned/) unless given
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--leaf", type=int, default=0)
    ap.add_argument("--refill", type=int, default=0)
    ap.add_argument("--persistent", type=int, default=None)
    ap.add_argument("--stack", type=int, default=0)
    ap.add_argument("--no-tuned", action="store_true", help="ignore the tuned record (defaults: 4-wide, leaf 3)")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-volume", action="store_true")
    ap.add_argument("--skip-c0", action="store_true")
    ap.add_argument("--skip-c4", action="store_true")
    ap.add_argument("--skip-c1", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-parity", action="store_true")
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
