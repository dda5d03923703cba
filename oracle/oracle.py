"""ctypes wrapper of the CPU oracle (liboracle.so, built from oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py, always as the checker, never on the product path.
All arrays are host numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

MODE_REF, MODE_DEFECT, MODE_DEV, MODE_MT = 0, 1, 2, 3

_lib = None


def build() -> str:
    src = os.path.join(HERE, "oracle.cpp")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


class Medium(C.Structure):
    _fields_ = [("sigma_s", C.c_float), ("sigma_a", C.c_float), ("g", C.c_float),
                ("rr_threshold", C.c_float), ("majorant", C.c_float)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.orc_build.restype = C.c_int64
        _lib.orc_grid_majorant.restype = C.c_float
        _lib.orc_grid_majorant.argtypes = [C.c_void_p, C.c_int64]
        _lib.orc_hg_p.restype = C.c_float
        _lib.orc_num_threads.restype = C.c_int
        for name in ("orc_hit_normals", "orc_volume_tr64_sub", "orc_volume_tr_adjoint_vox", "orc_stream_uniforms", "orc_volume_tr", "orc_volume_tr64", "orc_volume_tr_adjoint",
                     "orc_volume_sample"):
            getattr(_lib, name).restype = None
    return _lib


_keep = []


def _p(a):
    """Pointer to a numpy array's data.  The array is kept alive until the
    next top-level oracle call (temporaries built inline in an argument list
    would otherwise be freed before the C function runs)."""
    if a is None:
        return None
    _keep.append(a)
    if len(_keep) > 256:
        del _keep[:128]
    return C.c_void_p(a.ctypes.data)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(out))
    return out


def logf(x):
    x = _f32(x)
    y = np.zeros_like(x)
    lib().orc_logf(_p(x), _p(y), C.c_int64(x.size))
    return y


def stream_uniforms(seed: int, ray: int, n: int):
    out = np.zeros(n, np.float32)
    lib().orc_stream_uniforms(C.c_uint64(seed), C.c_int64(ray), C.c_int32(n), _p(out))
    return out


def scene_bound(pos, idx, n_tri):
    pos, idx = _f32(pos), _i32(idx)
    out = np.zeros(6, np.float32)
    lib().orc_scene_bound(_p(pos), _p(idx), C.c_int64(n_tri), _p(out))
    return out


def morton(pos, idx, n_tri, bound6):
    pos, idx, b = _f32(pos), _i32(idx), _f32(bound6)
    out = np.zeros(n_tri, np.uint32)
    lib().orc_morton(_p(pos), _p(idx), C.c_int64(n_tri), _p(b), _p(out))
    return out


def sort(codes):
    codes = np.ascontiguousarray(codes, np.uint32)
    n = codes.size
    s = np.zeros(n, np.uint32)
    p = np.zeros(n, np.int32)
    lib().orc_sort(_p(codes), C.c_int64(n), _p(s), _p(p))
    return s, p


def karras(sorted_codes):
    sc = np.ascontiguousarray(sorted_codes, np.uint32)
    n = sc.size
    m = max(n - 1, 0)
    split = np.zeros(m, np.int32)
    leaf = np.zeros(m, np.uint8)
    rj = np.zeros(m, np.int32)
    parent = np.zeros(m, np.int32)
    lp = np.zeros(n, np.int32)
    lib().orc_karras(_p(sc), C.c_int64(n), _p(split), _p(leaf), _p(rj), _p(parent), _p(lp))
    return {"split": split, "leaf_flags": leaf, "range_j": rj, "parent": parent, "leaf_parent": lp}


def refit(pos, idx, n, perm, topo):
    pos, idx = _f32(pos), _i32(idx)
    nb = np.zeros((max(n - 1, 0), 6), np.float32)
    lib().orc_refit(_p(pos), _p(idx), C.c_int64(n), _p(_i32(perm)), _p(topo["split"]), _p(topo["leaf_flags"]),
                    _p(topo["parent"]), _p(topo["leaf_parent"]), _p(nb))
    return nb


def build_bvh(pos, idx=None, n_tri=None):
    """Full reference-order build: dict with morton (sorted), perm, Karras
    arrays, node bounds and the scene bound."""
    pos = _f32(pos).reshape(-1, 3)
    idx = None if idx is None else _i32(idx).reshape(-1, 3)
    n = idx.shape[0] if idx is not None else pos.shape[0] // 3
    if n_tri is not None:
        n = n_tri
    b = scene_bound(pos, idx, n)
    codes = morton(pos, idx, n, b)
    sc, perm = sort(codes)
    topo = karras(sc)
    topo["bounds"] = refit(pos, idx, n, perm, topo)
    topo.update({"morton": sc, "perm": perm, "scene_bound": b, "codes_unsorted": codes, "n": n})
    return topo


def build_bvh_sah(pos, idx=None, n_tri=None):
    """Binned-SAH build (BasicBVHBuilder's ESAH rule at every node) in the
    Karras arrays' form: perm, split, leaf_flags, range_j, parent,
    leaf_parent, node bounds and the scene bound."""
    pos = _f32(pos).reshape(-1, 3)
    idx = None if idx is None else _i32(idx).reshape(-1, 3)
    n = idx.shape[0] if idx is not None else pos.shape[0] // 3
    if n_tri is not None:
        n = n_tri
    m = max(n - 1, 0)
    t = {"perm": np.zeros(n, np.int32), "split": np.zeros(m, np.int32), "leaf_flags": np.zeros(m, np.uint8),
         "range_j": np.zeros(m, np.int32), "parent": np.zeros(m, np.int32), "leaf_parent": np.zeros(n, np.int32),
         "bounds": np.zeros((m, 6), np.float32)}
    lib().orc_build_sah(_p(pos), _p(idx), C.c_int64(n), _p(t["perm"]), _p(t["split"]), _p(t["leaf_flags"]),
                        _p(t["range_j"]), _p(t["parent"]), _p(t["leaf_parent"]), _p(t["bounds"]))
    t.update({"scene_bound": scene_bound(pos, idx, n), "n": n})
    return t


def build_bvh_treelet(pos, idx=None, n_tri=None, rounds=3):
    """The LBVH after `rounds` passes of treelet restructuring (7-leaf
    treelets, SAH), renumbered in depth-first leaf order, in the Karras
    arrays' form: perm, split, leaf_flags, range_j, parent, leaf_parent, node
    bounds and the scene bound."""
    pos = _f32(pos).reshape(-1, 3)
    idx = None if idx is None else _i32(idx).reshape(-1, 3)
    n = idx.shape[0] if idx is not None else pos.shape[0] // 3
    if n_tri is not None:
        n = n_tri
    m = max(n - 1, 0)
    t = {"perm": np.zeros(n, np.int32), "split": np.zeros(m, np.int32), "leaf_flags": np.zeros(m, np.uint8),
         "range_j": np.zeros(m, np.int32), "parent": np.zeros(m, np.int32), "leaf_parent": np.zeros(n, np.int32),
         "bounds": np.zeros((m, 6), np.float32)}
    lib().orc_build_treelet(_p(pos), _p(idx), C.c_int64(n), C.c_int32(rounds), _p(t["perm"]), _p(t["split"]),
                            _p(t["leaf_flags"]), _p(t["range_j"]), _p(t["parent"]), _p(t["leaf_parent"]),
                            _p(t["bounds"]))
    t.update({"scene_bound": scene_bound(pos, idx, n), "n": n})
    return t


def build_timed(pos, idx, n):
    """Reference-performance build (parallel, 32-byte records); returns arrays."""
    pos, idx = _f32(pos), _i32(idx)
    m = max(n - 1, 0)
    out = {"morton": np.zeros(n, np.uint32), "perm": np.zeros(n, np.int32), "split": np.zeros(m, np.int32),
           "leaf_flags": np.zeros(m, np.uint8), "range_j": np.zeros(m, np.int32),
           "parent": np.zeros(m, np.int32), "leaf_parent": np.zeros(n, np.int32),
           "bounds": np.zeros((m, 6), np.float32)}
    lib().orc_build(_p(pos), _p(idx), C.c_int64(n), _p(out["morton"]), _p(out["perm"]), _p(out["split"]),
                    _p(out["leaf_flags"]), _p(out["range_j"]), _p(out["parent"]), _p(out["leaf_parent"]),
                    _p(out["bounds"]))
    return out


def _rays8(rays):
    r = _f32(rays)
    assert r.ndim == 2 and r.shape[0] == 8
    return r


def trace_closest(pos, idx, tree, rays, mode=MODE_REF):
    pos, idx, r = _f32(pos), _i32(idx), _rays8(rays)
    n = r.shape[1]
    prim = np.zeros(n, np.int32)
    t, u, v = (np.zeros(n, np.float32) for _ in range(3))
    lib().orc_trace_closest(_p(pos), _p(idx), C.c_int64(tree["n"]), _p(_i32(tree["perm"])),
                            _p(_i32(tree["split"])), _p(np.ascontiguousarray(tree["leaf_flags"], np.uint8)),
                            _p(_f32(tree["bounds"])), _p(r), C.c_int64(n), C.c_int32(mode), _p(prim), _p(t),
                            _p(u), _p(v))
    return {"prim": prim, "t": t, "u": u, "v": v}


def trace_any(pos, idx, tree, rays, mode=MODE_REF):
    pos, idx, r = _f32(pos), _i32(idx), _rays8(rays)
    n = r.shape[1]
    occ = np.zeros(n, np.uint8)
    lib().orc_trace_any(_p(pos), _p(idx), C.c_int64(tree["n"]), _p(_i32(tree["perm"])), _p(_i32(tree["split"])),
                        _p(np.ascontiguousarray(tree["leaf_flags"], np.uint8)), _p(_f32(tree["bounds"])), _p(r),
                        C.c_int64(n), C.c_int32(mode), _p(occ))
    return occ


def pluecker(a, b, c, o, d, mode=MODE_REF):
    out = np.zeros(3, np.float32)
    ok = lib().orc_pluecker(_p(_f32(a)), _p(_f32(b)), _p(_f32(c)), _p(_f32(o)), _p(_f32(d)), C.c_int32(mode),
                            _p(out))
    return (bool(ok), out)


def hit_normals(pos, idx, n_tri, rays, prim, mode=MODE_DEFECT):
    """Normal Ng of the Pluecker test of ray i against original triangle
    prim[i] ([n, 3] float32), as the reference stores it in BVHRayHit::hit_ng."""
    pos, idx, r = _f32(pos), _i32(idx), _rays8(rays)
    n = r.shape[1]
    ng = np.zeros((n, 3), np.float32)
    lib().orc_hit_normals(_p(pos), _p(idx), C.c_int64(n_tri), _p(r), C.c_int64(n), _p(_i32(prim)),
                          C.c_int32(mode), _p(ng))
    return ng


def hit_values64(pos, idx, n_tri, rays, prim):
    pos, idx, r = _f32(pos), _i32(idx), _rays8(rays)
    n = r.shape[1]
    tuv = np.zeros((n, 3), np.float64)
    ok = np.zeros(n, np.uint8)
    lib().orc_hit_values64(_p(pos), _p(idx), C.c_int64(n_tri), _p(r), C.c_int64(n), _p(_i32(prim)), _p(tuv),
                           _p(ok))
    return tuv, ok.astype(bool)


def hit_adjoint64(pos, idx, n_tri, n_vert, rays, prim, gt, gu, gv):
    pos, idx, r = _f32(pos), _i32(idx), _rays8(rays)
    n = r.shape[1]
    grad = np.zeros((n_vert, 3), np.float64)
    lib().orc_hit_adjoint64(_p(pos), _p(idx), C.c_int64(n_tri), C.c_int64(n_vert), _p(r), C.c_int64(n),
                            _p(_i32(prim)), _p(_f32(gt)), _p(_f32(gu)), _p(_f32(gv)), _p(grad))
    return grad


def _medium(m):
    return Medium(m.sigma_s, m.sigma_a, m.g, m.rr_threshold, m.majorant)


def volume_tr(rho, lo, hi, medium, rays, seed, want_ckpt=False):
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    T = np.zeros(n, np.float32)
    ck_t, ck_k, ck_c = np.zeros(n, np.float32), np.zeros(n, np.uint32), np.zeros(n, np.float32)
    m = _medium(medium)
    lib().orc_volume_tr(_p(rho), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r), C.c_int64(n),
                        C.c_uint64(seed), _p(T), _p(ck_t) if want_ckpt else None,
                        _p(ck_k) if want_ckpt else None, _p(ck_c) if want_ckpt else None)
    return (T, {"t": ck_t, "k": ck_k, "c": ck_c}) if want_ckpt else T


def volume_tr64(rho, lo, hi, medium, rays, seed, rho64=None):
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    T = np.zeros(n, np.float64)
    nrr = np.zeros(n, np.int32)
    m = _medium(medium)
    r64 = None if rho64 is None else np.ascontiguousarray(rho64, np.float64)
    lib().orc_volume_tr64(_p(rho), _p(r64), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r),
                          C.c_int64(n), C.c_uint64(seed), _p(T), _p(nrr))
    return T, nrr


def volume_tr64_sub(rho, lo, hi, medium, rays, ray_ids, seed, vox=-1, delta=0.0):
    """FP64 ratio tracking of a subset of rays (ray j draws from the stream of
    ray ray_ids[j]) with grid value `vox` (flat index) raised by `delta`.
    Returns (T, roulette counts)."""
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    ids = np.ascontiguousarray(ray_ids, np.int64)
    T = np.zeros(n, np.float64)
    nrr = np.zeros(n, np.int32)
    m = _medium(medium)
    lib().orc_volume_tr64_sub(_p(rho), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r), C.c_int64(n),
                              _p(ids), C.c_uint64(seed), C.c_int64(vox), C.c_double(delta), _p(T), _p(nrr))
    return T, nrr


def volume_tr_adjoint(rho, lo, hi, medium, rays, seed, dLdT):
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    grad = np.zeros(rho.shape, np.float64)
    m = _medium(medium)
    lib().orc_volume_tr_adjoint(_p(rho), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r), C.c_int64(n),
                                C.c_uint64(seed), _p(_f32(dLdT)), _p(grad))
    return grad


def volume_tr_adjoint_vox(rho, lo, hi, medium, rays, ray_ids, seed, vox):
    """Per-ray contributions (dL/dT = 1) to the gradient at one voxel (flat
    index) for a subset of rays keyed by ray_ids."""
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    ids = np.ascontiguousarray(ray_ids, np.int64)
    out = np.zeros(n, np.float64)
    m = _medium(medium)
    lib().orc_volume_tr_adjoint_vox(_p(rho), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r),
                                    C.c_int64(n), _p(ids), C.c_uint64(seed), C.c_int64(vox), _p(out))
    return out


def volume_sample(rho, lo, hi, medium, rays, seed):
    rho = _f32(rho)
    nz, ny, nx = rho.shape
    r = _rays8(rays)
    n = r.shape[1]
    ok = np.zeros(n, np.uint8)
    p = np.zeros((n, 3), np.float32)
    w = np.zeros(n, np.float32)
    m = _medium(medium)
    lib().orc_volume_sample(_p(rho), nx, ny, nz, _p(_f32(lo)), _p(_f32(hi)), C.byref(m), _p(r), C.c_int64(n),
                            C.c_uint64(seed), _p(ok), _p(p), _p(w))
    return ok, p, w


def majorant(rho):
    rho = _f32(rho)
    return float(lib().orc_grid_majorant(_p(rho), C.c_int64(rho.size)))


def set_threads(n: int) -> None:
    lib().orc_set_threads(C.c_int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def pathtrace(pos, idx, tree, light_first, light_count, le, albedo, eye, target, up, fov_deg, width, height,
              spp, max_depth, pixel_stride=1, grid=None, seed=0, mesh_medium=None):
    """CPU restatement of the path tracer; returns (radiance [h, w, 3], (closest, shadow) ray counts).
    With pixel_stride > 1 only every pixel_stride-th pixel is rendered.  grid = (rho [nz, ny, nx],
    lo, hi, Medium) adds the participating medium (volumetric path tracing).  mesh_medium =
    (first, count, sigma_s[3], sigma_a[3], g, density) adds a homogeneous medium bounded by
    triangles [first, first + count)."""
    pos, idx = _f32(pos), _i32(idx)
    out = np.zeros((height, width, 3), np.float32)
    rays = np.zeros(2, np.int64)
    f3 = lambda v: _f32(np.asarray(v, np.float32))
    args = [f3(le), f3(albedo), f3(eye), f3(target), f3(up)]
    if grid is not None:
        rho, glo, ghi, med = grid
        rho = _f32(rho)
        nz, ny, nx = rho.shape
        gargs = [_p(rho), C.c_int32(nx), C.c_int32(ny), C.c_int32(nz), _p(f3(glo)), _p(f3(ghi)), C.byref(med)]
    else:
        gargs = [None, C.c_int32(0), C.c_int32(0), C.c_int32(0), None, None, None]
    if mesh_medium is not None:
        first, count, ss, sa, g, dens = mesh_medium
        mt = np.array([first, count], np.int32)
        mc = np.array(list(ss) + list(sa) + [g, dens], np.float32)
        margs = [_p(mt), _p(mc)]
    else:
        margs = [None, None]
    lib().orc_pathtrace(_p(pos), _p(idx), C.c_int64(tree["n"]), _p(_i32(tree["perm"])), _p(_i32(tree["split"])),
                        _p(np.ascontiguousarray(tree["leaf_flags"], np.uint8)), _p(_f32(tree["bounds"])),
                        C.c_int32(light_first), C.c_int32(light_count), *[_p(a) for a in args], C.c_float(fov_deg),
                        C.c_int32(width), C.c_int32(height), C.c_int32(spp), C.c_int32(max_depth),
                        C.c_int32(pixel_stride), _p(out), _p(rays), *gargs, C.c_uint64(seed),
                        *margs)
    return out, (int(rays[0]), int(rays[1]))
