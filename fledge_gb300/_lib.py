"""ctypes binding of libflg.so (the C ABI declared in include/flg.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback behind these entry points.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflg.so")

FLG_OK, FLG_ERR_ARG, FLG_ERR_OOM, FLG_ERR_CUDA, FLG_ERR_TIMEOUT, FLG_ERR_STACK, FLG_ERR_STATE, \
    FLG_ERR_UNSUPPORTED = range(8)


class FlgRays(C.Structure):
    _fields_ = [("ox", C.c_void_p), ("oy", C.c_void_p), ("oz", C.c_void_p),
                ("dx", C.c_void_p), ("dy", C.c_void_p), ("dz", C.c_void_p),
                ("tmin", C.c_void_p), ("tmax", C.c_void_p),
                ("tmin_const", C.c_float), ("tmax_const", C.c_float)]


class FlgHits(C.Structure):
    _fields_ = [("prim", C.c_void_p), ("t", C.c_void_p), ("u", C.c_void_p), ("v", C.c_void_p)]


class FlgBuildOpts(C.Structure):
    _fields_ = [("node_width", C.c_int32), ("leaf_size", C.c_int32), ("keep_topology", C.c_int32),
                ("builder", C.c_int32), ("treelet_rounds", C.c_int32)]


FLG_BUILDER_LBVH, FLG_BUILDER_PLOC, FLG_BUILDER_SAH, FLG_BUILDER_TREELET = 0, 1, 2, 3


class FlgTraceOpts(C.Structure):
    _fields_ = [("stack_depth", C.c_int32), ("block_threads", C.c_int32), ("persistent", C.c_int32),
                ("refill_lanes", C.c_int32), ("ray_sort", C.c_int32), ("tri_test", C.c_int32)]


class FlgBvhInfo(C.Structure):
    _fields_ = [("n_tri", C.c_int64), ("n_scenes", C.c_int32), ("node_width", C.c_int32),
                ("n_wide_nodes", C.c_int64), ("device_bytes", C.c_int64), ("bound", C.c_float * 6)]


class FlgBvhTopology(C.Structure):
    _fields_ = [("morton", C.c_void_p), ("perm", C.c_void_p), ("split", C.c_void_p),
                ("leaf_flags", C.c_void_p), ("range_j", C.c_void_p), ("parent", C.c_void_p),
                ("leaf_parent", C.c_void_p), ("bounds", C.c_void_p), ("scene_bound", C.c_void_p)]


class FlgMedium(C.Structure):
    _fields_ = [("sigma_s", C.c_float), ("sigma_a", C.c_float), ("g", C.c_float),
                ("rr_threshold", C.c_float), ("majorant", C.c_float)]


class FlgTrCkpt(C.Structure):
    _fields_ = [("t", C.c_void_p), ("k", C.c_void_p), ("c", C.c_void_p)]


class FlgHostMesh(C.Structure):
    _fields_ = [("pos", C.POINTER(C.c_float)), ("normal", C.POINTER(C.c_float)), ("uv", C.POINTER(C.c_float)),
                ("idx", C.POINTER(C.c_int32)), ("n_vert", C.c_int64), ("n_tri", C.c_int64)]


class FlgPtScene(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("idx", C.c_void_p), ("n_tri", C.c_int64), ("n_vert", C.c_int64),
                ("light_first", C.c_int32), ("light_count", C.c_int32), ("light_le", C.c_float * 3),
                ("albedo", C.c_float * 3)]


class FlgPtCamera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("fov_deg", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32)]


class FlgMeshMedium(C.Structure):
    _fields_ = [("first", C.c_int32), ("count", C.c_int32), ("sigma_s", C.c_float * 3), ("sigma_a", C.c_float * 3),
                ("g", C.c_float), ("density", C.c_float)]


class FlgPtStats(C.Structure):
    _fields_ = [("closest_rays", C.c_int64), ("shadow_rays", C.c_int64)]


P = C.c_void_p
I32, I64, U32, U64, F32 = C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float
PP = C.POINTER(C.c_void_p)

# name -> argtypes (restype is int unless listed in _RESTYPE)
SIGNATURES = {
    "flg_ctx_create": [I32, P, PP],
    "flg_ctx_destroy": [P],
    "flg_ctx_sync": [P],
    "flg_ctx_stream": [P],
    "flg_ctx_launch_count": [P],
    "flg_ctx_set_spin_limit": [P, U32],
    "flg_ctx_set_stage_timing": [P, I32],
    "flg_ctx_stage_times": [P, C.c_char_p, C.c_size_t],
    "flg_status_string": [C.c_int],
    "flg_debug_wait_unset_flag": [P, U32],
    "flg_ctx_last_error": [P, C.c_char_p, C.c_size_t],
    "flg_bvh_build": [P, P, P, I64, I64, C.POINTER(FlgBuildOpts), PP],
    "flg_bvh_build_batched": [P, P, P, C.POINTER(I64), I32, I64, C.POINTER(FlgBuildOpts), PP],
    "flg_bvh_rebuild": [P, P, P],
    "flg_bvh_destroy": [P],
    "flg_bvh_info_get": [P, C.POINTER(FlgBvhInfo)],
    "flg_bvh_download": [P, I32, C.POINTER(FlgBvhTopology)],
    "flg_trace_closest": [P, P, C.POINTER(FlgRays), I64, C.POINTER(FlgTraceOpts), C.POINTER(FlgHits)],
    "flg_trace_any": [P, P, C.POINTER(FlgRays), I64, C.POINTER(FlgTraceOpts), P],
    "flg_trace_closest_batched": [P, P, C.POINTER(FlgRays), C.POINTER(I64), C.POINTER(FlgTraceOpts),
                                  C.POINTER(FlgHits)],
    "flg_trace_closest_host": [P, P, C.POINTER(FlgRays), I64, C.POINTER(FlgTraceOpts), C.POINTER(FlgHits)],
    "flg_trace_closest_noalloc": [P, P, C.POINTER(FlgRays), I64, C.POINTER(FlgHits)],
    "flg_autotune_trace": [P, P, C.POINTER(FlgRays), I64, C.POINTER(FlgTraceOpts), C.POINTER(I32),
                           C.c_char_p, C.c_size_t],
    "flg_autotune_trace_batched": [P, P, C.POINTER(FlgRays), C.POINTER(I64), I32, C.POINTER(FlgTraceOpts),
                                   C.POINTER(I32), C.POINTER(I32), C.c_char_p, C.c_size_t],
    "flg_bvh_set_width": [P, P, I32, I32],
    "flg_hit_adjoint": [P, P, P, I64, I64, C.POINTER(FlgRays), I64, C.POINTER(FlgHits), P, P, P, P],
    "flg_hit_normals": [P, P, C.POINTER(FlgRays), I64, P, I32, P],
    "flg_grid_create": [P, P, I32, I32, I32, C.POINTER(F32), C.POINTER(F32), C.POINTER(FlgMedium), PP],
    "flg_grid_destroy": [P],
    "flg_grid_majorant": [P, C.POINTER(F32)],
    "flg_volume_tr": [P, P, C.POINTER(FlgRays), I64, U64, P, C.POINTER(FlgTrCkpt)],
    "flg_volume_tr_adjoint": [P, P, C.POINTER(FlgRays), I64, U64, P, P, C.POINTER(FlgTrCkpt), P],
    "flg_volume_sample": [P, P, C.POINTER(FlgRays), I64, U64, P, P, P],
    "flg_pathtrace": [P, P, C.POINTER(FlgPtScene), C.POINTER(FlgPtCamera), I32, I32, C.POINTER(FlgTraceOpts), P,
                      C.POINTER(FlgPtStats)],
    "flg_volpath": [P, P, P, C.c_uint64, C.POINTER(FlgPtScene), C.POINTER(FlgPtCamera), I32, I32,
                    C.POINTER(FlgTraceOpts), P, C.POINTER(FlgPtStats)],
    "flg_volpath_mesh": [P, P, C.POINTER(FlgMeshMedium), C.c_uint64, C.POINTER(FlgPtScene), C.POINTER(FlgPtCamera),
                         I32, I32, C.POINTER(FlgTraceOpts), P, C.POINTER(FlgPtStats)],
    "flg_graph_begin": [P],
    "flg_graph_end": [P, PP],
    "flg_graph_launch": [P, P],
    "flg_graph_destroy": [P],
    "flg_gen_triangles": [P, U64, I64, I64, F32, P],
    "flg_gen_rays": [P, U64, I64, I64, C.POINTER(F32), F32, P, P, P, P, P, P],
    "flg_gen_noise_grid": [P, U64, I32, I32, I32, F32, P],
    "flg_version": [],
    "flg_ply_read": [C.c_char_p, C.POINTER(FlgHostMesh), C.c_char_p, C.c_size_t],
    "flg_grid_create_sparse": [P, P, P, I64, I32, I32, I32, C.POINTER(F32), C.POINTER(F32), C.POINTER(FlgMedium), PP],
    "flg_grid_sparsify": [P, P, I32, I32, I32, P, P, I64, C.POINTER(I64)],
    "flg_host_mesh_free": [C.POINTER(FlgHostMesh)],
}
_RESTYPE = {"flg_status_string": C.c_char_p, "flg_version": C.c_char_p, "flg_ctx_stream": C.c_void_p,
            "flg_ctx_launch_count": C.c_int64, "flg_host_mesh_free": None}

_lib = None


def load() -> C.CDLL:
    """Loads libflg.so; raises if it is missing (build with fledge_gb300._build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m fledge_gb300._build` "
                           "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, C.c_int)
    _lib = lib
    return lib


class FlgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"flg status {code}: {msg}")
        self.code = code


def check(code: int, ctx=None) -> None:
    if code != FLG_OK:
        lib = load()
        msg = lib.flg_status_string(code).decode()
        if ctx is not None:
            buf = C.create_string_buffer(512)
            lib.flg_ctx_last_error(ctx, buf, 512)
            if buf.value:
                msg += f" ({buf.value.decode()})"
        raise FlgError(code, msg)
