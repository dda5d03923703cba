"""ctypes wrapper of oracle/_ref/libfledge_ref.so: the reference's own Karras
LBVH (RadixBVHBuilder, src/experimental/radix_bvh.cpp of the fledge project)
and live-renderer triangle test (Triangle::intersect, src/shape.cpp:100-148),
compiled unchanged by `make -C oracle ref`.

TEST INFRASTRUCTURE ONLY: a second checker that pins the oracle to the
reference's code.  The library exists only where the reference sources were
present at build time; `available()` says whether it was built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libfledge_ref.so")
REF_SRC = os.environ.get("FLG_REFERENCE_SRC", "/root/reference/src")

_lib = None


def build() -> bool:
    """Compiles the library when the reference sources are present; returns
    whether the library exists afterwards."""
    if os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"], check=True)
    return os.path.exists(LIB)


def available() -> bool:
    return os.path.exists(LIB)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB)
        _lib.ref_radix_build.restype = C.c_void_p
        _lib.ref_radix_build.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]
        _lib.ref_radix_arrays.restype = None
        _lib.ref_radix_arrays.argtypes = [C.c_void_p] + [C.c_void_p] * 10
        _lib.ref_radix_intersect.restype = None
        _lib.ref_radix_intersect.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                             C.c_void_p]
        _lib.ref_radix_destroy.restype = None
        _lib.ref_radix_destroy.argtypes = [C.c_void_p]
        _lib.ref_triangle_intersect.restype = None
        _lib.ref_triangle_intersect.argtypes = [C.c_void_p] * 2 + [C.c_int64] + [C.c_void_p] * 3
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class RadixBVH:
    """RadixBVHBuilder over a mesh: pos [n_vert, 3] float32, ind [n_tri, 3]
    int32 or None (soup).  Builds on construction."""

    def __init__(self, pos, ind=None):
        self.pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        self.ind = None if ind is None else np.ascontiguousarray(ind, np.int32).reshape(-1, 3)
        self.n = self.ind.shape[0] if self.ind is not None else self.pos.shape[0] // 3
        if self.n < 2:
            raise ValueError("the reference LBVH needs at least two triangles")
        self.h = lib().ref_radix_build(_ptr(self.pos), self.pos.shape[0], _ptr(self.ind), self.n)

    def arrays(self) -> dict:
        n, m = self.n, self.n - 1
        out = {"morton": np.zeros(n, np.uint32), "perm": np.zeros(n, np.int32),
               "leaf_parent": np.zeros(n, np.int32), "split": np.zeros(m, np.int32),
               "leaf_flags": np.zeros(m, np.uint8), "n_triangles": np.zeros(m, np.int32),
               "direction": np.zeros(m, np.int32), "parent": np.zeros(m, np.int32),
               "bounds": np.zeros((m, 6), np.float32), "scene_bound": np.zeros(6, np.float32)}
        lib().ref_radix_arrays(self.h, *[_ptr(out[k]) for k in (
            "morton", "perm", "leaf_parent", "split", "leaf_flags", "n_triangles", "direction", "parent",
            "bounds", "scene_bound")])
        return out

    def intersect(self, rays8) -> dict:
        """rays8: [8, n] float32 (ox oy oz dx dy dz tnear tfar).  Returns hit
        (bool), tfar and ng [n, 3] as RadixBVHBuilder::intersect leaves them."""
        r = np.ascontiguousarray(rays8, np.float32)
        n = r.shape[1]
        hit = np.zeros(n, np.uint8)
        tfar = np.zeros(n, np.float32)
        ng = np.zeros((n, 3), np.float32)
        lib().ref_radix_intersect(self.h, _ptr(r), n, _ptr(hit), _ptr(tfar), _ptr(ng))
        return {"hit": hit.astype(bool), "tfar": tfar, "ng": ng}

    def close(self) -> None:
        if self.h:
            lib().ref_radix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def triangle_intersect(tri, rays8) -> dict:
    """Triangle::intersect of the live renderer for n (triangle, ray) pairs:
    tri [n, 3, 3] float32, rays8 [8, n] (row 7 = tMax).  Returns hit (bool),
    t and ng [n, 3] (zeros where missed)."""
    tri = np.ascontiguousarray(tri, np.float32)
    r = np.ascontiguousarray(rays8, np.float32)
    n = r.shape[1]
    hit = np.zeros(n, np.uint8)
    t = np.zeros(n, np.float32)
    ng = np.zeros((n, 3), np.float32)
    lib().ref_triangle_intersect(_ptr(tri), _ptr(r), n, _ptr(hit), _ptr(t), _ptr(ng))
    return {"hit": hit.astype(bool), "t": t, "ng": ng}
