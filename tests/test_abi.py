"""CPU-side checks of the C ABI: libflg.so loads, exports every entry point
include/flg.h declares, and fails cleanly (no crash) when no GPU is present."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "flg.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"FLG_API\s+[\w\s\*]+?\b(flg_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import fledge_gb300._build as B
    B.build()
    import fledge_gb300._lib as L
    return L.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("flg_bvh_build", "flg_bvh_build_batched", "flg_trace_closest", "flg_trace_any",
              "flg_volume_tr", "flg_volume_tr_adjoint", "flg_volume_sample", "flg_hit_adjoint",
              "flg_graph_begin", "flg_bvh_download"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "fledge_gb300", "libflg.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(flg_\w+)\b", out))
    assert set(declared_symbols()) <= exported
    # nothing beyond the C ABI leaks out of the library
    assert all(s in set(declared_symbols()) for s in exported)


def test_python_binding_covers_header():
    import fledge_gb300._lib as L
    assert set(L.SIGNATURES) == set(declared_symbols())


def test_status_strings(lib):
    assert lib.flg_status_string(0) == b"ok"
    assert lib.flg_status_string(4) == b"device wait timed out"
    assert lib.flg_version().startswith(b"fledge-gb300")


def test_no_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = C.c_void_p()
    rc = lib.flg_ctx_create(0, None, C.byref(h))
    assert rc == 3 and not h.value  # FLG_ERR_CUDA, no handle


def test_null_arguments_rejected(lib):
    assert lib.flg_ctx_create(0, None, None) == 1
    assert lib.flg_bvh_build(None, None, None, 0, 0, None, None) == 1
    assert lib.flg_trace_closest(None, None, None, 0, None, None) == 1
    assert lib.flg_volume_tr(None, None, None, 0, 0, None, None) == 1
    assert lib.flg_bvh_destroy(None) == 0


def test_product_path_never_imports_oracle():
    """The library and its Python mirror do not reference the oracle."""
    for dirpath, _, files in os.walk(os.path.join(ROOT, "fledge_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.replace("Oracle", "").lower() or f == "_build.py", f


def test_builder_ids_match_header():
    """FLG_BUILDER_* in include/flg.h, the ctypes constants and the Python
    mirror's builder names agree; unknown names are rejected."""
    import fledge_gb300 as F
    import fledge_gb300._lib as L
    text = open(HEADER).read()
    enum = dict(re.findall(r"(FLG_BUILDER_\w+)\s*=\s*(\d+)", text))
    assert enum == {"FLG_BUILDER_LBVH": "0", "FLG_BUILDER_PLOC": "1", "FLG_BUILDER_SAH": "2",
                    "FLG_BUILDER_TREELET": "3"}
    for k, v in enum.items():
        assert getattr(L, k) == int(v)
    assert [F._builder_id(n) for n in ("lbvh", "ploc", "sah", "treelet")] == [0, 1, 2, 3]
    with pytest.raises(ValueError):
        F._builder_id("median")


def test_build_opts_layout_and_tuner_candidates():
    """flg_build_opts in include/flg.h and its ctypes mirror list the same
    fields in the same order (treelet_rounds last); the tuner's candidate
    names map to builder arguments ('treelet<r>': r restructuring rounds)."""
    import fledge_gb300._lib as L
    from fledge_gb300 import autotune as A
    text = open(HEADER).read()
    body = re.search(r"typedef struct flg_build_opts \{(.*?)\} flg_build_opts;", text, re.S).group(1)
    fields = re.findall(r"int32_t\s+(\w+);", body)
    assert fields == [f for f, _ in L.FlgBuildOpts._fields_]
    assert fields[-1] == "treelet_rounds"
    assert A.builder_args("treelet1") == {"builder": "treelet", "treelet_rounds": 1}
    assert A.builder_args("treelet") == {"builder": "treelet"}
    assert A.builder_args("lbvh") == {"builder": "lbvh"}
    assert all(A.builder_args(b)["builder"] in ("lbvh", "ploc", "sah", "treelet") for b in A.BUILDERS)
