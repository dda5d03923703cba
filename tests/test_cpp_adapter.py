"""The C++ adapter header (include/flg_accel.hpp) compiles against the C ABI,
links with libflg.so, and (on the GPU) returns the oracle's hits."""
import os
import subprocess

import numpy as np
import pytest

import geometry as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "flg_accel_example.cpp")


def _compile(tmp_path):
    from fledge_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path / "flg_accel_example")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-std=c++17", "-O2", SRC, "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
           lib, "-L" + cuda + "/lib64", "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
           "-Wl,-rpath," + cuda + "/lib64", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_compiles_and_links(tmp_path):
    exe = _compile(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_adapter_traces_like_oracle(tmp_path, oracle):
    exe = _compile(tmp_path)
    pos = G.random_soup(20000, np.random.default_rng(5), half=0.02)
    r8 = G.sphere_rays(30000, np.random.default_rng(6))
    tf, rf, of = tmp_path / "t.bin", tmp_path / "r.bin", tmp_path / "o.bin"
    with open(tf, "wb") as f:
        f.write(np.int64(20000).tobytes() + pos.astype(np.float32).tobytes())
    with open(rf, "wb") as f:
        f.write(np.int64(30000).tobytes() + r8.astype(np.float32).tobytes())
    r = subprocess.run([exe, str(tf), str(rf), str(of)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(of, dtype=np.uint8)
    prim = raw[:4 * 30000].view(np.int32)
    tuv = raw[4 * 30000:].view(np.float32).reshape(3, 30000)
    tree = oracle.build_bvh(pos)
    ho = oracle.trace_closest(pos, None, tree, r8, oracle.MODE_DEV)
    same = prim == ho["prim"]
    assert same.mean() > 0.9999
    assert np.array_equal(tuv[0][same & (prim >= 0)], ho["t"][same & (prim >= 0)])
