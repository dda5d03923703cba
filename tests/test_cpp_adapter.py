"""The C++ adapter header (include/flg_accel.hpp) compiles against the C ABI,
links with libflg.so, binds to the reference's own Ray / SInteraction /
VInteraction / Sampler types, and (on the GPU) returns the oracle's results:

  * BVHRayHit adapter (RadixBVHBuilder::intersect): prim ids equal to the
    oracle except recorded exact ties, t/u/v bit-equal where ids agree,
    hit_ng = hit_ns = the Pluecker normal of the oracle (Euclidean norm);
  * GpuLBVH (Accel / Primitive::intersect, live renderer): hits and m_tMax of
    the oracle's Moller-Trumbore restatement, misses untouched, m_p, m_wo,
    m_ng and interpolated m_ns as the reference's arithmetic gives them;
  * DenseGridVolume::tr / sample through host rays and through a Sampler
    (stream key from two get1D draws): bit-equal to the oracle's tracking.
"""
import os
import subprocess

import numpy as np
import pytest

import geometry as G
import gpu_util as U

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
CUDA = "/usr/local/cuda"
REF_SRC = os.environ.get("FLG_REFERENCE_SRC", "/root/reference/src")


def _compile(tmp_path, name):
    from fledge_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", os.path.join(CPP, name + ".cpp"),
           "-I" + os.path.join(ROOT, "include"), "-I" + CUDA + "/include", lib, "-L" + CUDA + "/lib64", "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib), "-Wl,-rpath," + CUDA + "/lib64", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name", ["flg_accel_example", "live_renderer_example"])
def test_adapter_compiles_and_links(tmp_path, name):
    assert os.path.exists(_compile(tmp_path, name))


def test_adapter_binds_reference_types():
    """Instantiates the adapters with the reference's fledge::Ray,
    SInteraction, VInteraction, Sampler and Vector3f (compile only)."""
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources not present")
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-w", "-I" + os.path.join(ROOT, "oracle", "refshim"),
           "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"), "-I" + CUDA + "/include",
           os.path.join(CPP, "reference_types_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_bvhrayhit_adapter_matches_oracle(tmp_path, oracle):
    exe = _compile(tmp_path, "flg_accel_example")
    n_tri, n = 20000, 30000
    pos = G.random_soup(n_tri, np.random.default_rng(5), half=0.02)
    r8 = G.sphere_rays(n, np.random.default_rng(6))
    tf, rf, of = tmp_path / "t.bin", tmp_path / "r.bin", tmp_path / "o.bin"
    with open(tf, "wb") as f:
        f.write(np.int64(n_tri).tobytes() + pos.astype(np.float32).tobytes())
    with open(rf, "wb") as f:
        f.write(np.int64(n).tobytes() + r8.astype(np.float32).tobytes())
    r = subprocess.run([exe, str(tf), str(rf), str(of)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(of, dtype=np.uint8)
    prim = raw[:4 * n].view(np.int32)
    tuv = raw[4 * n:16 * n].view(np.float32).reshape(3, n)
    ng = raw[16 * n:].view(np.float32).reshape(n, 3)
    hg = {"prim": prim, "t": tuv[0], "u": tuv[1], "v": tuv[2]}
    tree = oracle.build_bvh(pos)
    bad, ties, ho = U.compare_closest(oracle, pos, None, tree, r8, hg, oracle.MODE_DEV)
    assert bad == 0, f"{bad} prim mismatches ({ties} exact ties)"
    same = prim == ho["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(hg[k][same], ho[k][same]), k
    want = oracle.hit_normals(pos, None, n_tri, r8, prim, oracle.MODE_REF)
    assert np.array_equal(ng, want)
    hit = prim >= 0
    assert hit.mean() > 0.3 and np.allclose(np.linalg.norm(ng[hit], axis=1), 1.0, atol=1e-6)
    assert np.all(ng[~hit] == 0)


def _geometric_normal(tri):
    """normalize(cross(p1 - p0, p2 - p0)) in fp32 with the reference's order."""
    e1, e2 = (tri[:, 1] - tri[:, 0]).astype(np.float32), (tri[:, 2] - tri[:, 0]).astype(np.float32)
    c = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1).astype(np.float32)
    s = np.sqrt((c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2]).astype(np.float32)
    return (c / s[:, None]).astype(np.float32)


@pytest.mark.gpu
def test_live_renderer_adapters_match_oracle(tmp_path, oracle):
    exe = _compile(tmp_path, "live_renderer_example")
    v, ind = G.meshed_sphere(96, 96, 1.0)
    nrm = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    n = 40000
    r8 = G.interior_rays(n, np.random.default_rng(21))
    ext = G.sphere_rays(n, np.random.default_rng(22), center=(0.0, 0.0, 0.0), radius=2.0)
    r8[:, n // 2:] = ext[:, n // 2:]  # half from inside, half from outside
    tmax = np.where(np.arange(n) % 3 == 0, np.float32(1.2), np.float32(np.finfo(np.float32).max))
    r8[6], r8[7] = 0.0, tmax
    mf, rf, gf, of = (tmp_path / x for x in ("m.bin", "r.bin", "g.bin", "o.bin"))
    with open(mf, "wb") as f:
        f.write(np.array([v.shape[0], ind.shape[0], 1], np.int64).tobytes() + v.tobytes() + ind.tobytes() +
                nrm.tobytes())
    with open(rf, "wb") as f:
        f.write(np.int64(n).tobytes() + np.concatenate([r8[:6], r8[7:8]]).astype(np.float32).tobytes())
    rho = G.value_noise_grid(32, np.random.default_rng(23))
    with open(gf, "wb") as f:
        f.write(np.int32(32).tobytes() + rho.tobytes())
    r = subprocess.run([exe, str(mf), str(rf), str(gf), str(of)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    raw = open(of, "rb").read()
    o = 0
    hit = np.frombuffer(raw, np.uint8, n, o).astype(bool)
    o += n
    tm = np.frombuffer(raw, np.float32, n, o)
    o += 4 * n
    it = np.frombuffer(raw, np.float32, 12 * n, o).reshape(n, 4, 3)
    o += 48 * n
    # Accel: the oracle's Moller-Trumbore closest hit (0 < t < tMax, refined t/u/v)
    tree = oracle.build_bvh(v, ind)
    ho = oracle.trace_closest(v, ind, tree, r8, oracle.MODE_MT)
    hp = ho["prim"]
    assert np.array_equal(hit, hp >= 0)
    assert np.array_equal(tm[hit], ho["t"][hit]) and np.array_equal(tm[~hit], r8[7][~hit])
    assert np.all(it[~hit] == 0)
    o_, d_ = r8[0:3].T, r8[3:6].T
    t = ho["t"][:, None]
    assert np.array_equal(it[hit, 0], (o_ + d_ * t).astype(np.float32)[hit])  # m_p = ray(t)
    tri = v[ind[hp[hit]]]
    assert np.array_equal(it[hit, 1], _geometric_normal(tri))  # m_ng
    u, w = ho["u"][hit][:, None], ho["v"][hit][:, None]
    n0, n1, n2 = nrm[ind[hp[hit], 0]], nrm[ind[hp[hit], 1]], nrm[ind[hp[hit], 2]]
    ns = (u * n0 + w * n1) + (np.float32(1.0) - u - w) * n2
    assert np.array_equal(it[hit, 2], ns.astype(np.float32))  # m_ns with the reference's weights
    assert np.array_equal(it[hit, 3], -d_[hit])  # m_wo
    assert 0.3 < hit.mean() < 0.99
    # Volume: batched host rays on streams (11, i)
    class Med:
        sigma_s, sigma_a, g, rr_threshold, majorant = 0.8, 0.2, 0.3, 0.1, 0.0
    T = np.frombuffer(raw, np.float32, n, o)
    o += 4 * n
    assert np.array_equal(T, oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], Med, r8, 11))
    m = 256
    rec = np.dtype([("key", "<u8"), ("T", "<f4"), ("key2", "<u8"), ("ok", "u1"), ("p", "<f4", 3), ("w", "<f4")])
    recs = np.frombuffer(raw, rec, m, o)
    for i in range(m):
        one = r8[:, i:i + 1]
        assert recs["T"][i] == oracle.volume_tr(rho, [0, 0, 0], [1, 1, 1], Med, one, int(recs["key"][i]))[0]
        ok, p, wgt = oracle.volume_sample(rho, [0, 0, 0], [1, 1, 1], Med, one, int(recs["key2"][i]))
        assert bool(recs["ok"][i]) == bool(ok[0]) and recs["w"][i] == wgt[0]
        if ok[0]:
            assert np.array_equal(recs["p"][i], p[0])
    assert 0.05 < recs["ok"].mean() < 0.95
