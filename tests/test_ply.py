"""PLY ingestion (flg_ply_read, the MakeTriangleMesh of plymesh.cpp:19-86):
ASCII and binary files of both byte orders, optional normals and texture
coordinates, extra elements and properties, polygon faces, and malformed
input.  Host code only: runs without a GPU."""
import struct

import numpy as np
import pytest

import fledge_gb300 as F
from fledge_gb300.scenes import icosphere


def _write_ply(path, fmt, pos, faces, normal=None, uv=None, extra=True, index_type="int", count_type="uchar"):
    n = len(pos)
    hdr = ["ply", f"format {fmt} 1.0", "comment written by the test", f"element vertex {n}",
           "property float x", "property float y", "property float z"]
    if normal is not None:
        hdr += ["property float nx", "property float ny", "property float nz"]
    if uv is not None:
        hdr += ["property float u", "property float v"]
    hdr += ["property uchar red"]  # an ignored property
    if extra:
        hdr += ["element material 1", "property float shininess"]
    hdr += [f"element face {len(faces)}", f"property list {count_type} {index_type} vertex_indices",
            "property int flags"]
    if extra:
        hdr += ["element edge 1", "property int vertex1", "property int vertex2"]
    hdr += ["end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(hdr) + "\n").encode())
        if fmt == "ascii":
            for i in range(n):
                row = list(pos[i]) + (list(normal[i]) if normal is not None else []) + \
                    (list(uv[i]) if uv is not None else [])
                f.write((" ".join(repr(float(x)) for x in row) + " 7\n").encode())
            if extra:
                f.write(b"0.5\n")
            for fc in faces:
                f.write((f"{len(fc)} " + " ".join(str(int(x)) for x in fc) + " 0\n").encode())
            if extra:
                f.write(b"0 1\n")
        else:
            e = "<" if fmt == "binary_little_endian" else ">"
            it = {"int": "i", "uint": "I", "short": "h", "ushort": "H"}[index_type]
            ct = {"uchar": "B", "int": "i", "ushort": "H"}[count_type]
            for i in range(n):
                row = list(pos[i]) + (list(normal[i]) if normal is not None else []) + \
                    (list(uv[i]) if uv is not None else [])
                f.write(struct.pack(e + "f" * len(row) + "B", *row, 7))
            if extra:
                f.write(struct.pack(e + "f", 0.5))
            for fc in faces:
                f.write(struct.pack(e + ct + it * len(fc) + "i", len(fc), *[int(x) for x in fc], 0))
            if extra:
                f.write(struct.pack(e + "ii", 0, 1))


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
def test_ply_roundtrip_icosphere(tmp_path, fmt):
    v, f = icosphere(2)
    rng = np.random.default_rng(5)
    nrm = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    uv = rng.random((len(v), 2)).astype(np.float32)
    p = tmp_path / "m.ply"
    _write_ply(p, fmt, v, f, nrm, uv)
    m = F.read_ply(str(p))
    assert m["pos"].shape == v.shape and m["idx"].shape == f.shape
    assert np.array_equal(m["pos"], v) and np.array_equal(m["idx"], f)
    assert np.array_equal(m["normal"], nrm) and np.array_equal(m["uv"], uv)


@pytest.mark.parametrize("index_type,count_type", [("uint", "uchar"), ("short", "int"), ("ushort", "ushort")])
def test_ply_types_and_polygons(tmp_path, index_type, count_type):
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.5, 2, 0]], np.float32)
    faces = [[0, 1, 2, 3], [3, 2, 4], [0, 1]]  # a quad, a triangle, a degenerate 2-gon
    p = tmp_path / "poly.ply"
    _write_ply(p, "binary_little_endian", pos, faces, index_type=index_type, count_type=count_type)
    m = F.read_ply(str(p))
    assert m["normal"] is None and m["uv"] is None
    # the quad is fan-triangulated, the 2-gon dropped
    assert m["idx"].tolist() == [[0, 1, 2], [0, 2, 3], [3, 2, 4]]
    assert np.array_equal(m["pos"], pos)


def test_ply_errors(tmp_path):
    with pytest.raises(F.FlgError, match="cannot open"):
        F.read_ply(str(tmp_path / "missing.ply"))
    bad = tmp_path / "bad.ply"
    bad.write_bytes(b"not a ply\n")
    with pytest.raises(F.FlgError, match="not a PLY"):
        F.read_ply(str(bad))
    oob = tmp_path / "oob.ply"
    _write_ply(oob, "ascii", np.zeros((3, 3), np.float32), [[0, 1, 5]], extra=False)
    with pytest.raises(F.FlgError, match="vertex 5"):
        F.read_ply(str(oob))
    trunc = tmp_path / "trunc.ply"
    _write_ply(trunc, "binary_little_endian", np.zeros((3, 3), np.float32), [[0, 1, 2]], extra=False)
    trunc.write_bytes(trunc.read_bytes()[:-6])
    with pytest.raises(F.FlgError, match="end of file"):
        F.read_ply(str(trunc))
    nofaces = tmp_path / "nofaces.ply"
    nofaces.write_bytes(b"ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nproperty float y\n"
                        b"property float z\nend_header\n0 0 0\n")
    with pytest.raises(F.FlgError, match="no vertex or no face"):
        F.read_ply(str(nofaces))
