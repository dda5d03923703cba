"""Seeded synthetic scenes for the path-tracing workload (host-side input
generation, numpy).

* ``icosphere``: an icosahedron subdivided `level` times (20 * 4^level
  triangles) on a sphere of radius `radius`, each vertex displaced radially
  by ``amplitude * noise(p)`` with 4-octave value noise.
* ``quad_light``: the 0.2 x 0.2 emitter at y = 2 facing -y, as 2 triangles.
"""
from __future__ import annotations

import numpy as np

_PHI = (1.0 + 5.0 ** 0.5) / 2.0
_ICO_V = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                   [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                   [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], np.float64)
_ICO_F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                   [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                   [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)


def _subdivide(v: np.ndarray, f: np.ndarray):
    """One 1:4 split; shared edge midpoints are created once."""
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
    e.sort(axis=1)
    key = e[:, 0] * (len(v) + 1) + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a, b = uniq // (len(v) + 1), uniq % (len(v) + 1)
    mid = v[a] + v[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    m = inv.reshape(3, -1).T + len(v)  # midpoint index of edges (01, 12, 20)
    v2 = np.concatenate([v, mid], 0)
    f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
    m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
    f2n = np.concatenate([np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
                          np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)], 0)
    return v2, f2n


def _hash01(ix, iy, iz, o, seed):
    """Lattice value in [-1, 1] from a 64-bit integer mix (splitmix64)."""
    x = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
         ^ iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)
         ^ iz.astype(np.uint64) * np.uint64(0x165667B19E3779F9)
         ^ np.uint64(o) * np.uint64(0x27D4EB2F165667C5) ^ np.uint64(seed))
    x ^= x >> np.uint64(30)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(27)
    x *= np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    return (x >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def value_noise(p: np.ndarray, seed: int, octaves: int = 4, base_freq: float = 2.0) -> np.ndarray:
    """Sum of octaves of smoothstep-trilinear lattice noise, frequencies
    base * 2^o, amplitudes 2^-o, normalised to [-1, 1]."""
    acc = np.zeros(len(p))
    norm = 0.0
    for o in range(octaves):
        q = p * (base_freq * 2 ** o) + 1024.0
        i = np.floor(q).astype(np.int64)
        f = q - i
        f = f * f * (3 - 2 * f)
        v = np.zeros(len(p))
        for c in range(8):
            cx, cy, cz = c & 1, (c >> 1) & 1, c >> 2
            w = (f[:, 0] if cx else 1 - f[:, 0]) * (f[:, 1] if cy else 1 - f[:, 1]) * (f[:, 2] if cz else 1 - f[:, 2])
            v += w * _hash01(i[:, 0] + cx, i[:, 1] + cy, i[:, 2] + cz, o, seed)
        acc += 2.0 ** -o * v
        norm += 2.0 ** -o
    return acc / norm


def icosphere(level: int = 8, radius: float = 1.0, amplitude: float = 0.05, seed: int = 0xF1ED0001):
    """(vertices float32 [nv, 3], indices int32 [nt, 3])."""
    v = _ICO_V / np.linalg.norm(_ICO_V, axis=1, keepdims=True)
    f = _ICO_F
    for _ in range(level):
        v, f = _subdivide(v, f)
    r = radius * (1.0 + amplitude * value_noise(v, seed))
    return (v * r[:, None]).astype(np.float32), f.astype(np.int32)


def quad_light(y: float = 2.0, half: float = 0.1):
    """Two triangles of the square emitter at height y, normal -y."""
    v = np.array([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]], np.float32)
    # winding so that (p1-p0) x (p2-p0) points down (-y)
    f = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    return v, f
