"""Seeded synthetic workloads (host-side input generation).

* ``icosphere``: an icosahedron subdivided `level` times (20 * 4^level
  triangles) on a sphere of radius `radius`, each vertex displaced radially
  by ``amplitude * noise(p)`` with 4-octave value noise.
* ``quad_light``: the 0.2 x 0.2 emitter at y = 2 facing -y, as 2 triangles.
* ``path_tracing_scene`` / ``PATH_TRACING_CAMERA``: the level-8 icosphere
  (1,310,720 triangles) under the light, and its 1920x1080 camera.
* ``batched_scene_counts``: triangle counts of the 256-scene batch,
  round(exp(U[ln 1e3, ln 1e6])).
* ``camera_rays_4k``: the 3840x2160x4 jittered pinhole rays of the
  8 M-triangle scene (device tensors).

Seeds are 0xF1ED0000 + k for workload k (0: random soup, 1: path tracing,
2: volume, 3: batched scenes).
"""
from __future__ import annotations

import math

import numpy as np

SEED_SOUP, SEED_PATH, SEED_VOLUME, SEED_BATCH = 0xF1ED0000, 0xF1ED0001, 0xF1ED0002, 0xF1ED0003
N_SCENES = 256
RAYS_PER_TRI = 64

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


def path_tracing_scene(level: int = 8):
    """(positions, indices, first light triangle): the displaced icosphere
    followed by the two light triangles."""
    v, f = icosphere(level)
    lv, lf = quad_light()
    return np.concatenate([v, lv], 0), np.concatenate([f, lf + len(v)], 0), len(f)


PATH_TRACING_CAMERA = dict(eye=(0.0, 0.6, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=40.0)


def batched_scene_counts(n_scenes: int = N_SCENES, seed: int = SEED_BATCH) -> np.ndarray:
    """Triangle counts of the batched workload, log-uniform in [1e3, 1e6]."""
    rng = np.random.default_rng(seed)
    c = np.round(np.exp(rng.uniform(math.log(1e3), math.log(1e6), N_SCENES))).astype(np.int64)
    return c[:n_scenes]


def camera_rays_4k(torch, device, seed: int = SEED_BATCH + 41, width: int = 3840, height: int = 2160,
                   spp: int = 4):
    """Jittered pinhole camera rays (6 x n device tensor, SoA ox..dz) from
    (0.5, 0.5, -1.5) looking along +z with a 45 degree vertical field of
    view, spp samples per pixel in pixel-major order."""
    n = width * height * spp
    g = torch.Generator(device=device).manual_seed(seed)
    pix = torch.arange(n, device=device)
    px = (pix // spp) % width
    py = (pix // spp) // width
    jx = torch.rand(n, device=device, generator=g)
    jy = torch.rand(n, device=device, generator=g)
    tan = math.tan(math.radians(22.5))
    sx = ((px.float() + jx) / width * 2 - 1) * tan * (width / height)
    sy = (1 - (py.float() + jy) / height * 2) * tan
    d = torch.stack([sx, sy, torch.ones_like(sx)], 0)
    d = d / d.norm(dim=0, keepdim=True)
    o = torch.tensor([0.5, 0.5, -1.5], device=device)[:, None].expand(3, n)
    return torch.cat([o, d], 0).contiguous()
