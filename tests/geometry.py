"""Host-side test geometry: seeded random soups and rays (numpy), and the
reference's meshed sphere (MakeMeshedSphere, plymesh.cpp:110-174) used by its
Triangle.Watertight test (shape_tests.cpp:22-48)."""
import math

import numpy as np


def random_soup(n, rng, half=0.01):
    c = rng.random((n, 1, 3), dtype=np.float32)
    off = (2.0 * rng.random((n, 3, 3), dtype=np.float32) - 1.0) * np.float32(half)
    return (c + off).reshape(-1, 3).astype(np.float32)


def sphere_rays(n, rng, center=(0.5, 0.5, 0.5), radius=2.0, tmin=1e-4, tmax=np.inf):
    u = rng.random((n, 5))
    z = 1.0 - 2.0 * u[:, 0]
    phi = 2.0 * np.pi * u[:, 1]
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    o = np.stack([center[0] + radius * s * np.cos(phi), center[1] + radius * s * np.sin(phi),
                  center[2] + radius * z], 0)
    d = u[:, 2:5].T - o
    d /= np.linalg.norm(d, axis=0, keepdims=True)
    r = np.zeros((8, n), np.float32)
    r[0:3] = o
    r[3:6] = d
    r[6] = tmin
    r[7] = tmax
    return r


def meshed_sphere(n_theta, n_phi, radius):
    """Vertices and indices of MakeMeshedSphere (plymesh.cpp:110-174)."""
    verts = []
    for t in range(n_theta):
        theta = math.pi * t / (n_theta - 1)
        ct, st = math.cos(theta), math.sin(theta)
        for p in range(n_phi):
            phi = 2 * math.pi * p / (n_phi - 1)
            if t == 0:
                verts.append((0.0, 0.0, radius))
            elif t == n_theta - 1:
                verts.append((0.0, 0.0, -radius))
            elif p == n_phi - 1:
                verts.append(verts[len(verts) - (n_phi - 1)])
            else:
                verts.append((radius * st * math.cos(phi), radius * st * math.sin(phi), radius * ct))
    off = lambda t, p: t * n_phi + p
    ind = []
    for p in range(n_phi - 1):
        ind += [off(0, 0), off(1, p), off(1, p + 1)]
    for t in range(1, n_theta - 2):
        for p in range(n_phi - 1):
            ind += [off(t, p), off(t + 1, p), off(t + 1, p + 1)]
            ind += [off(t, p), off(t + 1, p + 1), off(t, p + 1)]
    for p in range(n_phi - 1):
        ind += [off(n_theta - 1, 0), off(n_theta - 2, p), off(n_theta - 2, p + 1)]
    return np.array(verts, np.float32), np.array(ind, np.int32).reshape(-1, 3)


def interior_rays(n, rng, r_in=0.5):
    """Triangle.Watertight rays: origins 0.5 * uniform-sphere point, uniform
    directions (shape_tests.cpp:31-38)."""
    def usph(k):
        u = rng.random((k, 2))
        z = 1 - 2 * u[:, 1]
        phi = 2 * np.pi * u[:, 0]
        s = np.sqrt(np.maximum(0, 1 - z * z))
        return np.stack([s * np.cos(phi), s * np.sin(phi), z], 0)
    o = r_in * usph(n)
    d = usph(n)
    r = np.zeros((8, n), np.float32)
    r[0:3] = o
    r[3:6] = d
    r[6] = 0.0
    r[7] = np.inf
    return r


def value_noise_grid(res, rng, scale=4.0):
    """Smooth seeded density in [0, scale] on a res^3 lattice (z, y, x)."""
    base = rng.random((6, 6, 6))
    x = np.linspace(0, 5, res)
    i0 = np.clip(np.floor(x).astype(int), 0, 4)
    f = x - i0
    f = f * f * (3 - 2 * f)
    g = base
    g = g[i0] * (1 - f)[:, None, None] + g[i0 + 1] * f[:, None, None]
    g = g[:, i0] * (1 - f)[None, :, None] + g[:, i0 + 1] * f[None, :, None]
    g = g[:, :, i0] * (1 - f)[None, None, :] + g[:, :, i0 + 1] * f[None, None, :]
    return (scale * g).astype(np.float32)


def geometric_clusters(n_scales, per_scale, rng):
    """Clusters of per_scale small triangles at (2^-k, 2^-k, 2^-k), k < n_scales:
    a top-down split peels off one scale at a time, so trees reach any depth."""
    out = []
    for k in range(n_scales):
        c = np.float32(2.0 ** -k)
        tri = c + (rng.uniform(-1.0, 1.0, (per_scale, 3, 3)) * (0.02 * c)).astype(np.float32)
        out.append(tri.astype(np.float32))
    return np.concatenate(out).reshape(-1, 3)
