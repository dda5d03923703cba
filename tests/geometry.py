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


def sliver_comb(group, rng):
    """A scene whose every box is crossed by a bundle of rays that hit
    nothing but a target at the far end, so that traversal visits every node
    and its stack grows with the tree's depth.  Slivers along (1, 1, 1) (the
    third corner within 2^-13 of the axis) with
    boxes [c - 0.25, c + 0.25]^3 sit at centroids c = 0.5 + e_a 2^j / 1024
    (axis a, j < 9) and at c = 0.5: the Morton codes of the 28 groups differ in
    one bit each, a chain 27 levels deep, and each group of `group`
    equal-code slivers adds a balanced subtree.  Two corner specks fix the
    scene box to [0, 1]^3.  Returns (positions [n, 3], rays [8, m])."""
    cents = [np.full(3, 0.5, np.float32)]
    for a in range(3):
        for j in range(9):
            c = np.full(3, 0.5, np.float32)
            c[a] += np.float32(2.0 ** j / 1024.0)
            cents.append(c)
    tris = []
    eps = np.float32(2.0 ** -12)
    for c in cents:
        ang = rng.uniform(0, 2 * np.pi, group)
        off = np.stack([np.cos(ang), np.sin(ang), -np.cos(ang) - np.sin(ang)], 1).astype(np.float32) * eps * 0.5
        t = np.empty((group, 3, 3), np.float32)
        t[:, 0] = c - np.float32(0.25)
        t[:, 1] = c + np.float32(0.25)
        t[:, 2] = c + off
        tris.append(t)
    speck = np.float32(1e-6)
    tris.append(np.array([[[0, 0, 0], [speck, 0, 0], [0, speck, 0]],
                          [[1, 1, 1], [1 - speck, 1, 1], [1, 1 - speck, 1]]], np.float32))
    # the target: a triangle across the bundle beyond the slivers' boxes' near faces
    tris.append(np.array([[[0.95, 0.5, 0.5], [0.95, 0.75, 0.5], [0.95, 0.62, 0.75]]], np.float32))
    pos = np.concatenate(tris).reshape(-1, 3)
    # rays along +x at y - z = 0.04 +- 0.004: at least 0.0047 from every sliver
    # axis (where y - z = 0 or +-2^j / 1024), inside every sliver box in y and z
    m = 4096
    jit = rng.uniform(-0.002, 0.002, (2, m)).astype(np.float32)
    r = np.zeros((8, m), np.float32)
    r[0], r[1], r[2] = 0.0, np.float32(0.62) + jit[0], np.float32(0.58) + jit[1]
    r[3], r[4], r[5] = 1.0, 0.0, 0.0
    r[6], r[7] = 0.0, np.inf
    return pos.astype(np.float32), r


def edge_case_scene(rng):
    """Triangles and rays at the edges of the arithmetic: a 16 x 16 grid of
    axis-aligned squares in the plane z = 0.5 (two triangles each, sharing
    edges and vertices), collinear and single-point triangles, and a random
    soup; rays straight down through grid vertices and edges, rays in the
    grid's plane and along the axes, diagonal rays, a zero direction and NaN
    origins.  Returns (positions [n, 3], rays [8, m])."""
    tris = []
    k = 16
    for i in range(k):
        for j in range(k):
            x0, x1, y0, y1 = i / k, (i + 1) / k, j / k, (j + 1) / k
            tris.append([[x0, y0, 0.5], [x1, y0, 0.5], [x1, y1, 0.5]])
            tris.append([[x0, y0, 0.5], [x1, y1, 0.5], [x0, y1, 0.5]])
    tris.append([[0.1, 0.1, 0.2], [0.2, 0.2, 0.2], [0.3, 0.3, 0.2]])  # collinear
    tris.append([[0.4, 0.4, 0.3], [0.4, 0.4, 0.3], [0.4, 0.4, 0.3]])  # a point
    tris.append([[0.6, 0.1, 0.8], [0.6, 0.1, 0.8], [0.7, 0.2, 0.8]])  # a segment
    pos = np.concatenate([np.array(tris, np.float32).reshape(-1, 3), random_soup(1000, rng)])
    rays = []
    g = np.arange(k + 1, dtype=np.float32) / np.float32(k)
    for x in g:  # down through every grid vertex and the midpoints of vertical edges
        for y in g:
            rays.append([x, y, 2.0, 0.0, 0.0, -1.0])
            rays.append([x, y + np.float32(0.5 / k), 2.0, 0.0, 0.0, -1.0])
    for y in g:  # in the grid's plane and just above and below it, along +x and -y
        for z in (0.5, np.nextafter(np.float32(0.5), np.float32(1)), np.nextafter(np.float32(0.5), np.float32(0))):
            rays.append([-1.0, y, z, 1.0, 0.0, 0.0])
            rays.append([y, 2.0, z, 0.0, -1.0, 0.0])
    d = rng.normal(size=(512, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.float32(0.5) - 1.5 * d
    rays += [list(o[i]) + list(d[i]) for i in range(512)]
    rays.append([0.5, 0.5, 2.0, 0.0, 0.0, 0.0])  # zero direction
    rays.append([np.nan, 0.5, 2.0, 0.0, 0.0, -1.0])
    rays.append([0.5, 0.5, 2.0, np.nan, 0.0, -1.0])
    r = np.zeros((8, len(rays)), np.float32)
    r[:6] = np.array(rays, np.float32).T
    r[6], r[7] = 0.0, np.inf
    return pos.astype(np.float32), r


def volume_edge_rays(rng):
    """Rays at the edges of the volume's box arithmetic (box [0, 1]^3):
    origins inside the box, finite tmax ending inside it, rays in a face's
    plane and parallel to it (zero direction components), rays just outside a
    face, rays that miss the box, and NaN origins.  Returns rays [8, m]."""
    rays = []
    n = 512
    o = rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for i in range(n):  # inside, unbounded and ending inside
        rays.append(list(o[i]) + list(d[i]) + [0.0, np.inf])
        rays.append(list(o[i]) + list(d[i]) + [0.0, 0.1 + 0.3 * float(rng.random())])
    g = np.linspace(0.0, 1.0, 9, dtype=np.float32)
    for a in g:  # in the faces' planes x = 0, y = 1, along axes, and just outside x = 0
        for b in g:
            rays.append([0.0, a, -0.5, 0.0, 0.0, 1.0, 0.0, np.inf])
            rays.append([a, 1.0, b - 2.0, 0.0, 0.0, 1.0, 0.0, np.inf])
            rays.append([-0.5, a, b, 1.0, 0.0, 0.0, 0.0, np.inf])
            rays.append([np.nextafter(np.float32(0), np.float32(-1)), a, -0.5, 0.0, 0.0, 1.0, 0.0, np.inf])
    for i in range(64):  # misses
        rays.append([2.0, 2.0, float(i) / 64, 1.0, 0.0, 0.0, 0.0, np.inf])
    rays.append([np.nan, 0.5, 0.5, 1.0, 0.0, 0.0, 0.0, np.inf])
    rays.append([0.5, 0.5, -1.0, 0.0, np.nan, 1.0, 0.0, np.inf])
    return np.array(rays, np.float32).T.copy()
