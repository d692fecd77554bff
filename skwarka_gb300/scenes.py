"""Seeded synthetic scenes and ray sets for the benchmarks and parity tests.

The same arrays feed the CUDA path and the CPU oracle, so both see identical
float32 geometry and rays.

* ``sphere_mesh(n)`` -- the reference's tessellated sphere
  (Shapes/Sphere.cpp:42-197): a tetrahedron whose triangles are split 4-way
  ``n`` times, edge midpoints pushed to the unit sphere, 4 * 4**n triangles.
  Vertex and triangle order follow the reference: new vertices in order of
  first use, each triangle replaced by its four children in place.
* ``displaced_sphere`` -- that sphere with a seeded radial gradient-noise
  displacement (the ray-query workload: n = 9 gives 1,048,576 triangles).
* ``random_triangles`` -- small triangles with uniform centroids.
* ``uniform_rays`` -- origins uniform in a box, directions uniform on S^2.
"""
from __future__ import annotations

import math

import numpy as np


def sphere_mesh(subdivisions: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit sphere: (float64 (nv, 3) vertices, int32 (4*4**n, 3) triangles)."""
    base = math.sqrt(8.0) / 3.0
    c, s = math.cos(2.0 * math.pi / 3.0), math.sin(2.0 * math.pi / 3.0)
    verts = [np.array([[0.0, 0.0, 1.0], [base, 0.0, -1.0 / 3.0], [base * c, base * s, -1.0 / 3.0],
                       [base * c, -base * s, -1.0 / 3.0]])]
    nv = 4
    tris = np.array([[1, 3, 2], [1, 0, 3], [1, 2, 0], [0, 2, 3]], dtype=np.int64)
    allv = verts[0]
    for _ in range(subdivisions):
        m = tris.shape[0]
        a = tris[:, [0, 1, 2]].reshape(-1)
        b = tris[:, [1, 2, 0]].reshape(-1)
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo * (1 << 32) + hi
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")          # unique edges by first use
        rank = np.empty_like(order)
        rank[order] = np.arange(order.size)
        mid_index = nv + rank[inv.reshape(-1)]             # new vertex id per (tri, edge)
        ea, eb = a[first[order]], b[first[order]]
        mid = (allv[ea] + allv[eb]) * 0.5
        length = np.sqrt(mid[:, 0] * mid[:, 0] + mid[:, 1] * mid[:, 1] + mid[:, 2] * mid[:, 2])
        mid = mid * (1.0 / length)[:, None]
        allv = np.concatenate([allv, mid])
        nv += mid.shape[0]
        mi = mid_index.reshape(m, 3)  # (m01, m12, m20)
        i0, i1, i2 = tris[:, 0], tris[:, 1], tris[:, 2]
        m01, m12, m20 = mi[:, 0], mi[:, 1], mi[:, 2]
        tris = np.stack([
            np.stack([i0, m01, m20], 1), np.stack([i1, m12, m01], 1),
            np.stack([i2, m20, m12], 1), np.stack([m01, m12, m20], 1)], 1).reshape(-1, 3)
    return allv, tris.astype(np.int32)


def _gradient_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3-D gradient (Perlin-style) noise in about [-1, 1]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm])
    g = rng.normal(size=(256, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255

    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    u, v, w = fade(pf[:, 0]), fade(pf[:, 1]), fade(pf[:, 2])
    out = np.zeros(p.shape[0])
    acc = {}
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                h = perm[perm[perm[pi[:, 0] + dx] + pi[:, 1] + dy] + pi[:, 2] + dz]
                d = pf - np.array([dx, dy, dz], dtype=np.float64)
                acc[(dx, dy, dz)] = np.einsum("ij,ij->i", g[h], d)
    x00 = acc[(0, 0, 0)] * (1 - u) + acc[(1, 0, 0)] * u
    x10 = acc[(0, 1, 0)] * (1 - u) + acc[(1, 1, 0)] * u
    x01 = acc[(0, 0, 1)] * (1 - u) + acc[(1, 0, 1)] * u
    x11 = acc[(0, 1, 1)] * (1 - u) + acc[(1, 1, 1)] * u
    y0 = x00 * (1 - v) + x10 * v
    y1 = x01 * (1 - v) + x11 * v
    out = y0 * (1 - w) + y1 * w
    return np.clip(out * 1.8, -1.0, 1.0)


def displaced_sphere(subdivisions: int = 9, radius: float = 1.0, amplitude: float = 0.05, frequency: float = 4.0,
                     seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Sphere of the given radius with radial displacement amplitude*noise."""
    v, t = sphere_mesh(subdivisions)
    n = _gradient_noise(v * frequency + 17.0, seed)
    r = radius * (1.0 + amplitude * n)
    return (v * r[:, None]).astype(np.float32), t


def random_triangles(n: int = 50_000, edge: float = 0.01, lo: float = 0.0, hi: float = 1.0,
                     seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """n independent triangles with centroids uniform in [lo, hi]^3 and mean edge ~ `edge`."""
    rng = np.random.default_rng(seed + 1000)
    c = rng.uniform(lo, hi, size=(n, 1, 3))
    u = rng.normal(size=(n, 3, 3))
    u /= np.linalg.norm(u, axis=2, keepdims=True)
    v = (c + u * (edge * 0.75)).astype(np.float32).reshape(-1, 3)
    t = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return v, t


def uniform_rays(n: int, lo, hi, seed: int, tmax_range: tuple[float, float] | None = None) -> np.ndarray:
    """(n, 8) float32 rays: origin uniform in [lo, hi], direction uniform on
    S^2 (normalised in double, then rounded), tmin = 0, tmax = inf or
    uniform in tmax_range."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3:6] = d
    r[:, 6] = 0.0
    if tmax_range is None:
        r[:, 7] = np.inf
    else:
        r[:, 7] = rng.uniform(tmax_range[0], tmax_range[1], size=n)
    return r


def ray_query_scene(sphere_subdivisions: int = 9, n_random: int = 50_000, seed: int = 3):
    """Displaced unit sphere (4*4**n triangles) plus `n_random` small random
    triangles in the unit cube: list of (vertices float32, triangles int32)."""
    sv, st = displaced_sphere(sphere_subdivisions, 1.0, 0.05, 4.0, seed)
    meshes = [(sv, st)]
    if n_random:
        meshes.append(random_triangles(n_random, 0.01, 0.0, 1.0, seed))
    return meshes


def scene_bounds(meshes) -> tuple[np.ndarray, np.ndarray]:
    lo = np.min([v.min(0) for v, _ in meshes], axis=0)
    hi = np.max([v.max(0) for v, _ in meshes], axis=0)
    return lo.astype(np.float64), hi.astype(np.float64)
