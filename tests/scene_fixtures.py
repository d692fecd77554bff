"""Scenes and ray sets shared by the tests (seeded, small enough for the
oracle to finish in seconds)."""
import numpy as np

from skwarka_gb300 import scenes


def unit_test_spheres():
    """The four tessellated spheres of the reference's accelerator unit test
    (UnitTests/MainTests/Raytracer/Core/TriangleAccelerator.test.h:35-42):
    (center, radius, subdivisions)."""
    spec = [((0, 0, 0), 10.0, 5), ((-20, 0, 0), 20.0, 5), ((0, -10, 0), 0.5, 5), ((1000, 0, 0), 1000.0, 6)]
    meshes = []
    for c, r, n in spec:
        v, t = scenes.sphere_mesh(n)
        meshes.append(((v * r + np.asarray(c, np.float64)).astype(np.float32), t))
    return meshes


def unit_test_rays(meshes, n=1000, seed=11):
    """Random rays like the unit test's: origin uniform in the world bounds,
    direction from U[0,1]^3 normalised, tmin in U[-10, 10], tmax in U[100, 10000]."""
    lo, hi = scenes.scene_bounds(meshes)
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.uniform(0, 1, size=(n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    r = np.zeros((n, 8), np.float32)
    r[:, :3] = o
    r[:, 3:6] = d
    r[:, 6] = rng.uniform(-10, 10, n)
    r[:, 7] = rng.uniform(100, 10000, n)
    return r


def small_query_scene():
    """A 16k-triangle displaced sphere plus 2,000 random triangles."""
    return scenes.ray_query_scene(sphere_subdivisions=6, n_random=2000, seed=5)


def flat_tiles(n=64, seed=2):
    """Axis-aligned coplanar squares (z = 0.5), two triangles each: every node
    above the leaves has zero extent in z, exercising that split path."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(0, 1, size=(n, 2)).astype(np.float32)
    s = np.float32(0.02)
    v = np.zeros((n, 4, 3), np.float32)
    v[:, 0, :2] = xy
    v[:, 1, :2] = xy + [s, 0]
    v[:, 2, :2] = xy + [s, s]
    v[:, 3, :2] = xy + [0, s]
    v[:, :, 2] = 0.5
    t = np.zeros((n, 2, 3), np.int32)
    base = (np.arange(n) * 4)[:, None]
    t[:, 0] = base + [0, 1, 2]
    t[:, 1] = base + [0, 2, 3]
    return [(v.reshape(-1, 3), t.reshape(-1, 3))]


def canonical_leaf_order(info, tri_prim, tri_index):
    """(prim, tri) pairs with each leaf's range sorted.  The reference orders
    its primitives by mesh address before building (a std::map keyed by
    pointer, TriangleAccelerator.cpp:25-38), which only permutes triangles
    inside a leaf; comparisons with it use this canonical order."""
    pairs = np.stack([tri_prim, tri_index], 1).astype(np.int64)
    out = pairs.copy()
    leaves = info[info[:, 0] == 0]
    for b, e in leaves[:, 4:6]:
        seg = pairs[b:e]
        out[b:e] = seg[np.lexsort((seg[:, 1], seg[:, 0]))]
    return out
