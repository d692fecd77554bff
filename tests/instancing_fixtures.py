"""Scenes with meshes shared by several primitives (instancing)."""
import numpy as np

from skwarka_gb300 import scenes


def _rot(axis, a):
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4)
    i, j = [(1, 2), (0, 2), (0, 1)][axis]
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    if axis == 1:
        m[i, j], m[j, i] = s, -s
    return m


def random_transform(rng, spread=100.0, scale=(0.01, 3.01)):
    """Translation * scale * rotation Y * rotation Z * rotation X, as the
    reference's instancing test composes them
    (UnitTests/MainTests/Raytracer/Core/TriangleAccelerator.test.h:170-173)."""
    t = np.eye(4)
    t[:3, 3] = rng.uniform(0, spread, 3)
    s = np.diag(list(rng.uniform(*scale, 3)) + [1.0])
    return t @ s @ _rot(1, rng.uniform(0, 6)) @ _rot(2, rng.uniform(0, 6)) @ _rot(0, rng.uniform(0, 6))


def tetrahedron():
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    t = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], np.int32)
    return v, t


def instanced_scene(seed=61, n_spheres=300, n_tetras=50):
    """meshes [(v, t)], mesh_of_prim, transforms (n_prims, 4, 4) or None
    entries: a 256-triangle sphere shared by n_spheres primitives, a
    tetrahedron shared by n_tetras, and two meshes of their own (a
    displaced sphere and a random triangle soup), one of them transformed."""
    rng = np.random.default_rng(seed)
    sv, st = scenes.sphere_mesh(3)
    meshes = [(sv.astype(np.float32), st), tetrahedron()]
    own = scenes.ray_query_scene(sphere_subdivisions=5, n_random=300, seed=seed)
    meshes += [(own[0][0] * np.float32(20) + np.float32(50), own[0][1]), (own[1][0] * np.float32(100), own[1][1])]
    mesh_of, xforms = [], []
    for _ in range(n_spheres):
        mesh_of.append(0)
        xforms.append(random_transform(rng))
    for _ in range(n_tetras):
        mesh_of.append(1)
        xforms.append(random_transform(rng, scale=(1.0, 4.0)))
    mesh_of += [2, 3]
    xforms += [None, random_transform(rng, spread=10.0, scale=(0.9, 1.1))]
    return meshes, mesh_of, xforms


def tetra_instancing_test(n=10_000, seed=62):
    """The reference's instancing test scene with the mesh really shared:
    one tetrahedron used by n primitives with random transforms."""
    rng = np.random.default_rng(seed)
    return [tetrahedron()], [0] * n, [random_transform(rng) for _ in range(n)]
