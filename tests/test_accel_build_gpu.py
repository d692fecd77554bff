"""The accelerator's tree built on the GPU (skw_flat_tree_build_device) is
the host build's tree node for node -- same node boxes (bit for bit), split
axes, child masks, leaf ranges and triangle order -- and so the reference's
(the host build is pinned to it in test_tree_build.py).  Cases: the 1.1M
triangle ray-query scene, random soups, degenerate and duplicated triangles
(wide middle classes, the depth limit), a planar mesh with -0.0 and +0.0
coordinates (zero-extent axes, the sign rule of the node boxes), tiny
meshes and transformed primitives."""
import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.accel import Context, Primitive, TriangleAccelerator, TriangleMesh, build_flat_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    return Context(0)


def _same(prims, ctx):
    host = build_flat_tree(prims)
    dev = build_flat_tree(prims, device=ctx, min_device_triangles=0)
    assert dev["on_device"]
    assert host["nodes"].shape == dev["nodes"].shape
    assert np.array_equal(host["nodes"], dev["nodes"])
    assert np.array_equal(host["tris"].view(np.uint32), dev["tris"].view(np.uint32))
    assert np.array_equal(host["tri_prim"], dev["tri_prim"])
    assert np.array_equal(host["tri_index"], dev["tri_index"])
    assert host["max_depth"] == dev["max_depth"]
    return dev


def test_ray_query_scene(ctx):
    meshes = scenes.ray_query_scene(9, 50_000, 3)
    dev = _same([Primitive(TriangleMesh(v, t)) for v, t in meshes], ctx)
    assert dev["nodes"].shape[0] > 500_000


@pytest.mark.parametrize("n,edge,seed", [(5, 0.3, 1), (17, 0.5, 2), (1000, 0.05, 3), (60_000, 0.01, 4)])
def test_random_soups(ctx, n, edge, seed):
    v, t = scenes.random_triangles(n, edge, 0.0, 1.0, seed)
    _same([Primitive(TriangleMesh(v, t))], ctx)


def test_tiny_meshes(ctx):
    for n in (1, 2, 3, 4):
        v, t = scenes.random_triangles(n, 0.1, 0.0, 1.0, 10 + n)
        _same([Primitive(TriangleMesh(v, t))], ctx)


def test_duplicates_and_degenerates(ctx):
    # many copies of a few triangles (every split leaves them in the middle
    # class: the middle-split axes and the depth limit end the recursion),
    # zero-area triangles, and large triangles straddling every plane
    rng = np.random.default_rng(5)
    base = rng.uniform(0, 1, size=(8, 3, 3)).astype(np.float32)
    rep = np.repeat(base, 300, axis=0)
    flat = rng.uniform(0, 1, size=(500, 1, 3)).astype(np.float32).repeat(3, axis=1)
    big = rng.uniform(-1, 2, size=(200, 3, 3)).astype(np.float32)
    small = rng.uniform(0, 1, size=(4000, 1, 3)) + rng.normal(size=(4000, 3, 3)) * 0.004
    tri = np.concatenate([rep, flat, big, small.astype(np.float32)])
    tri = tri[rng.permutation(len(tri))]
    v = tri.reshape(-1, 3)
    t = np.arange(len(v), dtype=np.int32).reshape(-1, 3)
    _same([Primitive(TriangleMesh(v, t))], ctx)


def test_planar_signed_zero(ctx):
    # a grid in the plane z = 0 (zero extent: the candidate scale is
    # infinite) with x = -0.0 and +0.0 on the left column
    n = 120
    xs, ys = np.meshgrid(np.linspace(0.0, 1.0, n, dtype=np.float32), np.linspace(-1.0, 1.0, n, dtype=np.float32))
    v = np.stack([xs.ravel(), ys.ravel(), np.zeros(n * n, np.float32)], 1)
    rng = np.random.default_rng(8)
    left = np.nonzero(v[:, 0] == 0.0)[0]
    v[left[rng.uniform(size=left.size) < 0.5], 0] = np.float32(-0.0)
    v[rng.uniform(size=n * n) < 0.3, 2] = np.float32(-0.0)
    q = (np.arange(n - 1)[None, :] + n * np.arange(n - 1)[:, None]).ravel()
    t = np.concatenate([np.stack([q, q + 1, q + n], 1), np.stack([q + 1, q + n + 1, q + n], 1)]).astype(np.int32)
    t = t[rng.permutation(len(t))]
    _same([Primitive(TriangleMesh(v, t))], ctx)


def test_transformed_primitives(ctx):
    sv, st = scenes.sphere_mesh(5)
    prims = []
    for k in range(4):
        m = np.eye(4)
        m[:3, :3] *= 0.3 + 0.1 * k
        m[:3, 3] = (k * 0.7, 0.2 * k, -0.1 * k)
        prims.append(Primitive(TriangleMesh(sv.copy(), st.copy()), m))
    _same(prims, ctx)


def test_accelerator_builds_on_device(ctx):
    meshes = scenes.ray_query_scene(7, 5_000, 3)
    acc = TriangleAccelerator([Primitive(TriangleMesh(v, t)) for v, t in meshes], ctx)
    assert acc.info["built_on_device"]
    small = TriangleAccelerator([Primitive(TriangleMesh(*scenes.random_triangles(100, 0.05, 0, 1, 2)))], ctx)
    assert not small.info["built_on_device"]
    nodes, tp, ti = acc.export()
    host = build_flat_tree([Primitive(TriangleMesh(v, t)) for v, t in meshes])
    assert np.array_equal(nodes, host["nodes"])
    assert np.array_equal(tp, host["tri_prim"]) and np.array_equal(ti, host["tri_index"])
