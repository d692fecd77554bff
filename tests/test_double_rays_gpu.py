"""Double-precision rays (skw_ray_d) through the C ABI against the oracle
and the reference's own TriangleAccelerator::Intersect / IntersectTest on
the same double rays (Math/Ray.h:57-59): hit ids and the double t equal
bit for bit, any-hit answers equal.

The rays are the reference unit test's kind (origin uniform in the world
bounds, direction from U[0,1)^3 normalised in double, tmin in U[-10, 10],
tmax in U[100, 10000]; UnitTests/MainTests/Raytracer/Core/
TriangleAccelerator.test.h:65-98) plus uniform rays on the query scene,
with origins and directions that are not float-representable, so the
traversal's rounding bounds are exercised."""
import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import scenes
from skwarka_gb300.accel import Primitive, TriangleAccelerator, TriangleMesh, unpack_hits_d

pytestmark = pytest.mark.gpu


def double_rays(lo, hi, n, seed, unit_test=False, tmax_range=None):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.uniform(0, 1, size=(n, 3)) if unit_test else rng.normal(size=(n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    r = np.zeros((n, 8), np.float64)
    r[:, :3], r[:, 3:6] = o, d
    if unit_test:
        r[:, 6] = rng.uniform(-10, 10, n)
        r[:, 7] = rng.uniform(100, 10000, n)
    else:
        r[:, 6] = 0.0
        r[:, 7] = np.inf if tmax_range is None else rng.uniform(*tmax_range, n)
    return r


def _accel(meshes):
    return TriangleAccelerator([Primitive(TriangleMesh(v, t)) for v, t in meshes])


def _check(acc, oa, rays, label):
    import torch
    got = unpack_hits_d(acc.intersect_d(torch.from_numpy(rays).cuda()))
    want = oa.intersect_d(rays)
    same = (got["prim"] == want["prim"]) & (got["tri"] == want["tri"])
    print(f"[{label}] rays={len(rays)} id agreement={same.mean():.6f} hits={(want['prim'] >= 0).sum()}")
    assert same.all()
    assert np.array_equal(got["t"].view(np.uint64), want["t"].view(np.uint64))
    occ = acc.intersect_test_d(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert np.array_equal(occ, oa.intersect_test_d(rays))


def test_unit_test_spheres_double_rays(gpu, oracle):
    meshes = sf.unit_test_spheres()
    lo, hi = scenes.scene_bounds(meshes)
    rays = double_rays(lo, hi, 20_000, 31, unit_test=True)
    _check(_accel(meshes), oracle.accel(meshes), rays, "unit-test spheres, double rays")


def test_query_scene_double_rays(gpu, oracle):
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    acc, oa = _accel(meshes), oracle.accel(meshes)
    _check(acc, oa, double_rays(lo, hi, 200_000, 32), "query scene, double rays")
    _check(acc, oa, double_rays(lo, hi, 200_000, 33, tmax_range=(0.0, 2.0)), "query scene, double shadow rays")


def test_double_rays_against_reference(gpu, reference):
    """The reference's own Intersect on the same double rays."""
    import torch
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    rays = double_rays(lo, hi, 50_000, 34)
    acc = _accel(meshes)
    got = unpack_hits_d(acc.intersect_d(torch.from_numpy(rays).cuda()))
    want = reference.accel(meshes).intersect_d(rays)
    # the reference orders primitives by mesh address, which only permutes
    # triangles within a leaf: ids are compared directly, t bit for bit
    assert np.array_equal(got["prim"], want["prim"]) and np.array_equal(got["tri"], want["tri"])
    assert np.array_equal(got["t"].view(np.uint64), want["t"].view(np.uint64))


def test_double_rays_host_equals_device(gpu):
    """The host-buffer double-ray entry points (chunks over two streams
    above 2^21 rays) equal the device ones bit for bit."""
    import torch
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    rays = double_rays(lo, hi, 2_200_000, 35)
    acc = _accel(meshes)
    dev = unpack_hits_d(acc.intersect_d(torch.from_numpy(rays).cuda()))
    host = acc.intersect_d(rays)
    for k in ("prim", "tri"):
        assert np.array_equal(dev[k], host[k])
    assert np.array_equal(dev["t"].view(np.uint64), host["t"].view(np.uint64))
    assert np.array_equal(acc.intersect_test_d(torch.from_numpy(rays).cuda()).cpu().numpy(),
                          acc.intersect_test_d(rays))
