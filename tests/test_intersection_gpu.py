"""The whole Intersection on the GPU (skw_scene_intersection: the
DifferentialGeometry of TriangleMesh::ComputeDifferentialGeometry,
Raytracer/Core/TriangleMesh.cpp:414-561, and the m_cross / m_dot of
TriangleAccelerator::Intersect, TriangleAccelerator.cpp:303-347) against the
reference's own Intersect on the same double ray differentials, bit for bit;
the reference's GetNextMinT (CoreUtils.h:139-149) on it; and the reference's
"no self re-hit" known-answer test (UnitTests/MainTests/Raytracer/Core/
TriangleAccelerator.test.h:101-135) on the outgoing rays the renders make."""
import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import scenes
from skwarka_gb300.accel import TriangleMesh, unpack_hits, unpack_hits_d
from skwarka_gb300.render import Material, RenderPrimitive, RenderScene

pytestmark = pytest.mark.gpu


def sphere_normals(v, center):
    n = v.astype(np.float64) - np.asarray(center, np.float64)
    return (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)


def dg_scene():
    """Two spheres with vertex normals (so shading normals interpolate), one
    without, and a box wall without: identity transforms."""
    meshes = sf.unit_test_spheres()[:3]
    centers = [(0, 0, 0), (-20, 0, 0), (0, -10, 0)]
    normals = [sphere_normals(meshes[0][0], centers[0]), None, sphere_normals(meshes[2][0], centers[2])]
    wall_v = np.array([[-45, -25, 15], [15, -25, 15], [15, 25, 15], [-45, 25, 15]], np.float32)
    wall_t = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    meshes = meshes + [(wall_v, wall_t)]
    normals = normals + [None]
    prims = [RenderPrimitive(TriangleMesh(v, t), 0, vertex_normals=n) for (v, t), n in zip(meshes, normals)]
    return meshes, normals, prims


def ray_differentials(n, seed):
    """Camera-like double rays from in front of the spheres toward them, with
    next-pixel rays offset by ~1e-3 (the reference's RayDifferential)."""
    rng = np.random.default_rng(seed)
    o = np.array([-10.0, 0.0, -60.0]) + rng.normal(scale=0.5, size=(n, 3))
    target = rng.uniform([-40, -20, -5], [10, 20, 5], size=(n, 3))
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8))
    rays[:, :3], rays[:, 3:6], rays[:, 6], rays[:, 7] = o, d, 0.0, np.inf
    diffs = np.zeros((n, 12))
    for k, off in ((0, np.array([1e-3, 0, 0])), (6, np.array([0, 1e-3, 0]))):
        dd = d + off
        diffs[:, k:k + 3] = o + rng.normal(scale=1e-4, size=(n, 3))
        diffs[:, k + 3:k + 6] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
    return rays, diffs


@pytest.mark.parametrize("with_diffs", [True, False])
def test_intersection_matches_reference(gpu, reference, with_diffs):
    import torch
    meshes, normals, prims = dg_scene()
    sc = RenderScene(prims, [Material()])
    rays, diffs = ray_differentials(20_000, 41)
    rt = torch.from_numpy(rays).cuda()
    hits = sc.accelerator().intersect_d(rt)
    got = sc.intersection(rt, hits, torch.from_numpy(diffs).cuda() if with_diffs else None).cpu().numpy()
    want = reference.accel(meshes, normals=normals).intersection(rays, diffs if with_diffs else None)
    ids = got[:, 35].copy().view(np.int32).reshape(-1, 2)
    hit = want[:, 35] >= 0
    print(f"[intersection diffs={with_diffs}] rays={len(rays)} hits={hit.sum()}")
    assert hit.sum() > 10_000
    assert np.array_equal(ids[:, 0], np.where(hit, want[:, 35], -1).astype(np.int32))
    assert np.array_equal(ids[:, 1], np.where(hit, want[:, 36], -1).astype(np.int32))
    g, w = got[hit, :35], want[hit, :35]
    diff = g.view(np.uint64) != w.view(np.uint64)
    names = ["point"] * 3 + ["ng"] * 3 + ["ns"] * 3 + ["uv"] * 2 + ["pdx"] * 3 + ["pdy"] * 3 + ["ndx"] * 3 + \
        ["ndy"] * 3 + ["duvdx"] * 2 + ["duvdy"] * 2 + ["tangent"] * 3 + ["cross"] * 3 + ["dot", "t"]
    bad = sorted({names[c] for c in np.nonzero(diff.any(0))[0]})
    print(f"   fields differing: {bad}")
    assert not diff.any()
    assert np.isnan(got[~hit, :35]).all()


def test_next_min_t_matches_reference(gpu, reference):
    """GetNextMinT of each Intersection for a random direction: the host
    restatement (skw_next_min_t) on the GPU's Intersection equals the
    reference's on its own, bit for bit."""
    import ctypes as C

    import torch
    from skwarka_gb300 import _lib
    meshes, normals, prims = dg_scene()
    sc = RenderScene(prims, [Material()])
    rays, _ = ray_differentials(5_000, 42)
    rng = np.random.default_rng(43)
    nd = rng.normal(size=(len(rays), 3))
    nd /= np.linalg.norm(nd, axis=1, keepdims=True)
    rt = torch.from_numpy(rays).cuda()
    got = sc.intersection(rt, sc.accelerator().intersect_d(rt)).cpu().numpy()
    _, want = reference.accel(meshes, normals=normals).intersection(rays, None, nd)
    lib = _lib.load()
    hit = ~np.isnan(want)
    t = np.array([lib.skw_next_min_t(got[i].ctypes.data, nd[i].ctypes.data) if hit[i] else np.nan
                  for i in range(len(rays))])
    assert hit.sum() > 2_000
    assert np.array_equal(t[hit].view(np.uint64), want[hit].view(np.uint64))


def test_outgoing_rays_never_rehit_their_triangle(gpu):
    """The reference's epsilon test (TriangleAccelerator.test.h:101-135) on
    its own scene: 1000 random rays, and from each hit 1000 outgoing rays in
    directions from U[0,1)^3, started as the renders start them (float hit
    point, tmin = GetNextMinT); none may hit the triangle it leaves."""
    import torch
    meshes = sf.unit_test_spheres()
    sc = RenderScene([RenderPrimitive(TriangleMesh(v, t), 0) for v, t in meshes], [Material()])
    acc = sc.accelerator()
    rays = sf.unit_test_rays(meshes, 1000, seed=44)
    rt = torch.from_numpy(rays).cuda()
    h = acc.intersect(rt)
    hit = (h[:, 1] >= 0).cpu().numpy()
    idx = np.nonzero(hit)[0]
    n2 = 1000
    rep = torch.from_numpy(np.repeat(idx, n2)).cuda()
    rng = np.random.default_rng(45)
    dirs = rng.uniform(0, 1, size=(len(idx) * n2, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    out = sc.next_rays(rt[rep].contiguous(), h[rep].contiguous(), torch.from_numpy(dirs).cuda())
    h2 = unpack_hits(acc.intersect(out))
    src = unpack_hits(h[rep])
    rehit = (h2["prim"] == src["prim"]) & (h2["tri"] == src["tri"])
    print(f"[epsilon] {len(idx)} hits x {n2} outgoing rays; re-hits {rehit.sum()}")
    assert len(idx) > 500
    assert not rehit.any()


def test_outgoing_rays_keep_nearby_geometry(gpu):
    """Thin slabs: two parallel quads very close together.  A ray leaving
    the lower quad upward starts at its own plane crossing plus 1e-14
    (GetNextMinT, rounded up to float), so it must still hit the upper quad:
    1e-5 apart near the origin, and three float steps (2.3e-5) apart at
    z = 100 in a scene of size 100, where the former fixed offset
    (2e-6 (1 + scene size) = 2e-4) skipped the upper quad."""
    import torch
    z_lo = np.float32(100.0)
    z_hi = z_lo
    for _ in range(3):
        z_hi = np.nextafter(z_hi, np.float32(np.inf))
    for zl, zh, scale in ((np.float32(0.0), np.float32(1e-5), 1.0), (z_lo, z_hi, 100.0)):
        q = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32) * np.float32(scale)
        v0, v1 = q.copy(), q.copy()
        v0[:, 2], v1[:, 2] = zl, zh
        tris = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
        sc = RenderScene([RenderPrimitive(TriangleMesh(v0, tris), 0), RenderPrimitive(TriangleMesh(v1, tris), 0)],
                         [Material()])
        acc = sc.accelerator()
        rng = np.random.default_rng(46)
        n = 10_000
        rays = np.zeros((n, 8), np.float32)
        rays[:, :2] = rng.uniform(-0.5, 0.5, size=(n, 2)) * scale
        rays[:, 2] = zl - 1.0
        rays[:, 5] = 1.0
        rays[:, 7] = np.inf
        rt = torch.from_numpy(rays).cuda()
        h = acc.intersect(rt)
        assert bool((h[:, 1] == 0).all())
        d = rng.uniform(-0.3, 0.3, size=(n, 3))
        d[:, 2] = 1.0
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        out = sc.next_rays(rt, h, torch.from_numpy(d).cuda())
        h2 = unpack_hits(acc.intersect(out))
        frac = (h2["prim"] == 1).mean()
        print(f"[thin slab {float(zh) - float(zl):.3g} at z={float(zl)}] outgoing rays reaching the upper quad: {frac:.4f}")
        assert frac == 1.0
