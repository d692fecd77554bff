"""Traversal of accelerators with instances (meshes shared by several
primitives) on the GPU against the reference's own TriangleAccelerator over
the same shared meshes and transforms (TriangleAccelerator.cpp:54-102,
213-233): closest-hit ids and t, any-hit answers, for float and double
rays; the reference's instancing test (TriangleAccelerator.test.h:164-203:
instanced tetrahedra against the same tetrahedra transformed into world
space, t and points within 1e-3); and a render of an instanced scene against
the same scene with every instance copied into world space."""
import numpy as np
import pytest

import instancing_fixtures as inf
from skwarka_gb300 import scenes
from skwarka_gb300.accel import TriangleAccelerator, unpack_hits, unpack_hits_d
from test_double_rays_gpu import double_rays
from test_instancing import primitives, ref_accel

pytestmark = pytest.mark.gpu


def _bounds(meshes, mesh_of, xforms):
    pts = []
    for m, x in zip(mesh_of, xforms):
        v = meshes[m][0].astype(np.float64)
        if x is not None:
            v = v @ np.asarray(x)[:3, :3].T + np.asarray(x)[:3, 3]
        pts.append(v)
    p = np.concatenate(pts)
    return p.min(0), p.max(0)


def test_instanced_hits_match_reference(gpu, reference):
    import torch
    meshes, mesh_of, xforms = inf.instanced_scene()
    acc = TriangleAccelerator(primitives(meshes, mesh_of, xforms))
    ra = ref_accel(reference, meshes, mesh_of, xforms)
    lo, hi = _bounds(meshes, mesh_of, xforms)
    rays = scenes.uniform_rays(100_000, lo, hi, seed=64)
    got = unpack_hits(acc.intersect(torch.from_numpy(rays).cuda()))
    want = ra.intersect(rays)
    same = (got["prim"] == want["prim"]) & (got["tri"] == want["tri"])
    hit = same & (want["prim"] >= 0)
    rel = np.abs(got["t"][hit] - want["t"][hit]) / np.abs(want["t"][hit])
    uses = np.bincount(mesh_of)
    inst_hits = np.isin(want["prim"], [p for p, m in enumerate(mesh_of) if uses[m] > 1])
    print(f"[instanced float rays] agree {same.mean():.6f}, hits {int((want['prim'] >= 0).sum())} "
          f"({int(inst_hits.sum())} on instances), max t rel {rel.max():.2e}")
    assert same.mean() >= 0.9999 and inst_hits.sum() > 1000
    assert rel.max() <= 1e-5
    srays = scenes.uniform_rays(100_000, lo, hi, seed=65, tmax_range=(0.0, 20.0))
    occ = acc.intersect_test(torch.from_numpy(srays).cuda()).cpu().numpy()
    assert (occ == ra.intersect_test(srays)).mean() >= 0.9999
    # double rays: the reference's exact t
    drays = double_rays(lo, hi, 50_000, 66)
    gd = unpack_hits_d(acc.intersect_d(torch.from_numpy(drays).cuda()))
    wd = ra.intersect_d(drays)
    same = (gd["prim"] == wd["prim"]) & (gd["tri"] == wd["tri"])
    print(f"[instanced double rays] agree {same.mean():.6f}")
    assert same.mean() >= 0.9999
    assert np.array_equal(gd["t"][same].view(np.uint64), wd["t"][same].view(np.uint64))


def test_reference_instancing_test_on_gpu(gpu):
    """TriangleAccelerator.test.h:164-203 with 10,000 instances of one shared
    tetrahedron: the same hits (mesh triangle index), t and hit points
    within 1e-3 of an accelerator over the tetrahedra transformed into world
    space."""
    import torch
    from skwarka_gb300.accel import Primitive, TriangleMesh
    meshes, mesh_of, xforms = inf.tetra_instancing_test(10_000, seed=67)
    inst = TriangleAccelerator(primitives(meshes, mesh_of, xforms))
    v, t = meshes[0]
    flat = []
    for x in xforms:
        w = (v.astype(np.float64) @ x[:3, :3].T + x[:3, 3]).astype(np.float32)
        flat.append(Primitive(TriangleMesh(w, t)))
    world = TriangleAccelerator(flat)
    rng = np.random.default_rng(68)
    n = 10_000
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.uniform(0, 100, size=(n, 3))
    d = rng.uniform(0, 1, size=(n, 3))
    rays[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = np.inf
    r = torch.from_numpy(rays).cuda()
    a, b = unpack_hits(inst.intersect(r)), unpack_hits(world.intersect(r))
    assert np.array_equal(a["prim"] >= 0, b["prim"] >= 0)
    h = a["prim"] >= 0
    print(f"[instanced tetrahedra] {int(h.sum())} hits of {n}")
    assert h.sum() > 1000
    assert np.array_equal(a["tri"][h], b["tri"][h])
    assert np.abs(a["t"][h] - b["t"][h]).max() <= 1e-3
    pa = rays[h, :3] + rays[h, 3:6] * a["t"][h, None]
    pb = rays[h, :3] + rays[h, 3:6] * b["t"][h, None]
    assert np.abs(pa - pb).max() <= 1e-3


def test_instanced_render_equals_world_copies(gpu):
    """A direct-lighting render of the box with spheres instanced from one
    shared mesh equals (mean luminance within 0.5 %, 8x8 blocks within 3 %)
    the render of the same scene with each sphere its own world-space mesh."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import RenderPrimitive, RenderScene
    prims, mats, camf = scenes.direct_lighting_box(sphere_subdivisions=(4, 3))
    sv, st = scenes.sphere_mesh(4)
    shared = TriangleMesh(sv.astype(np.float32), st)
    rng = np.random.default_rng(69)
    inst, copies = list(prims[:1]) + [p for p in prims[1:] if any(p.emission)], []
    copies = list(inst)
    for k in range(6):
        m = np.eye(4)
        m[:3, :3] *= rng.uniform(0.08, 0.15)
        m[:3, 3] = [rng.uniform(-0.7, 0.7), rng.uniform(-0.8, -0.2), rng.uniform(-0.3, 0.7)]
        nrm = sv.astype(np.float32)
        inst.append(RenderPrimitive(shared, 0, mesh_to_world=m, vertex_normals=nrm))
        w = (sv @ m[:3, :3].T + m[:3, 3]).astype(np.float32)
        copies.append(RenderPrimitive(TriangleMesh(w, st), 0, vertex_normals=nrm))
    cam = camf(64, 64)
    a = RenderScene(inst, mats).render_direct(cam, 8, 8, seed=5).cpu().numpy()
    b = RenderScene(copies, mats).render_direct(cam, 8, 8, seed=5).cpu().numpy()
    lum = np.array([0.05316285, 0.58515348, 0.36168367])
    la, lb = a @ lum, b @ lum
    blk = lambda im: im.reshape(8, 8, 8, 8).mean(axis=(1, 3))  # noqa: E731
    rel = np.abs(blk(la) - blk(lb)) / np.maximum(blk(lb), 0.25 * lb.mean())
    print(f"[instanced render] mean {la.mean():.5f} vs world copies {lb.mean():.5f}; worst block {rel.max():.4f}")
    assert abs(la.mean() / lb.mean() - 1) <= 0.005
    assert rel.max() <= 0.03
