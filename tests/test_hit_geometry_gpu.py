"""skw_scene_hit_geometry: the differential geometry that the reference's
TriangleAccelerator::Intersect completes each hit with
(TriangleMesh::ComputeDifferentialGeometry, Raytracer/Core/TriangleMesh.cpp:
414-484) -- point, geometric and shading normals, barycentrics and t of the
double Moller-Trumbore test -- against a numpy restatement of the same
double arithmetic (bit for bit), on the closest hits of the scene's own
accelerator."""
import ctypes as C

import numpy as np
import pytest

from skwarka_gb300 import _lib, scenes
from skwarka_gb300.accel import TriangleMesh
from skwarka_gb300.render import Material, RenderPrimitive, RenderScene

pytestmark = pytest.mark.gpu


def _scene():
    bv, bt = scenes._box_inward()
    v, t = scenes.sphere_mesh(4)
    sv = (v * 0.35 + np.array([0.1, -0.2, 0.05])).astype(np.float32)
    normals = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    prims = [RenderPrimitive(TriangleMesh(bv, bt), 0), RenderPrimitive(TriangleMesh(sv, t), 0, vertex_normals=normals)]
    return prims, RenderScene(prims, [Material()])


def _expected(prims, rays, hits):
    out = np.full((len(rays), 12), np.nan)
    for i, (r, h) in enumerate(zip(rays.astype(np.float64), hits)):
        if h[1] < 0:
            continue
        m = prims[h[1]].mesh
        tri = m.triangles[h[2]]
        v0, v1, v2 = (m.vertices[tri[k]].astype(np.float64) for k in range(3))
        o, d = r[:3], r[3:6]
        e1, e2 = v1 - v0, v2 - v0
        s1 = np.cross(d, e2)
        inv = 1.0 / ((s1[0] * e1[0] + s1[1] * e1[1]) + s1[2] * e1[2])
        dd = o - v0
        b1 = ((dd[0] * s1[0] + dd[1] * s1[1]) + dd[2] * s1[2]) * inv
        s2 = np.cross(dd, e1)
        b2 = ((d[0] * s2[0] + d[1] * s2[1]) + d[2] * s2[2]) * inv
        t = ((e2[0] * s2[0] + e2[1] * s2[1]) + e2[2] * s2[2]) * inv
        p = o + d * t

        def normalized(a):
            l2 = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]
            return a * (1.0 / np.sqrt(l2))

        ng = normalized(np.cross(e1, e2))
        ns = ng
        if prims[h[1]].vertex_normals is not None:
            # the mesh stores each vertex normal as Vector3D<float>::Normalized
            # makes it: squared length and root in float, the double
            # reciprocal, each coordinate times it rounded to float
            n = prims[h[1]].vertex_normals.astype(np.float32)
            l2 = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
            inv = 1.0 / np.sqrt(l2).astype(np.float64)
            n = (n.astype(np.float64) * inv[:, None]).astype(np.float32).astype(np.float64)
            b0 = (1.0 - b1) - b2
            ns = normalized((n[tri[0]] * b0 + n[tri[1]] * b1) + n[tri[2]] * b2)
        out[i] = np.concatenate([p, ng, ns, [b1, b2, t]])
    return out


def test_hit_geometry_matches_restatement(gpu):
    import torch
    prims, sc = _scene()
    lib = _lib.load()
    accel = lib.skw_scene_accel(sc.handle)
    rng = np.random.default_rng(4)
    n = 4000
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.uniform(-0.9, 0.9, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = np.inf
    r = torch.from_numpy(rays).cuda()
    hits = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.skw_intersect(accel, r.data_ptr(), n, hits.data_ptr(), s), sc.ctx.handle)
    geo = sc.hit_geometry(r, hits).cpu().numpy()
    h = hits.cpu().numpy()
    want = _expected(prims, rays, h)
    hit = h[:, 1] >= 0
    on_sphere = h[:, 1] == 1
    print(f"[hit geometry] {hit.sum()} hits, {on_sphere.sum()} on the sphere (interpolated normals)")
    assert hit.all() and on_sphere.sum() > 100  # every ray starts inside the closed box
    diff = geo[hit] != want[hit]
    print("[hit geometry] mismatching entries per column:", diff.sum(0).tolist())
    assert not diff.any()
    t_float = h[:, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(geo[hit, 11] - t_float[hit]) <= 1e-5 * np.abs(geo[hit, 11]))
    assert np.allclose(np.linalg.norm(geo[hit, 3:6], axis=1), 1.0) and np.allclose(np.linalg.norm(geo[hit, 6:9], axis=1), 1.0)
    # a miss gives NaN
    miss = torch.tensor([[5, 5, 5, 1, 0, 0, 0, np.inf]], dtype=torch.float32, device="cuda")
    mh = torch.tensor([[0x7F800000, -1, -1, 0]], dtype=torch.int32, device="cuda")
    assert np.isnan(sc.hit_geometry(miss, mh).cpu().numpy()).all()
