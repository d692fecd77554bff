"""Direct-lighting adjoint (skw_render_direct_adjoint, hand-written CUDA,
replaying the forward's rays from the same seed) against central finite
differences of the forward render (skw_render_direct) on the same seed.

With geometry and visibility fixed the estimator is linear in each albedo
and in the emission scale, and the L2 loss is quadratic, so a central
difference is exact up to the float rounding of the forward images (about
6e-8 of a pixel's value, which dominates only for triangles covering a tiny
fraction of a pixel).  The gradients must agree within 1e-3 relative (eps =
1e-3): as a vector over all tested entries, and per entry relative to
max(|fd|, 1 % of the largest tested |fd|).  Triangles that no camera ray
reaches must get exactly zero from both."""
import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.adjoint import DirectLighting
from skwarka_gb300.render import Camera, RenderScene

pytestmark = pytest.mark.gpu
EPS = 1e-3


def _scene():
    """The box with its quad light and three spheres in view: matte (1,024
    triangles), plastic (256) and metal (64)."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import METAL, PLASTIC, Material, RenderPrimitive
    rng = np.random.default_rng(2)
    bv, bt = scenes._box_inward()
    mats = [Material(kd=(0.5, 0.5, 0.5)), Material(kd=(0.0, 0.0, 0.0)), Material(kd=(0.6, 0.5, 0.4)),
            Material(kind=PLASTIC, kd=(0.3, 0.4, 0.6), ks=(0.4, 0.4, 0.4), roughness=0.15),
            Material(kind=METAL, eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2), roughness=0.2)]
    prims = [RenderPrimitive(TriangleMesh(bv, bt), 0)]
    for lvl, c, r, m in ((4, (-0.35, -0.6, 0.25), 0.38, 2), (3, (0.45, -0.68, -0.2), 0.3, 3),
                         (2, (0.1, -0.2, 0.5), 0.15, 4)):
        v, t, n = scenes._jittered_sphere(lvl, c, r, rng)
        prims.append(RenderPrimitive(TriangleMesh(v, t), m, vertex_normals=n))
    lv = np.array([[-0.3, 0.98, -0.3], [0.3, 0.98, -0.3], [0.3, 0.98, 0.3], [-0.3, 0.98, 0.3]], np.float32)
    prims.append(RenderPrimitive(TriangleMesh(lv, np.array([[0, 1, 2], [0, 2, 3]], np.int32)), 1,
                                 emission=(10.0, 10.0, 10.0)))
    return prims, mats


def _setup(spp=(4, 4), size=64):
    import torch
    prims, mats = _scene()
    sc = RenderScene(prims, mats)
    cam = Camera.look_at((0.0, 0.1, -0.95), (0.0, -0.3, 1.0), (0, 1, 0), np.radians(75), size, size)
    r = DirectLighting(sc, cam, spp[0], spp[1], 1, seed=21)
    rng = np.random.default_rng(6)
    n = sc.n_triangles
    albedo = torch.tensor(rng.uniform(0.1, 0.9, size=(n, 3)), dtype=torch.float32, device="cuda")
    target_alb = (albedo + torch.tensor(rng.normal(0, 0.05, size=(n, 3)), dtype=torch.float32,
                                        device="cuda")).clamp(0.0, 1.0)
    target = r.forward_image(target_alb, 1.0).double()
    return r, albedo, target


def _loss(r, albedo, scale, target):
    return float(((r.forward_image(albedo, scale).double() - target) ** 2).sum())


def test_adjoint_matches_finite_differences(gpu):
    import torch
    r, albedo, target = _setup()
    img = r.forward_image(albedo, 1.0)
    d_img = 2.0 * (img.double() - target)
    g_alb, g_em = r.adjoint(albedo, 1.0, d_img.float())
    g = g_alb.double().cpu().numpy()
    nz = np.flatnonzero(np.abs(g).sum(1) > 0)
    zero = np.flatnonzero(np.abs(g).sum(1) == 0)
    print(f"[adjoint] {nz.size} triangles with a gradient, {zero.size} without")
    assert nz.size > 100 and zero.size > 0
    rng = np.random.default_rng(7)
    got, want = [], []
    for t in rng.choice(nz, size=min(32, nz.size), replace=False):
        for c in range(3):
            a_p, a_m = albedo.clone(), albedo.clone()
            a_p[t, c] += EPS
            a_m[t, c] -= EPS
            want.append((_loss(r, a_p, 1.0, target) - _loss(r, a_m, 1.0, target)) / (2 * EPS))
            got.append(g[t, c])
    got, want = np.array(got), np.array(want)
    vec = np.linalg.norm(got - want) / np.linalg.norm(want)
    per = np.abs(got - want) / np.maximum(np.abs(want), 0.01 * np.abs(want).max())
    worst = float(per.max())
    assert vec <= 1e-3, vec
    assert worst <= 1e-3, (worst, got[per.argmax()], want[per.argmax()])
    for t in rng.choice(zero, size=min(8, zero.size), replace=False):
        a_p = albedo.clone()
        a_p[t] += EPS
        assert torch.equal(r.forward_image(a_p, 1.0), img)
    fd_em = (_loss(r, albedo, 1.0 + EPS, target) - _loss(r, albedo, 1.0 - EPS, target)) / (2 * EPS)
    em = float(g_em.item())
    print(f"[adjoint] albedo: vector rel err {vec:.2e}, worst entry {worst:.2e}; "
          f"emission grad {em:.6e} fd {fd_em:.6e}")
    assert abs(em - fd_em) <= 1e-3 * abs(fd_em)


def test_autograd_harness(gpu):
    import torch
    r, albedo, target = _setup(spp=(2, 2), size=32)
    a = albedo.clone().requires_grad_(True)
    s = torch.tensor(1.3, dtype=torch.float64, device="cuda", requires_grad=True)
    loss = ((r(a, s).double() - target) ** 2).sum()
    loss.backward()
    img = r.forward_image(albedo, 1.3)
    g_alb, g_em = r.adjoint(albedo, 1.3, (2.0 * (img.double() - target)).float())
    assert torch.allclose(a.grad, g_alb, rtol=1e-5, atol=1e-8)
    assert abs(float(s.grad) - float(g_em.item())) <= 1e-6 * abs(float(g_em.item()))


def test_adjoint_is_linear_in_dfilm(gpu):
    import torch
    r, albedo, _ = _setup(spp=(2, 2), size=32)
    d1 = torch.rand((32, 32, 3), device="cuda")
    d2 = torch.rand((32, 32, 3), device="cuda")
    g1, e1 = r.adjoint(albedo, 1.0, d1)
    g2, e2 = r.adjoint(albedo, 1.0, d2)
    g12, e12 = r.adjoint(albedo, 1.0, d1 + 2.0 * d2)
    assert torch.allclose(g12, g1 + 2.0 * g2, rtol=1e-4, atol=1e-6)
    assert abs(float(e12) - float(e1) - 2.0 * float(e2)) <= 1e-4 * abs(float(e12))
