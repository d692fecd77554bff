"""The plain direct-lighting and differentiation configurations at their
stated sizes.

Plain direct lighting (256 x 256, 2x2 stratified samples, the 12-triangle
box with the two jittered spheres and the quad light): against the
reference's SamplerBasedRenderer renders of the same scene at 256 x 256
(tests/golden/direct_box_256.npz: its 16x16-sample image and the statistics
of its 2x2 image).  The GPU's 2x2 image must have a mean relative error
(pixel luminance, against the reference's 16x16 image) within 15 % of the
reference's own 2x2 image's: equal image error at equal sample count.  Its
mean luminance must be within 1 % of the reference's, and at 16x16 samples
every 8x8-pixel block's mean luminance within 3 % of the reference's
16x16 image (relative to the block, or to a quarter of the image mean in
shadow).

Differentiation (the 201,742-triangle scene, 512 x 512, 16 samples per
pixel, per-triangle RGB albedo in [0.1, 0.9] and a scalar emission scale,
L2 loss against a target rendered with the albedo perturbed by N(0, 0.05)):
adjoint gradients against central finite differences (eps 1e-3) of every
colour channel of 256 random triangles, within 1e-3 relative as a vector
and per entry relative to max(|fd|, 1 % of the largest).  The triangles
are drawn among those the camera sees (a nonzero adjoint gradient); a
uniform draw over all triangles, most of them hidden, must give zero from
both sides.  With the configuration's medium (sigma_a 0.05, sigma_s 0.2,
HG g = 0.3) the forward render costs ~14 times more, so that case runs the
same camera at 128 x 128 (the whole view at a quarter of the resolution;
the centre crop of the 512 x 512 image shows only a few dozen triangles)
with the same 16 samples per pixel."""
from pathlib import Path

import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.render import Camera, RenderScene

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
LUM = np.array([0.05316285, 0.58515348, 0.36168367])
EPS = 1e-3


def test_c1_box_at_configuration_size(gpu):
    g = np.load(GOLD / "direct_box_256.npz")
    prims, mats, cam = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats)
    c = cam(256, 256)
    ref_hi = g["ref_16x16"].astype(np.float64)
    lh = ref_hi @ LUM
    lo = sc.render_direct(c, 2, 2, seed=101).cpu().numpy() @ LUM
    hi = sc.render_direct(c, 16, 16, seed=102).cpu().numpy() @ LUM
    e_gpu = float(np.mean(np.abs(lo - lh) / np.maximum(lh, 1e-3 * lh.mean())))
    e_ref = float(g["ref_2x2_mre"])
    m_ref, m_gpu = float(lh.mean()), float(hi.mean())
    blocks = lambda im: im.reshape(32, 8, 32, 8).mean(axis=(1, 3))  # noqa: E731
    rb = blocks(lh)
    rel = np.abs(blocks(hi) - rb) / np.maximum(rb, 0.25 * m_ref)
    print(f"[C1 256x256] 2x2 MRE: reference {e_ref:.4f}, GPU {e_gpu:.4f}; mean luminance reference {m_ref:.5f} "
          f"GPU {m_gpu:.5f} (GPU 2x2 {float(lo.mean()):.5f}, reference 2x2 {float(g['ref_2x2_mean']):.5f}); "
          f"worst 8x8 block {rel.max():.4f}")
    assert abs(e_gpu / e_ref - 1.0) <= 0.15
    assert abs(m_gpu / m_ref - 1.0) <= 0.01
    assert abs(float(lo.mean()) / float(g["ref_2x2_mean"]) - 1.0) <= 0.02
    assert rel.max() <= 0.03


def _c5(size, crop=1, medium=False):
    """The differentiation configuration's renderer, albedo and target; crop
    > 1 renders the centre 1/crop of the 512 x 512 image at the same pixel
    pitch (same camera, view angle tangent divided by crop)."""
    import torch
    from skwarka_gb300.adjoint import DirectLighting
    from skwarka_gb300.render import Medium
    prims, mats = scenes.batching_scene()
    sc = RenderScene(prims, mats)
    if medium:
        sc.set_medium(Medium(sigma_a=(0.05,) * 3, sigma_s=(0.2,) * 3, g=0.3, step=0.05))
    fov = 2.0 * np.arctan(np.tan(np.radians(70) / 2.0) / crop)
    cam = Camera.look_at((0.0, 0.3, -0.9), (0.0, -0.4, 0.6), (0, 1, 0), fov, size, size)
    r = DirectLighting(sc, cam, 4, 4, 1, seed=3)
    rng = np.random.default_rng(6)
    albedo = torch.tensor(rng.uniform(0.1, 0.9, size=(sc.n_triangles, 3)), dtype=torch.float32, device="cuda")
    target = r.forward_image((albedo + torch.tensor(rng.normal(0, 0.05, size=albedo.shape), dtype=torch.float32,
                                                    device="cuda")).clamp(0, 1), 1.0).double()
    return sc, r, albedo, target


def _check_fd(r, albedo, target, n_tri, label, per_entry=1e-3):
    import torch

    def loss(a, s=1.0):
        return float(((r.forward_image(a, s).double() - target) ** 2).sum())

    img = r.forward_image(albedo, 1.0)
    g_alb, g_em = r.adjoint(albedo, 1.0, (2.0 * (img.double() - target)).float())
    g = g_alb.double().cpu().numpy()
    seen = np.flatnonzero(np.abs(g).sum(1) > 0)
    rng = np.random.default_rng(7)
    pick = rng.choice(seen, size=min(n_tri, seen.size), replace=False)
    got, want = [], []
    for t in pick:
        for c in range(3):
            ap, am = albedo.clone(), albedo.clone()
            ap[t, c] += EPS
            am[t, c] -= EPS
            want.append((loss(ap) - loss(am)) / (2 * EPS))
            got.append(g[t, c])
    got, want = np.array(got), np.array(want)
    vec = np.linalg.norm(got - want) / np.linalg.norm(want)
    per = np.abs(got - want) / np.maximum(np.abs(want), 0.01 * np.abs(want).max())
    # hidden triangles: zero both ways (a uniform draw over all triangles)
    hidden = np.setdiff1d(rng.choice(g.shape[0], size=64, replace=False), seen)[:8]
    for t in hidden:
        ap, am = albedo.clone(), albedo.clone()
        ap[t] += EPS
        am[t] -= EPS
        # the medium's in-scattering sums use float atomics, so two renders
        # differ in their last bits; hidden triangles must not move the loss
        # beyond that
        lp, lm = loss(ap), loss(am)
        assert abs(lp - lm) <= 1e-7 * abs(lp) and not g[t].any()
    fd_em = (loss(albedo, 1.0 + EPS) - loss(albedo, 1.0 - EPS)) / (2 * EPS)
    em = float(g_em)
    print(f"[{label}] {seen.size} triangles seen of {g.shape[0]}; {len(pick)} checked x 3 channels: vector rel err "
          f"{vec:.2e}, worst entry {per.max():.2e}; emission {em:.6e} fd {fd_em:.6e}; {len(hidden)} hidden ok")
    assert len(pick) == n_tri
    assert vec <= 1e-3 and per.max() <= per_entry
    assert abs(em - fd_em) <= 1e-3 * abs(fd_em)


def test_c5_adjoint_at_configuration_size(gpu):
    sc, r, albedo, target = _c5(512)
    assert sc.n_triangles == 201_742
    _check_fd(r, albedo, target, 256, "C5 512x512x16")


def test_c5_adjoint_with_medium(gpu):
    sc, r, albedo, target = _c5(128, medium=True)
    # the medium's in-scattering sums use float atomics: two forward renders
    # differ in their last bits, which the difference quotient divides by
    # 2e-3, so single small entries get 1e-2 (the vector stays within 1e-3)
    _check_fd(r, albedo, target, 256, "C5 medium, 128x128 x16", per_entry=1e-2)
