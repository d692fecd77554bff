"""Homogeneous participating medium (HomogeneousVolumeRegion + HG phase,
DirectLightingLTEIntegrator's single-scattering march) on the GPU against
the reference's renders (tests/golden/medium_32.npz, 16x16 spp): mean
luminance within 2 % and 8x8 blocks within 5 % for every case, including
in-scattering from an area light; a zero-density medium renders exactly like
no medium; and the adjoint with a medium against finite differences.

In-scattering from AREA lights depends on a double-rounding outcome: the
reference's march samples the light with a shadow ray that ends exactly on
the light (DiffuseAreaLightSource::SampleLighting, DiffuseAreaLightSource.cpp:
87-90, tested as is in DirectLightingLTEIntegrator.cpp:149, without the
1e-4 pull-back of the surface path), so the light's own triangle occludes
the sample whenever the double slab test and Moller-Trumbore t put the hit
inside [0, length] -- about a third of the samples in the box scene.  The
GPU march restates that decision in double for the light's own leaf, so
the box-with-area-light case is held to the same bounds as the others."""
from pathlib import Path

import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300.render import Medium, RenderScene

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "medium_32.npz"
LUM = np.array([0.05316285, 0.58515348, 0.36168367])


@pytest.mark.parametrize("name", ["point_scatter", "point_emit", "box_absorb", "box_area"])
def test_medium_matches_reference(gpu, name):
    prims, mats, lights, cam, med = sf.medium_cases()[name]
    ref = np.load(GOLD)[name]
    img = RenderScene(prims, mats, lights, medium=med).render_direct(cam, 32, 32, seed=4).cpu().numpy()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    b = lambda im: (im @ LUM).reshape(4, 8, 4, 8).mean(axis=(1, 3))  # noqa: E731
    rb = b(ref)
    rel = np.abs(b(img) - rb) / np.maximum(rb, 0.25 * rb.mean())
    print(f"[medium {name}] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}; worst block {rel.max():.4f}")
    assert abs(m_gpu / m_ref - 1) <= 0.02
    assert rel.max() <= 0.05


def test_area_light_inscattering_matches_reference(gpu):
    """The in-scattered part alone (the area-light render minus the absorbing
    render, same medium without scattering) within 3 % of the reference's:
    the term the light's self-occlusion decides."""
    prims, mats, lights, cam, med = sf.medium_cases()["box_area"]
    g = np.load(GOLD)
    ref_in = float((g["box_area"] @ LUM).mean()) - float((g["box_absorb"] @ LUM).mean())
    _, _, _, cam_a, med_a = sf.medium_cases()["box_absorb"]
    full = RenderScene(prims, mats, lights, medium=med).render_direct(cam, 32, 32, seed=4).cpu().numpy()
    absorb = RenderScene(prims, mats, lights, medium=med_a).render_direct(cam_a, 32, 32, seed=4).cpu().numpy()
    gpu_in = float((full @ LUM).mean()) - float((absorb @ LUM).mean())
    print(f"[medium box_area] in-scattering gpu {gpu_in:.5f} reference {ref_in:.5f}")
    assert abs(gpu_in / ref_in - 1) <= 0.03


def test_empty_medium_is_no_medium(gpu):
    prims, mats, lights, cam, _ = sf.medium_cases()["point_scatter"]
    sc = RenderScene(prims, mats, lights)
    a = sc.render_direct(cam, 2, 2, seed=1).cpu().numpy()
    sc.set_medium(Medium(sigma_a=(0, 0, 0), sigma_s=(0, 0, 0), emission=(0, 0, 0), step=0.1))
    b = sc.render_direct(cam, 2, 2, seed=1).cpu().numpy()
    assert np.array_equal(a, b)


def test_adjoint_with_medium(gpu):
    """Albedo and emission-scale gradients with the configuration's medium in
    the box: central differences (eps 1e-3) within 1e-3 relative."""
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.adjoint import DirectLighting
    prims, mats, camf = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats, medium=Medium(sigma_a=(0.05,) * 3, sigma_s=(0.2,) * 3, g=0.3, step=0.05))
    r = DirectLighting(sc, camf(24, 24), 2, 2, 1, seed=2)
    rng = np.random.default_rng(6)
    n = sc.n_triangles
    albedo = torch.tensor(rng.uniform(0.1, 0.9, size=(n, 3)), dtype=torch.float32, device="cuda")
    target = r.forward_image((albedo + 0.05).clamp(0, 1), 1.0).double()
    img = r.forward_image(albedo, 1.0)
    g_alb, g_em = r.adjoint(albedo, 1.0, (2.0 * (img.double() - target)).float())

    def loss(a, s):
        return float(((r.forward_image(a, s).double() - target) ** 2).sum())

    g = g_alb.double().cpu().numpy()
    order = np.argsort(-np.abs(g).sum(1))[:12]  # the walls and the most visible sphere triangles
    got, want = [], []
    for t in order:
        for c in range(3):
            ap, am = albedo.clone(), albedo.clone()
            ap[t, c] += 1e-3
            am[t, c] -= 1e-3
            want.append((loss(ap, 1.0) - loss(am, 1.0)) / 2e-3)
            got.append(g[t, c])
    got, want = np.array(got), np.array(want)
    vec = np.linalg.norm(got - want) / np.linalg.norm(want)
    fd_em = (loss(albedo, 1.001) - loss(albedo, 0.999)) / 2e-3
    print(f"[medium adjoint] albedo vector rel err {vec:.2e}; emission {float(g_em):.6e} fd {fd_em:.6e}")
    assert vec <= 1e-3
    assert abs(float(g_em) - fd_em) <= 1e-3 * abs(fd_em)
