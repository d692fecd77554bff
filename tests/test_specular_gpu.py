"""Specular materials (TransparentMaterial: SpecularReflection with a
dielectric Fresnel + SpecularTransmission) on the GPU.

* Direct-lighting renders follow the specular tree of every camera sample
  (LTEIntegrator::_SpecularReflect / _SpecularTransmit while the depth is at
  most m_max_specular_depth) and are compared with the reference's renders
  of the same scenes at 16x16 spp (tests/golden/specular_48x32.npz, maximum
  specular depth 6): mean luminance within 2 % and 8x8 blocks within 6 %.
* Depth 0 keeps only the first reflection / transmission, so its image is
  darker than depth 6 inside the sphere and equal on the floor seen
  directly.
* Photon shooting deposits caustic photons (a diffuse hit after specular
  bounces only) and no direct photon on glass; the map sizes agree with the
  reference's ShootPhotons over the same 200,000 paths.
* The scenes with a specular material are refused where the GPU path does not
  follow specular paths (adjoint, photon render, medium).
"""
from pathlib import Path

import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import _lib
from skwarka_gb300.photon import PhotonMap
from skwarka_gb300.render import Medium, RenderScene

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "specular_48x32.npz"
LUM = np.array([0.05316285, 0.58515348, 0.36168367])


def _blocks(img):
    return (img @ LUM).reshape(4, 8, 6, 8).mean(axis=(1, 3))


@pytest.mark.parametrize("name", ["glass_area", "glass_point", "tinted_area", "mirror_area"])
def test_specular_render_matches_reference(gpu, name):
    prims, mats, lights, cam = sf.specular_cases()[name]
    ref = np.load(GOLD)[name]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(6)
    img = sc.render_direct(cam, 32, 32, seed=7).cpu().numpy()
    assert np.isfinite(img).all() and (img >= 0).all()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    rb = _blocks(ref)
    rel = np.abs(_blocks(img) - rb) / np.maximum(rb, 0.25 * rb.mean())
    print(f"[specular {name}] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}; worst block {rel.max():.4f}")
    assert abs(m_gpu / m_ref - 1) <= 0.02
    assert rel.max() <= 0.06


def test_specular_depth_limits_the_tree(gpu):
    prims, mats, lights, cam = sf.specular_cases()["glass_area"]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(6)
    deep = sc.render_direct(cam, 8, 8, seed=3).cpu().numpy() @ LUM
    sc.set_max_specular_depth(0)
    shallow = sc.render_direct(cam, 8, 8, seed=3).cpu().numpy() @ LUM
    # camera ray -> sphere: depth 0 keeps the reflected and the refracted ray
    # but not what the refracted ray meets inside (the back of the sphere)
    assert shallow.sum() < 0.98 * deep.sum()
    floor_only = (np.abs(deep - shallow) <= 1e-6 * np.maximum(deep, 1e-3))
    assert floor_only.mean() > 0.3  # pixels that see the floor directly are unchanged
    with pytest.raises(_lib.SkwError):
        sc.set_max_specular_depth(12)


def test_photon_shooting_through_glass(gpu):
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    sc = RenderScene(prims, mats, lights)
    pm = PhotonMap.shoot(sc, 200_000, max_bounces=64, seed=5)
    info = pm.info()
    want = np.load(GOLD)["photon_counts"]
    got = np.array([info["n_caustic"], info["n_direct"], info["n_indirect"]])
    print(f"[specular photons] caustic / direct / indirect: gpu {got.tolist()} reference {want.tolist()}")
    assert abs(got[1] / want[1] - 1) <= 0.005  # first hits: radical-inverse emission, no roulette
    assert abs(got[0] / want[0] - 1) <= 0.06
    assert abs(got[2] / want[2] - 1) <= 0.05
    assert info["paths_caustic"] == 200_000
    c = pm.export("caustic")
    # caustics land on the floor, inside the region lit through the sphere
    assert np.allclose(c["position"][:, 2], 0.0, atol=1e-4)
    assert np.hypot(c["position"][:, 0], c["position"][:, 1]).max() < 2.5
    d = pm.export("direct")
    assert (d["position"][:, 2] < 1e-4).all()  # no direct photon on the glass


def test_specular_scene_refusals(gpu):
    import torch
    from skwarka_gb300.adjoint import DirectLighting
    from skwarka_gb300.photon import render_photon
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    sc = RenderScene(prims, mats, lights)
    sc.set_medium(Medium())
    with pytest.raises(_lib.SkwError, match="medium"):
        sc.render_direct(cam, 1, 1, seed=1)
    sc.set_medium(None)
    dl = DirectLighting(sc, cam, 1, 1)
    albedo = torch.full((sc.n_triangles, 3), 0.5, device="cuda")
    with pytest.raises(_lib.SkwError, match="specular"):
        dl.adjoint(albedo, 1.0, torch.ones(cam.height, cam.width, 3, device="cuda"))
    pm = PhotonMap.shoot(sc, 10_000, seed=1)
    with pytest.raises(_lib.SkwError, match="specular"):
        render_photon(sc, pm, cam, 1, 1)
