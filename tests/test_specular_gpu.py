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
  bounces only) and no direct photon on glass; the maps agree with the
  reference's ShootPhotons over the same 2,000,000 paths.
* The photon-mapping render follows the same trees, with caustic-map
  radiance and final gather at their diffuse hits, against the reference's
  photon renders.
* The direct-lighting adjoint replays the same trees (finite differences).
* A medium along the specular rays (single-camera render), against the
  reference's render; the batch refuses that combination.
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
    """2,000,000 paths from the point light above the glass sphere, against
    the reference's ShootPhotons over the same paths.  Direct photons (first
    hits; radical-inverse emission) within 0.5 %; caustic photons (floor hits
    after specular bounces only) in count within 3 %, centroid within 0.01 and
    spread within 2 %; indirect photons on the floor within 5 %.  Most
    indirect photons lie on the glass itself: photons trapped by total
    internal reflection inside the faceted sphere, whose number of bounces
    before numerical error lets them out depends on each implementation's
    arithmetic (double in the reference, float here), compared within 12 %.
    The reference has no bounce limit; the GPU's is set to 1024 here (with
    the default 64 a double-precision restatement of the walk loses ~3 % of
    the floor photons and ~8 % of those on the glass)."""
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    sc = RenderScene(prims, mats, lights)
    pm = PhotonMap.shoot(sc, 2_000_000, max_bounces=1024, seed=5)
    info = pm.info()
    g = np.load(GOLD)
    want = g["photon_counts"]
    ind = pm.export("indirect")
    floor = int((np.abs(ind["position"][:, 2]) < 1e-4).sum())
    got = np.array([info["n_caustic"], info["n_direct"], info["n_indirect"], floor])
    print(f"[specular photons] caustic / direct / indirect / indirect on the floor: gpu {got.tolist()} "
          f"reference {want.tolist()}")
    assert abs(got[1] / want[1] - 1) <= 0.005
    assert abs(got[0] / want[0] - 1) <= 0.03
    assert abs(got[3] / want[3] - 1) <= 0.05
    assert abs(got[2] / want[2] - 1) <= 0.12
    assert info["paths_caustic"] == 2_000_000
    c = pm.export("caustic")["position"]
    assert np.allclose(c[:, 2], 0.0, atol=1e-4)  # caustics land on the floor
    cxy = np.concatenate([c[:, :2].mean(0), [np.sqrt((c[:, :2] ** 2).sum(1).mean())]])
    print(f"[specular photons] caustic centroid and spread gpu {cxy.round(4).tolist()} "
          f"reference {g['caustic_xy'].round(4).tolist()}")
    assert np.abs(cxy[:2] - g["caustic_xy"][:2]).max() <= 0.01
    assert abs(cxy[2] / g["caustic_xy"][2] - 1) <= 0.02
    d = pm.export("direct")
    assert (d["position"][:, 2] < 1e-4).all()  # no direct photon on the glass


@pytest.mark.parametrize("name", ["glass_point", "glass_area"])
def test_specular_photon_render_matches_reference(gpu, name):
    """PhotonLTEIntegrator with the sphere of glass: caustic-map radiance and
    final gather at every diffuse hit of every sample's specular tree, 1,000,000
    photon paths, 16 gather samples, 8x8 spp.  The photon-map part (photon
    render minus direct render) within 6 % in mean luminance and the photon
    image's 8x8 blocks within 8 % of the reference's (the reference's own
    photon part moves by 2-3 % in the mean and up to 10 % in the caustic's
    blocks between 200,000 and 2,000,000 paths)."""
    from skwarka_gb300.photon import render_photon
    g = np.load(GOLD)
    prims, mats, lights, cam = sf.specular_cases()[name]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(6)
    pm = PhotonMap.shoot(sc, 1_000_000, max_bounces=1024, seed=11)
    img = render_photon(sc, pm, cam, 8, 8, gather_samples=16, seed=13).cpu().numpy()
    direct = sc.render_direct(cam, 8, 8, seed=13).cpu().numpy()
    assert np.isfinite(img).all() and (img >= 0).all()
    ph_gpu, ph_ref = ((img - direct) @ LUM).mean(), ((g[name + "_photon"] - g[name]) @ LUM).mean()
    rb = _blocks(g[name + "_photon"])
    rel = np.abs(_blocks(img) - rb) / np.maximum(rb, 0.25 * rb.mean())
    print(f"[specular photon {name}] photon-map part gpu {ph_gpu:.5f} reference {ph_ref:.5f}; "
          f"worst block {rel.max():.4f}")
    assert abs(ph_gpu / ph_ref - 1) <= 0.06
    assert rel.max() <= 0.08


def test_specular_adjoint_matches_finite_differences(gpu):
    """The adjoint replays the specular trees too: with the glass fixed (a
    transparent surface's reflectance is its material's, not a per-triangle
    albedo) the image is linear in the floor's albedo and in the emission
    scale, so central differences (eps 1e-3) of a weighted sum of the image
    match the adjoint within 1e-3 relative; the glass triangles get exactly
    zero."""
    import torch
    from skwarka_gb300.adjoint import DirectLighting
    prims, mats, lights, cam = sf.specular_cases()["glass_area"]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(6)
    r = DirectLighting(sc, cam, 4, 4, 1, seed=5)
    n = sc.n_triangles
    rng = np.random.default_rng(3)
    albedo = torch.tensor(rng.uniform(0.2, 0.8, size=(n, 3)), dtype=torch.float32, device="cuda")
    w = torch.tensor(rng.uniform(0.5, 1.5, size=(cam.height, cam.width, 3)), dtype=torch.float64, device="cuda")
    g_alb, g_em = r.adjoint(albedo, 1.0, w.float())
    g = g_alb.double().cpu().numpy()
    loss = lambda a, sc_: float((r.forward_image(a, sc_).double() * w).sum())  # noqa: E731
    eps = 1e-3
    got, want = [], []
    for t in (0, 1):  # the floor's two triangles (mesh order: the floor is primitive 0)
        for c in range(3):
            a_p, a_m = albedo.clone(), albedo.clone()
            a_p[t, c] += eps
            a_m[t, c] -= eps
            want.append((loss(a_p, 1.0) - loss(a_m, 1.0)) / (2 * eps))
            got.append(g[t, c])
    fd_em = (loss(albedo, 1.0 + eps) - loss(albedo, 1.0 - eps)) / (2 * eps)
    got, want = np.array(got), np.array(want)
    print(f"[specular adjoint] floor albedo: adjoint {got.round(3).tolist()} fd {want.round(3).tolist()}; "
          f"emission adjoint {float(g_em[0]):.4f} fd {fd_em:.4f}")
    assert np.linalg.norm(got - want) <= 1e-3 * np.linalg.norm(want)
    assert abs(float(g_em[0]) - fd_em) <= 1e-3 * abs(fd_em)
    assert np.all(g[2:2 + 1024] == 0.0)  # the sphere (primitive 1): transparent


def test_specular_in_medium_matches_reference(gpu):
    """The glass sphere under the point light inside a scattering medium:
    every specular ray is marched through the medium like the camera ray
    (LTEIntegrator::Radiance at every depth) -- its in-scattering added and
    its transmittance applied to what it reaches.  Mean luminance within 2 %
    and 8x8 blocks within 6 % of the reference's render."""
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    sc = RenderScene(prims, mats, lights, medium=sf.specular_medium())
    sc.set_max_specular_depth(6)
    img = sc.render_direct(cam, 32, 32, seed=17).cpu().numpy()
    ref = np.load(GOLD)["glass_point_medium"]
    assert np.isfinite(img).all() and (img >= 0).all()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    rb = _blocks(ref)
    rel = np.abs(_blocks(img) - rb) / np.maximum(rb, 0.25 * rb.mean())
    print(f"[specular medium] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}; worst block {rel.max():.4f}")
    assert abs(m_gpu / m_ref - 1) <= 0.02
    assert rel.max() <= 0.06


def test_specular_in_medium_batch_matches_single_renders(gpu):
    """A medium together with specular materials in a batch: the graph
    marches each specular level's rays through the medium in a conditional
    loop over device-counted chunks (no host round trip), and gives the
    single-camera renders' images (whose levels read their lengths back).
    The specular slot adds its shadow and BSDF samples with atomics, so the
    two agree to float rounding, not bit for bit."""
    import torch
    from skwarka_gb300.render import RenderBatch
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    sc = RenderScene(prims, mats, lights, medium=sf.specular_medium())
    sc.set_max_specular_depth(4)
    cams = [cam, cam]
    b = RenderBatch(sc, cams, 2, 2, seed=3)
    films = b.new_films()
    b.run(films)
    b.run(films)  # a second launch of the same graph resets its loop state
    torch.cuda.synchronize()
    for v in range(len(cams)):
        single = sc.render_direct(cams[v], 2, 2, seed=3 + v).cpu().numpy()
        got = b.view(films, v).cpu().numpy()
        err = np.abs(got - single).max() / max(float(np.abs(single).max()), 1e-6)
        print(f"[specular medium batch] view {v}: max rel diff {err:.2e}, mean {got.mean():.5f} vs {single.mean():.5f}")
        assert np.isfinite(got).all() and err <= 1e-4


def test_specular_in_medium_adjoint_matches_finite_differences(gpu):
    """The adjoint with a medium around glass: every specular level's rays
    are marched through the medium in the replay too (their weights take the
    segments' transmittance, the in-scattering adds its emission-scale
    derivative), so central differences (eps 1e-3) of a weighted sum of the
    image match the adjoint within 1e-3 relative for the floor's albedo and
    the emission scale."""
    import torch
    from skwarka_gb300.adjoint import DirectLighting
    prims, mats, lights, cam = sf.specular_cases()["glass_area"]
    sc = RenderScene(prims, mats, lights, medium=sf.specular_medium())
    sc.set_max_specular_depth(4)
    r = DirectLighting(sc, cam, 3, 3, 1, seed=7)
    n = sc.n_triangles
    rng = np.random.default_rng(4)
    albedo = torch.tensor(rng.uniform(0.2, 0.8, size=(n, 3)), dtype=torch.float32, device="cuda")
    w = torch.tensor(rng.uniform(0.5, 1.5, size=(cam.height, cam.width, 3)), dtype=torch.float64, device="cuda")
    g_alb, g_em = r.adjoint(albedo, 1.0, w.float())
    g = g_alb.double().cpu().numpy()
    loss = lambda a, sc_: float((r.forward_image(a, sc_).double() * w).sum())  # noqa: E731
    eps = 1e-3
    got, want = [], []
    for t in (0, 1):  # the floor's two triangles
        for c in range(3):
            a_p, a_m = albedo.clone(), albedo.clone()
            a_p[t, c] += eps
            a_m[t, c] -= eps
            want.append((loss(a_p, 1.0) - loss(a_m, 1.0)) / (2 * eps))
            got.append(g[t, c])
    fd_em = (loss(albedo, 1.0 + eps) - loss(albedo, 1.0 - eps)) / (2 * eps)
    got, want = np.array(got), np.array(want)
    print(f"[specular medium adjoint] floor albedo: adjoint {got.round(3).tolist()} fd {want.round(3).tolist()}; "
          f"emission adjoint {float(g_em[0]):.4f} fd {fd_em:.4f}")
    assert np.linalg.norm(got - want) <= 1e-3 * np.linalg.norm(want)
    assert abs(float(g_em[0]) - fd_em) <= 1e-3 * abs(fd_em)


def test_specular_edge_cases(gpu):
    """Depth 11 (the deepest: 4,095 rays per sample) renders; depths outside
    [0, 11] and a non-positive refractive index are refused; a transparent
    material with neither reflection nor transmission scatters nothing (the
    sphere goes dark where it is seen directly)."""
    from skwarka_gb300.render import TRANSPARENT, Material
    prims, mats, lights, cam = sf.specular_cases()["glass_area"]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(11)
    deep = sc.render_direct(cam, 1, 1, seed=2).cpu().numpy()
    assert np.isfinite(deep).all() and (deep >= 0).all() and deep.mean() > 0
    for bad in (-1, 12):
        with pytest.raises(_lib.SkwError):
            sc.set_max_specular_depth(bad)
    with pytest.raises(_lib.SkwError, match="refractive index"):
        RenderScene(prims, [mats[0], Material(kind=TRANSPARENT, refractive_index=0.0), mats[2]], lights)
    dark = RenderScene(prims, [mats[0], Material(kind=TRANSPARENT, kd=(0, 0, 0), ks=(0, 0, 0)), mats[2]], lights)
    img = dark.render_direct(cam, 2, 2, seed=2).cpu().numpy() @ LUM
    glass = sc.render_direct(cam, 2, 2, seed=2).cpu().numpy() @ LUM
    center = (slice(cam.height // 2 - 2, cam.height // 2 + 2), slice(cam.width // 2 - 2, cam.width // 2 + 2))
    assert np.all(img[center] == 0.0) and glass[center].mean() > 0.0
