"""SubstrateMaterial (one- and two-roughness: Blinn and Ashikhmin-Shirley,
the latter under each source of the shading tangent), UberMaterial and
MixMaterial on the GPU against the reference's own renders of the same
scenes (tests/golden/materials.npz,
from tests/golden/make_golden.py materials: SamplerBasedRenderer with
DirectLightingLTEIntegrator, 16x16 spp, maximum specular depth 6).

The GPU renders at 32x32 spp; the mean luminance agrees within 2 % and
8x8-pixel blocks of the sphere scenes within 6 %, as for the other BSDFs.
The substrate's lobe-sampling probability is the GPU's own (the reference
reads it from a tabulated fit): it changes the variance, not the
expectation."""
from pathlib import Path

import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import _lib
from skwarka_gb300.render import MATTE, MIX, TRANSPARENT, UBER, Material, RenderScene

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "materials.npz"
LUM = np.array([0.05316285, 0.58515348, 0.36168367])


@pytest.mark.parametrize("name", ["plane_substrate", "plane_substrate_rough", "plane_uber_opaque",
                                  "plane_mix_matte_plastic", "sphere_uber", "sphere_mix_glass_matte",
                                  "plane_substrate_aniso", "plane_substrate_aniso_uv", "sphere_substrate_aniso"])
def test_material_render_matches_reference(gpu, name):
    prims, mats, lights, cam = sf.material_cases()[name]
    ref = np.load(GOLD)[name]
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(6)
    img = sc.render_direct(cam, 32, 32, seed=11).cpu().numpy()
    assert np.isfinite(img).all() and (img >= 0).all()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    msg = f"[material {name}] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}"
    if name.startswith("sphere"):
        rb = (ref @ LUM).reshape(4, 8, 6, 8).mean(axis=(1, 3))
        gb = (img @ LUM).reshape(4, 8, 6, 8).mean(axis=(1, 3))
        rel = np.abs(gb - rb) / np.maximum(rb, 0.25 * rb.mean())
        msg += f"; worst block {rel.max():.4f}"
        assert rel.max() <= 0.06, msg
    elif "aniso" in name:
        # the highlight's shape follows the shading tangent: 4x4-pixel blocks
        rb = (ref @ LUM).reshape(4, 4, 6, 4).mean(axis=(1, 3))
        gb = (img @ LUM).reshape(4, 4, 6, 4).mean(axis=(1, 3))
        rel = np.abs(gb - rb) / np.maximum(rb, 0.25 * rb.mean())
        msg += f"; worst block {rel.max():.4f}"
        assert rel.max() <= 0.06, msg
    print(msg)
    assert abs(m_gpu / m_ref - 1.0) <= 0.02, msg


def test_uber_and_mix_photon_render_is_finite(gpu):
    """Photon shooting samples every component of a mixed BSDF (specular ones
    included, each with probability 1 / count): the shoot deposits photons on
    the uber sphere's diffuse part and the render stays finite and
    non-negative."""
    from skwarka_gb300.photon import PhotonMap, render_photon
    for name in ("sphere_uber", "sphere_mix_glass_matte"):
        prims, mats, lights, cam = sf.material_cases()[name]
        sc = RenderScene(prims, mats, lights)
        pm = PhotonMap.shoot(sc, 100_000, max_bounces=8, rr_probability=0.7, seed=3)
        info = pm.info()
        img = render_photon(sc, pm, cam, 2, 2, gather_samples=4).cpu().numpy()
        print(f"[material photons {name}] direct {info['n_direct']} indirect {info['n_indirect']} "
              f"caustic {info['n_caustic']} mean {img.mean():.5f}")
        assert info["n_direct"] > 0 and np.isfinite(img).all() and (img >= 0).all() and img.mean() > 0


def test_material_refusals(gpu):
    """A mix of mixes, a mix of two materials that both have specular
    components, a mix index outside the material array and an uber material
    without a positive refractive index are refused."""
    prims, mats, lights, cam = sf.material_cases()["plane_mix_matte_plastic"]
    glass = Material(kind=TRANSPARENT, kd=(1, 1, 1), ks=(1, 1, 1))
    cases = [
        ([Material(kind=MIX, mix=(1, 2)), Material(kind=MIX, mix=(2, -1)), Material(), Material(kd=(0, 0, 0))],
         "mix of mix"),
        ([Material(kind=MIX, mix=(1, 2)), glass, glass, Material(kd=(0, 0, 0))], "specular"),
        ([Material(kind=MIX, mix=(1, 7)), Material(), Material(), Material(kd=(0, 0, 0))], "indices"),
        ([Material(kind=UBER, refractive_index=0.0), Material(), Material(), Material(kd=(0, 0, 0))],
         "refractive index"),
    ]
    for ms, what in cases:
        with pytest.raises(_lib.SkwError, match=what):
            RenderScene(prims, ms, lights)
    # a mix with one side only (mix[1] = -1) renders the first material scaled
    half = RenderScene(prims, [Material(kind=MIX, mix=(1, -1), mix_scale=(0.5, 0.5, 0.5)),
                               Material(kind=MATTE, kd=(0.8, 0.6, 0.4)), Material(), Material(kd=(0, 0, 0))],
                       lights).render_direct(cam, 4, 4, seed=1).cpu().numpy()
    full = RenderScene(prims, [Material(kind=MATTE, kd=(0.8, 0.6, 0.4)), Material(), Material(),
                               Material(kd=(0, 0, 0))], lights).render_direct(cam, 4, 4, seed=1).cpu().numpy()
    assert abs(half.mean() / full.mean() - 0.5) <= 0.02
