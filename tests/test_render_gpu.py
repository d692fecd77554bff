"""GPU direct-lighting render through the C ABI: analytic known answers (the
reference's own DirectLightingIntegrator / SamplerBasedRenderer test cases)
and statistical image parity with the reference's CPU render.

Image parity: the GPU draws its own random numbers (a counter-based
generator, not the reference's per-chunk Mersenne Twister streams), so images
are compared statistically against the reference's
16x16-sample render (tests/golden/direct_box_64.npz):

* noise level: at the configuration's 2x2 samples the GPU image's mean
  relative error (MRE) of pixel luminance must be within 15 % (+0.005) of the
  reference's own 2x2 MRE;
* convergence: at 16x16 samples the GPU MRE must fall to at most 0.3 of the
  2x2 noise level (independent noise of two 16x16 images gives about 0.2);
* bias: mean luminance within 1 %, and every 8x8-pixel block's mean luminance
  within 3 % (relative to the block's mean, or to a quarter of the image mean
  for blocks in shadow, whose relative noise is large).

Per-BSDF parity (tests/golden/direct_planes.npz): a plane of each material
under an area light and under a point light; GPU mean luminance at 32x32
samples within 2 % of the reference's at 16x16."""
from pathlib import Path

import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.accel import TriangleMesh
from skwarka_gb300.render import Camera, Material, PointLight, RenderPrimitive, RenderScene

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
LUM = np.array([0.05316285, 0.58515348, 0.36168367])  # the reference's luminance weights


def mre(a, b):
    la, lb = a @ LUM, b @ LUM
    return float(np.mean(np.abs(la - lb) / np.maximum(lb, 1e-3 * lb.mean())))


def _quad(z, half, normal_up=True):
    v = np.array([[-half, -half, z], [half, -half, z], [half, half, z], [-half, half, z]], np.float32)
    t = np.array([[0, 1, 2], [0, 2, 3]] if normal_up else [[0, 2, 1], [0, 3, 2]], np.int32)
    return TriangleMesh(v, t)


def test_point_light_known_answer(gpu):
    """DirectLightingIntegrator.test.h:46-71: a point light of intensity 100 at
    distance 9 above a white Lambertian surface: L = 100/81 / pi."""
    prims = [RenderPrimitive(_quad(0.0, 50.0), 0)]
    sc = RenderScene(prims, [Material(kd=(1.0, 1.0, 1.0))], [PointLight((0, 0, 9.0), (100.0, 100.0, 100.0))])
    cam = Camera.look_at((0, 0, 5.0), (0, 0, 0), (0, 1, 0), 0.001, 4, 4)
    img = sc.render_direct(cam, 1, 1).cpu().numpy()
    want = 100.0 / 81.0 / np.pi
    assert np.allclose(img, want, rtol=1e-4), (img.mean(), want)


def test_occluded_is_black(gpu):
    """DirectLightingIntegrator.test.h:173-201: an occluder between the light
    and the point gives exactly zero."""
    prims = [RenderPrimitive(_quad(0.0, 50.0), 0), RenderPrimitive(_quad(7.0, 1.0), 0)]
    sc = RenderScene(prims, [Material(kd=(1.0, 1.0, 1.0))], [PointLight((0, 0, 9.0), (100.0, 100.0, 100.0))])
    cam = Camera.look_at((0, 0, 5.0), (0, 0, 0), (0, 1, 0), 0.001, 4, 4)
    assert np.all(sc.render_direct(cam, 2, 2).cpu().numpy() == 0.0)


def test_point_light_inside_sphere(gpu):
    """SamplerBasedRenderer.test.h:76-105 analogue: inside a white sphere of
    radius 2 (shading normals) with a point light at the centre every pixel
    shows rho/pi * I / R^2, within 2 %."""
    v, t = scenes.sphere_mesh(5)
    prims = [RenderPrimitive(TriangleMesh((v * 2.0).astype(np.float32), t), 0, vertex_normals=v.astype(np.float32))]
    sc = RenderScene(prims, [Material(kd=(0.6, 0.6, 0.6))], [PointLight((0, 0, 0), (10.0, 10.0, 10.0))])
    cam = Camera.look_at((0.1, 0.05, 0.0), (1, 0.3, 0.2), (0, 1, 0), 1.2, 10, 10)
    img = sc.render_direct(cam, 1, 1).cpu().numpy()
    want = 0.6 / np.pi * 10.0 / 4.0
    assert np.allclose(img, want, rtol=0.02), (img.min(), img.max(), want)


def _block_means(img, b=8):
    lum = img @ LUM
    h, w = lum.shape
    return lum[: h // b * b, : w // b * b].reshape(h // b, b, w // b, b).mean(axis=(1, 3))


def test_box_image_parity_with_reference(gpu):
    g = np.load(GOLD / "direct_box_64.npz")
    prims, mats, cam = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats)
    c = cam(64, 64)
    gpu_lo = sc.render_direct(c, 2, 2, seed=11).cpu().numpy()
    gpu_hi = sc.render_direct(c, 16, 16, seed=12).cpu().numpy()
    ref_lo, ref_hi = g["ref_2x2"], g["ref_16x16"]
    e_ref, e_gpu, e_hi = mre(ref_lo, ref_hi), mre(gpu_lo, ref_hi), mre(gpu_hi, ref_hi)
    m_ref, m_gpu = float((ref_hi @ LUM).mean()), float((gpu_hi @ LUM).mean())
    rb = _block_means(ref_hi)
    blocks = np.abs(_block_means(gpu_hi) - rb) / np.maximum(rb, 0.25 * m_ref)
    print(f"[box 64x64] MRE vs reference 16x16: reference 2x2 {e_ref:.4f}, GPU 2x2 {e_gpu:.4f}, GPU 16x16 {e_hi:.4f}; "
          f"mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}; worst 8x8 block {blocks.max():.4f}")
    assert np.isfinite(gpu_lo).all() and (gpu_lo >= 0).all()
    assert e_gpu <= 1.15 * e_ref + 0.005
    assert e_hi <= 0.3 * e_ref
    assert abs(m_gpu / m_ref - 1.0) <= 0.01
    assert blocks.max() <= 0.03


@pytest.mark.parametrize("name", sorted(np.load(GOLD / "direct_planes.npz").files))
def test_bsdf_plane_parity_with_reference(gpu, name):
    import scene_fixtures as sf
    prims, mats, lights, cam = sf.material_plane_scenes()[name]
    ref = np.load(GOLD / "direct_planes.npz")[name]
    img = RenderScene(prims, mats, lights).render_direct(cam, 32, 32, seed=3).cpu().numpy()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    print(f"[{name}] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}")
    assert abs(m_gpu / m_ref - 1.0) <= 0.02


def test_render_is_deterministic(gpu):
    prims, mats, cam = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats)
    c = cam(32, 32)
    a = sc.render_direct(c, 2, 2, seed=5).cpu().numpy()
    b = sc.render_direct(c, 2, 2, seed=5).cpu().numpy()
    assert np.array_equal(a, b)


def test_sphere_area_lights_known_answer(gpu):
    """DirectLightingIntegrator.test.h:104-135 analogue: two spherical area
    lights (radiance 10 and 20) seen from a Lambertian point; the GPU estimate
    at 128x128 samples per pixel agrees with the closed form of ideal spheres
    within 2 % (the tessellated lights subtend about 1 % less; the estimate's
    own noise is about 0.5 %)."""
    import scene_fixtures as sf
    prims, mats, cam, want = sf.sphere_area_lights_case()
    img = RenderScene(prims, mats).render_direct(cam, 128, 128, seed=7).cpu().numpy()
    print(f"[sphere lights] gpu {img.mean():.5f} closed form {want:.5f}")
    assert abs(img.mean() / want - 1.0) <= 0.02


def test_square_light_known_answer(gpu):
    """A point under a square area light: the GPU estimate at 32x32 samples
    per pixel, one light sample each, agrees with the numerical integral of
    the irradiance within 1 %."""
    import scene_fixtures as sf
    prims, mats, cam, want = sf.square_light_case()
    img = RenderScene(prims, mats).render_direct(cam, 32, 32, seed=9).cpu().numpy()
    print(f"[square light] gpu {img.mean():.5f} integral {want:.5f}")
    assert abs(img.mean() / want - 1.0) <= 0.01


@pytest.mark.parametrize("name", ["area_measured", "point_measured"])
def test_measured_brdf_plane_parity(gpu, name):
    """A plane with the synthetic measured BRDF (MERLMeasuredMaterial) under
    an area light and a point light: GPU mean luminance at 32x32 samples
    within 2 % of the reference's at 16x16 (tests/golden/measured_planes.npz)."""
    import scene_fixtures as sf
    from skwarka_gb300.render import MeasuredBRDF
    m = MeasuredBRDF(scenes.merl_table())
    prims, mats, lights, cam = sf.measured_plane_scenes(m)[name]
    ref = np.load(GOLD / "measured_planes.npz")[name]
    img = RenderScene(prims, mats, lights).render_direct(cam, 32, 32, seed=3).cpu().numpy()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    print(f"[{name}] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}")
    assert abs(m_gpu / m_ref - 1.0) <= 0.02


def test_two_area_lights_parity(gpu):
    """Two area lights of different size and radiance: the light is chosen
    per shading point by the reference's irradiance strategy (bounds' solid
    angle x intensity x average cosine); mean luminance within 2 % and 8x8
    blocks within 5 % of the reference's 16x16-spp render."""
    import scene_fixtures as sf
    p, m, c = sf.two_light_scene()
    ref = np.load(GOLD / "two_lights_32.npz")["ref"]
    img = RenderScene(p, m).render_direct(c, 32, 32, seed=8).cpu().numpy()
    m_ref, m_gpu = float((ref @ LUM).mean()), float((img @ LUM).mean())
    b = lambda im: (im @ LUM).reshape(4, 8, 4, 8).mean(axis=(1, 3))  # noqa: E731
    rb = b(ref)
    rel = np.abs(b(img) - rb) / np.maximum(rb, 0.25 * rb.mean())
    print(f"[two lights] mean luminance ref {m_ref:.5f} gpu {m_gpu:.5f}; worst block {rel.max():.4f}")
    assert abs(m_gpu / m_ref - 1.0) <= 0.02
    assert rel.max() <= 0.05


def test_ld_sampler_parity_with_reference(gpu):
    """LDSampler (the GUI's sampler) at 4 samples per pixel on the box:
    the reference's LD render and this one have the same expectation (mean
    luminance within 1 % of the 16x16 stratified reference) and a similar
    quality: MRE against the 16x16 reference (averaged over four seeds: one
    render's MRE moves by ~10 % from seed to seed, dark pixels dominate it)
    within 25 % of the reference LD render's own, and at most 0.92 of the
    stratified 2x2 GPU renders' (the reference: 0.136 LD vs 0.171
    stratified)."""
    from skwarka_gb300.render import LD
    g = np.load(GOLD / "direct_box_64.npz")
    ref_ld = np.load(GOLD / "ld_box_64.npz")["ref_ld_4"]
    prims, mats, cam = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats)
    c = cam(64, 64)
    ref_hi = g["ref_16x16"]
    gpu_ld = sc.render_direct(c, 2, 2, seed=21, sampler=LD).cpu().numpy()
    gpu_ld_hi = sc.render_direct(c, 16, 16, seed=30, sampler=LD).cpu().numpy()
    seeds = (21, 22, 23, 24)
    e_ld = float(np.mean([mre(sc.render_direct(c, 2, 2, seed=k, sampler=LD).cpu().numpy(), ref_hi) for k in seeds]))
    e_st = float(np.mean([mre(sc.render_direct(c, 2, 2, seed=k).cpu().numpy(), ref_hi) for k in seeds]))
    e_ref = mre(ref_ld, ref_hi)
    m_ref, m_ld = float((ref_hi @ LUM).mean()), float((gpu_ld_hi @ LUM).mean())
    print(f"[box LD] MRE vs reference 16x16: reference LD 4 spp {e_ref:.4f}, GPU LD 4 spp {e_ld:.4f}, "
          f"GPU stratified 2x2 {e_st:.4f}; mean luminance ref {m_ref:.5f} GPU LD 256 spp {m_ld:.5f}")
    assert np.isfinite(gpu_ld).all() and (gpu_ld >= 0).all()
    assert e_ld <= 1.25 * e_ref + 0.005
    assert e_ld <= 0.92 * e_st
    assert abs(m_ld / m_ref - 1.0) <= 0.01
    # the same seed renders the same image; another seed, another scramble
    again = sc.render_direct(c, 2, 2, seed=21, sampler=LD).cpu().numpy()
    other = sc.render_direct(c, 2, 2, seed=23, sampler=LD).cpu().numpy()
    assert np.array_equal(again, gpu_ld) and not np.array_equal(other, gpu_ld)


def test_ld_sampler_rounds_counts_to_powers_of_two(gpu):
    """LDSampler(n) takes the next power of two samples per pixel, and the
    light-sample count is rounded the same way (Sampler::AddSamplesSequence*):
    3 x 1, 4 x 1 and 2 x 2 are all 4 samples; 3 light samples are 4."""
    from skwarka_gb300.render import LD
    prims, mats, cam = scenes.direct_lighting_box()
    sc = RenderScene(prims, mats)
    c = cam(16, 16)
    a = sc.render_direct(c, 3, 1, seed=5, sampler=LD).cpu().numpy()
    b = sc.render_direct(c, 4, 1, seed=5, sampler=LD).cpu().numpy()
    d = sc.render_direct(c, 2, 2, seed=5, sampler=LD).cpu().numpy()
    assert np.array_equal(a, b) and np.array_equal(a, d)
    l3 = sc.render_direct(c, 2, 2, light_samples=3, seed=5, sampler=LD).cpu().numpy()
    l4 = sc.render_direct(c, 2, 2, light_samples=4, seed=5, sampler=LD).cpu().numpy()
    assert np.array_equal(l3, l4)
