"""Generates tests/golden/*.npz from the reference's own code
(oracle/_ref/libskw_ref.so, built from the reference sources by
oracle/build_ref.py).  Run from the repository root:

    python tests/golden/make_golden.py

The fixtures hold inputs and the reference's answers; the tests check the
oracle and the CUDA path against them without needing the reference."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from oracle import build_ref  # noqa: E402
from oracle.api import Reference  # noqa: E402
from skwarka_gb300 import scenes  # noqa: E402
import scene_fixtures as sf  # noqa: E402

OUT = Path(__file__).resolve().parent


def accel_golden():
    meshes = scenes.ray_query_scene(sphere_subdivisions=4, n_random=300, seed=21)
    lo, hi = scenes.scene_bounds(meshes)
    rays = scenes.uniform_rays(3000, lo, hi, seed=22)
    srays = scenes.uniform_rays(3000, lo, hi, seed=23, tmax_range=(0.0, 2.0))
    ref = Reference()
    ra = ref.accel(meshes)
    h = ra.intersect(rays, threads=1)
    occ = ra.intersect_test(srays, threads=1)
    bbox, info, tp, ti = ra.export()
    arrays = {"rays": rays, "shadow_rays": srays, "hit_prim": h["prim"], "hit_tri": h["tri"], "hit_t": h["t"],
              "occluded": occ, "node_bbox": bbox, "node_info": info, "tri_prim": tp, "tri_index": ti}
    for i, (v, t) in enumerate(meshes):
        arrays[f"mesh{i}_vertices"] = v
        arrays[f"mesh{i}_triangles"] = t
    np.savez_compressed(OUT / "accel_small.npz", **arrays)


def knn_golden():
    rng = np.random.default_rng(31)
    n = 4000
    pos = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    pos[:100] = pos[100:200]  # duplicated points, as in the reference's KDTree test
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ref = Reference()
    nids = np.array([ref.lib.skw_ref_compress_direction(*v) for v in nrm], np.uint16)
    kd = ref.kdtree(pos, nids)
    q = rng.uniform(0, 1, size=(500, 3))
    qn = rng.normal(size=(500, 3))
    qn /= np.linalg.norm(qn, axis=1, keepdims=True)
    res_f = kd.knn(q, qn, 20, 0.15, 0.5, threads=1)
    res_u = kd.knn(q, None, 20, 0.2, -1.0, threads=1)
    np.savez_compressed(OUT / "knn_small.npz", pos=pos, normal_ids=nids, perm=kd.perm, nodes=kd.nodes, q=q, qn=qn,
                        filt_idx=res_f["idx"], filt_d2=res_f["d2"], filt_count=res_f["count"],
                        all_idx=res_u["idx"], all_d2=res_u["d2"], all_count=res_u["count"])


def direction_golden():
    tab = Reference().direction_table()
    sample = np.arange(0, 1 << 16, 97)
    np.savez_compressed(OUT / "compressed_direction.npz", ids=sample, vectors=tab[sample])


if __name__ == "__main__" and len(sys.argv) == 1:
    if build_ref.build() is None:
        sys.exit("the reference sources are needed to generate the golden fixtures")
    accel_golden()
    knn_golden()
    direction_golden()
    print("golden fixtures written to", OUT)


def render_golden():
    """Reference renders of the plain direct-lighting box at 64 x 64: 2x2 spp
    (the noise level at the configuration's sample count) and 16x16 spp (the
    comparison image)."""
    from skwarka_gb300 import scenes
    prims, mats, cam = scenes.direct_lighting_box()
    c = cam(64, 64)
    ref = Reference()
    lo, _ = ref.render_direct(prims, mats, [], c, 2, 2)
    hi, _ = ref.render_direct(prims, mats, [], c, 16, 16)
    np.savez_compressed(OUT / "direct_box_64.npz", ref_2x2=lo, ref_16x16=hi)
    # One plane per BSDF under an area light and under a point light, 16x16 spp.
    planes = {}
    for name, (p, m, pl, c) in sf.material_plane_scenes().items():
        planes[name], _ = ref.render_direct(p, m, pl, c, 16, 16)
    np.savez_compressed(OUT / "direct_planes.npz", **planes)


def measured_golden():
    """The reference's renders of a plane with the synthetic measured BRDF
    (scenes.merl_table) under an area light and a point light, 16x16 spp."""
    from skwarka_gb300.render import MeasuredBRDF
    ref = Reference()
    m = MeasuredBRDF(scenes.merl_table(), device=False)
    out = {}
    for name, (p, mats, l, c) in sf.measured_plane_scenes(m).items():
        out[name], _ = ref.render_direct(p, mats, l, c, 16, 16)
    np.savez_compressed(OUT / "measured_planes.npz", **out)


def two_lights_golden():
    """The reference's render of the box with two area lights, 32 x 32,
    16x16 spp (its IrradianceLightsSamplingStrategy chooses the light)."""
    p, m, c = sf.two_light_scene()
    img, _ = Reference().render_direct(p, m, [], c, 16, 16)
    np.savez_compressed(OUT / "two_lights_32.npz", ref=img)


def medium_golden():
    """The reference's direct-lighting renders with a homogeneous medium
    (scene_fixtures.medium_cases) at 32 x 32, 16x16 spp."""
    ref = Reference()
    out = {}
    for name, (p, m, l, c, med) in sf.medium_cases().items():
        out[name], _ = ref.render_direct(p, m, l, c, 16, 16, 1, medium=med)
    np.savez_compressed(OUT / "medium_32.npz", **out)


def photon_golden():
    """The reference's irradiance photon map (_ConstructIrradiancePhotonMap)
    over the seeded synthetic photon maps of scene_fixtures.synthetic_photon_maps."""
    maps, paths, area = sf.synthetic_photon_maps()
    pos, ext, intr, nrm, md = Reference().photon_irradiance(maps, paths, area)
    np.savez_compressed(OUT / "photon_irradiance.npz", pos=pos, ext=ext, int=intr, nrm=nrm, max_dist=np.float64(md))
    # Photon-mapping render of the direct-lighting box: 200,000 photon paths,
    # 16 gather samples, 64 x 64 at 4x4 spp; and its direct-lighting part.
    prims, mats, cam = scenes.direct_lighting_box()
    c = cam(64, 64)
    ref = Reference()
    photon, info = ref.render_photon(prims, mats, [], c, 4, 4, 200_000, gather_samples=16)
    direct, _ = ref.render_direct(prims, mats, [], c, 4, 4)
    np.savez_compressed(OUT / "photon_box_64.npz", photon=photon, direct=direct,
                        counts=np.array([info["caustic"], info["direct"], info["indirect"], info["irradiance"]]))


def caustic_golden():
    """The reference's photon-mapping render (gather and indirect maps
    empty, so direct lighting + _LookupCausticRadiance) of each
    scene_fixtures.caustic_cases() case with its seeded caustic map, at 16x16
    samples per pixel."""
    out = {}
    ref = Reference()
    for name, (prims, mats, lights, cam, maps, paths, k, r) in sf.caustic_cases().items():
        film, info = ref.render_photon_maps(prims, mats, lights, cam, 16, 16, maps, paths, gather_samples=4,
                                            caustic_lookup=k, max_caustic_dist=r)
        assert info["caustic"] == len(maps[0]) and info["irradiance"] == 0, info
        out[name] = film
        direct, _ = ref.render_direct(prims, mats, lights, cam, 16, 16)
        out[name + "_direct"] = direct
    np.savez_compressed(OUT / "caustic_32.npz", **out)


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "caustic":
    caustic_golden()
    print("caustic golden written")

if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "measured":
    measured_golden()
    print("measured golden written")

if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "lights":
    two_lights_golden()
    print("two-light golden written")

if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "medium":
    medium_golden()
    print("medium golden written")

if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "photon":
    photon_golden()
    print("photon golden written")

if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "render":
    render_golden()
    print("render golden written")


def specular_golden():
    """The reference's direct-lighting renders (maximum specular depth 6) of
    scene_fixtures.specular_cases() at 48 x 32, 16x16 spp, and its photon
    shooting (ShootPhotons, 2,000,000 paths, its own bounce and roulette rules)
    in the clear-glass sphere scene under the point light: the sizes of its
    caustic, direct and indirect maps, the indirect photons on the floor, and
    the caustic photons' mean (x, y) and RMS distance from the axis; and its
    photon-mapping renders of the clear-glass scenes."""
    out = {}
    ref = Reference()
    for name, (prims, mats, lights, cam) in sf.specular_cases().items():
        out[name], _ = ref.render_direct(prims, mats, lights, cam, 16, 16)
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    caustic, direct, indirect = ref.shoot_photons(prims, mats, lights, 2_000_000)
    on_floor = np.abs(indirect[:, 2]) < 1e-4
    out["photon_counts"] = np.array([len(caustic), len(direct), len(indirect), on_floor.sum()], np.int64)
    out["caustic_xy"] = np.concatenate([caustic[:, :2].mean(0), [np.sqrt((caustic[:, :2] ** 2).sum(1).mean())]])
    # the clear-glass sphere under the point light inside a scattering medium
    from skwarka_gb300.render import Medium
    prims, mats, lights, cam = sf.specular_cases()["glass_point"]
    out["glass_point_medium"], _ = ref.render_direct(prims, mats, lights, cam, 16, 16, 1,
                                                     medium=sf.specular_medium())
    # photon-mapping renders (1,000,000 paths, 16 gather samples, 8x8 spp)
    for name in ("glass_point", "glass_area"):
        prims, mats, lights, cam = sf.specular_cases()[name]
        out[name + "_photon"], _ = ref.render_photon(prims, mats, lights, cam, 8, 8, 1_000_000, gather_samples=16)
    np.savez_compressed(OUT / "specular_48x32.npz", **out)


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "specular":
    specular_golden()


def ld_golden():
    """The reference's direct-lighting render of the box (64 x 64) with its
    LDSampler at 4 samples per pixel (ConsecutiveImagePixelsOrder)."""
    prims, mats, cam = scenes.direct_lighting_box()
    img, _ = Reference().render_direct(prims, mats, [], cam(64, 64), 2, 2, ld=True)
    np.savez_compressed(OUT / "ld_box_64.npz", ref_ld_4=img)


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "ld":
    ld_golden()


def c1_golden():
    """The plain direct-lighting configuration at its own size: the box at
    256 x 256 rendered by the reference's SamplerBasedRenderer with 2x2
    stratified samples (the configuration's 4 spp) and with 16x16 (the
    comparison image, stored as float16).  The 2x2 image itself is not
    stored, only its mean relative error against the 16x16 image, its mean
    luminance and its 8x8-block mean luminances."""
    from skwarka_gb300 import scenes
    prims, mats, cam = scenes.direct_lighting_box()
    c = cam(256, 256)
    ref = Reference()
    lo, t_lo = ref.render_direct(prims, mats, [], c, 2, 2)
    hi, t_hi = ref.render_direct(prims, mats, [], c, 16, 16)
    lum = np.array([0.05316285, 0.58515348, 0.36168367])
    lh, ll = hi @ lum, lo @ lum
    mre = float(np.mean(np.abs(ll - lh) / np.maximum(lh, 1e-3 * lh.mean())))
    blocks = ll.reshape(32, 8, 32, 8).mean(axis=(1, 3)).astype(np.float32)
    np.savez_compressed(OUT / "direct_box_256.npz", ref_16x16=hi.astype(np.float16), ref_2x2_mre=mre,
                        ref_2x2_mean=float(ll.mean()), ref_2x2_blocks=blocks, seconds=np.array([t_lo, t_hi]))
    print(f"c1: reference 2x2 MRE {mre:.4f}; render seconds {t_lo:.2f} / {t_hi:.2f}")


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "c1":
    c1_golden()


def materials_golden():
    """The reference's direct-lighting renders (16x16 spp, maximum specular
    depth 6) of scene_fixtures.material_cases(): SubstrateMaterial,
    UberMaterial and MixMaterial planes under an area light and spheres over
    the floor."""
    ref = Reference()
    out = {}
    for name, (prims, mats, lights, cam) in sf.material_cases().items():
        out[name], _ = ref.render_direct(prims, mats, lights, cam, 16, 16)
        print(f"materials: {name} mean {out[name].mean():.5f}")
    np.savez_compressed(OUT / "materials.npz", **out)


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "materials":
    materials_golden()

