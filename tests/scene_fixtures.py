"""Scenes and ray sets shared by the tests (seeded, small enough for the
oracle to finish in seconds)."""
import numpy as np

from skwarka_gb300 import scenes


def unit_test_spheres():
    """The four tessellated spheres of the reference's accelerator unit test
    (UnitTests/MainTests/Raytracer/Core/TriangleAccelerator.test.h:35-42):
    (center, radius, subdivisions)."""
    spec = [((0, 0, 0), 10.0, 5), ((-20, 0, 0), 20.0, 5), ((0, -10, 0), 0.5, 5), ((1000, 0, 0), 1000.0, 6)]
    meshes = []
    for c, r, n in spec:
        v, t = scenes.sphere_mesh(n)
        meshes.append(((v * r + np.asarray(c, np.float64)).astype(np.float32), t))
    return meshes


def unit_test_rays(meshes, n=1000, seed=11):
    """Random rays like the unit test's: origin uniform in the world bounds,
    direction from U[0,1]^3 normalised, tmin in U[-10, 10], tmax in U[100, 10000]."""
    lo, hi = scenes.scene_bounds(meshes)
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.uniform(0, 1, size=(n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    r = np.zeros((n, 8), np.float32)
    r[:, :3] = o
    r[:, 3:6] = d
    r[:, 6] = rng.uniform(-10, 10, n)
    r[:, 7] = rng.uniform(100, 10000, n)
    return r


def small_query_scene():
    """A 16k-triangle displaced sphere plus 2,000 random triangles."""
    return scenes.ray_query_scene(sphere_subdivisions=6, n_random=2000, seed=5)


def flat_tiles(n=64, seed=2):
    """Axis-aligned coplanar squares (z = 0.5), two triangles each: every node
    above the leaves has zero extent in z, exercising that split path."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(0, 1, size=(n, 2)).astype(np.float32)
    s = np.float32(0.02)
    v = np.zeros((n, 4, 3), np.float32)
    v[:, 0, :2] = xy
    v[:, 1, :2] = xy + [s, 0]
    v[:, 2, :2] = xy + [s, s]
    v[:, 3, :2] = xy + [0, s]
    v[:, :, 2] = 0.5
    t = np.zeros((n, 2, 3), np.int32)
    base = (np.arange(n) * 4)[:, None]
    t[:, 0] = base + [0, 1, 2]
    t[:, 1] = base + [0, 2, 3]
    return [(v.reshape(-1, 3), t.reshape(-1, 3))]


def canonical_leaf_order(info, tri_prim, tri_index):
    """(prim, tri) pairs with each leaf's range sorted.  The reference orders
    its primitives by mesh address before building (a std::map keyed by
    pointer, TriangleAccelerator.cpp:25-38), which only permutes triangles
    inside a leaf; comparisons with it use this canonical order."""
    pairs = np.stack([tri_prim, tri_index], 1).astype(np.int64)
    out = pairs.copy()
    leaves = info[info[:, 0] == 0]
    for b, e in leaves[:, 4:6]:
        seg = pairs[b:e]
        out[b:e] = seg[np.lexsort((seg[:, 1], seg[:, 0]))]
    return out


def material_plane_scenes():
    """One 10 x 10 plane under a 0.6 x 0.6 area light of radiance 10 at height 1
    (and, separately, under a point light of intensity 3), for each BSDF the
    direct-lighting path supports.  Returns {name: (prims, materials,
    point_lights, camera)}; a 24 x 16 camera looks down at the lit region at
    about 35 degrees, so glossy lobes reflect the light."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import METAL, PLASTIC, Camera, Material, PointLight, RenderPrimitive
    s, a = 5.0, 0.6
    plane = TriangleMesh(np.array([[-s, -s, 0], [s, -s, 0], [s, s, 0], [-s, s, 0]], np.float32),
                         np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    light = TriangleMesh(np.array([[-a / 2, -a / 2, 1], [a / 2, -a / 2, 1], [a / 2, a / 2, 1], [-a / 2, a / 2, 1]],
                                  np.float32), np.array([[0, 2, 1], [0, 3, 2]], np.int32))  # emits towards -z
    cam = Camera.look_at((1.2, 0.3, 0.9), (-0.2, 0.0, 0.0), (0, 0, 1), np.radians(50.0), 24, 16)
    copper = dict(eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2))
    mats = {
        "matte": Material(kd=(0.8, 0.6, 0.4)),
        "oren_nayar": Material(kd=(0.8, 0.6, 0.4), sigma=20.0),
        "plastic": Material(kind=PLASTIC, kd=(0.4, 0.3, 0.2), ks=(0.5, 0.5, 0.5), roughness=0.1),
        "plastic_rough": Material(kind=PLASTIC, kd=(0.4, 0.3, 0.2), ks=(0.5, 0.5, 0.5), roughness=0.6),
        "metal": Material(kind=METAL, roughness=0.05, **copper),
        "metal_rough": Material(kind=METAL, roughness=0.5, **copper),
    }
    out = {}
    for name, m in mats.items():
        out["area_" + name] = ([RenderPrimitive(plane, 0), RenderPrimitive(light, 1, emission=(10.0, 10.0, 10.0))],
                               [m, Material(kd=(0.0, 0.0, 0.0))], [], cam)
        out["point_" + name] = ([RenderPrimitive(plane, 0)], [m], [PointLight((0.1, -0.2, 0.8), (3.0, 3.0, 3.0))], cam)
    return out


def _ray_mesh_hit(o, d, v, t):
    """Closest hit of one ray with a triangle mesh (float64 Moller-Trumbore):
    (point, unit geometric normal facing the ray origin)."""
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    e1, e2 = b - a, c - a
    p = np.cross(d, e2)
    det = (e1 * p).sum(1)
    ok = np.abs(det) > 1e-14
    inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
    s = o - a
    u = (s * p).sum(1) * inv
    q = np.cross(s, e1)
    w = (q * d).sum(1) * inv
    tt = (e2 * q).sum(1) * inv
    hit = ok & (u >= 0) & (w >= 0) & (u + w <= 1) & (tt > 0)
    i = int(np.argmin(np.where(hit, tt, np.inf)))
    n = np.cross(e1[i], e2[i])
    n /= np.linalg.norm(n)
    if np.dot(n, d) > 0:
        n = -n
    return o + tt[i] * d, n


def sphere_area_lights_case():
    """Analogue of the reference's DirectLightingIntegrator area-light test
    (UnitTests/MainTests/Raytracer/Core/DirectLightingIntegrator.test.h:104-135):
    unit spheres at the origin (white Lambertian), at (10,0,0) (emitting 10)
    and at (0,10,0) (emitting 20); the point seen from (5,5,0) towards the
    origin.  Its radiance is sum_i L_i/pi * integral of cos over the sphere's
    cone, and for a cone of half-angle beta fully above the horizon that
    integral is pi sin^2(beta) cos(alpha).  Returns (prims, materials, camera,
    expected radiance)."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import Camera, Material, RenderPrimitive
    v, t = scenes.sphere_mesh(6)
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    outward = (np.cross(b - a, c - a) * (a + b + c)).sum(1) > 0
    t = np.where(outward[:, None], t, t[:, [0, 2, 1]]).astype(np.int32)
    centers, radiance = [(0.0, 0.0, 0.0), (10.0, 0.0, 0.0), (0.0, 10.0, 0.0)], [0.0, 10.0, 20.0]
    prims = [RenderPrimitive(TriangleMesh((v + np.asarray(cc)).astype(np.float32), t), 0 if i == 0 else 1,
                             emission=(radiance[i],) * 3) for i, cc in enumerate(centers)]
    mats = [Material(kd=(1.0, 1.0, 1.0)), Material(kd=(0.0, 0.0, 0.0))]
    eye = np.array([5.0, 5.0, 0.0])
    d = -eye / np.linalg.norm(eye)
    p, n = _ray_mesh_hit(eye, d, v.astype(np.float32).astype(np.float64), t)
    want = 0.0
    for cc, le in zip(centers[1:], radiance[1:]):
        to_c = np.asarray(cc) - p
        dist = np.linalg.norm(to_c)
        want += le / np.pi * np.pi * (1.0 / dist) ** 2 * np.dot(n, to_c / dist)
    cam = Camera.look_at(tuple(eye), (0.0, 0.0, 0.0), (0, 0, 1), 1e-5, 2, 2)
    return prims, mats, cam, float(want)


def square_light_case(a=0.6, h=1.0, p=(0.3, 0.2)):
    """A white Lambertian plane z=0 under an a x a square light of radiance 10
    at height h facing down; the point p on the plane is seen by a camera of
    tiny field of view.  The expected radiance rho/pi * E is the irradiance E
    integrated numerically over the light (2000^2 midpoint rule).  Returns
    (prims, materials, camera, expected radiance)."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import Camera, Material, RenderPrimitive
    s = 5.0
    plane = TriangleMesh(np.array([[-s, -s, 0], [s, -s, 0], [s, s, 0], [-s, s, 0]], np.float32),
                         np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    light = TriangleMesh(np.array([[-a / 2, -a / 2, h], [a / 2, -a / 2, h], [a / 2, a / 2, h], [-a / 2, a / 2, h]],
                                  np.float32), np.array([[0, 2, 1], [0, 3, 2]], np.int32))
    prims = [RenderPrimitive(plane, 0), RenderPrimitive(light, 1, emission=(10.0, 10.0, 10.0))]
    mats = [Material(kd=(1.0, 1.0, 1.0)), Material(kd=(0.0, 0.0, 0.0))]
    n = 2000
    xs = (np.arange(n) + 0.5) / n * a - a / 2
    x, y = np.meshgrid(xs - p[0], xs - p[1])
    r2 = x * x + y * y + h * h
    e = 10.0 * (h * h / (r2 * r2)).sum() * (a / n) ** 2
    cam = Camera.look_at((p[0], p[1], 0.5), (p[0], p[1], 0.0), (0, 1, 0), 1e-3, 2, 2)
    return prims, mats, cam, float(e / np.pi)


def synthetic_photon_maps(seed=31, sizes=(400, 5000, 8000), paths=(15000, 15000, 15000)):
    """Photon maps on the inside of the box [-1, 1]^3: every photon on a face
    (positions uniform on it, the face's inward normal), incident directions
    mostly from the inside (1 in 8 from behind, to give internal irradiance),
    weights U[0, 1e-3]^3.  Returns ([caustic, direct, indirect] structured
    arrays, paths, scene area 24)."""
    from skwarka_gb300.kdtree import compress_directions
    from skwarka_gb300.photon import PHOTON_DTYPE
    rng = np.random.default_rng(seed)
    maps = []
    for n in sizes:
        face = rng.integers(0, 6, size=n)
        axis, side = face // 2, np.where(face % 2 == 0, -1.0, 1.0)
        p = rng.uniform(-1.0, 1.0, size=(n, 3))
        p[np.arange(n), axis] = side
        nrm = np.zeros((n, 3))
        nrm[np.arange(n), axis] = -side
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        flip = (d * nrm).sum(1) < 0
        back = rng.uniform(size=n) < 0.125
        d[flip ^ back] *= -1.0
        a = np.zeros(n, PHOTON_DTYPE)
        a["position"] = p.astype(np.float32)
        a["weight"] = rng.uniform(0.0, 1e-3, size=(n, 3)).astype(np.float32)
        a["incident"] = compress_directions(d)
        a["normal"] = compress_directions(nrm)
        maps.append(a)
    return maps, list(paths), 24.0


def photon_box_scene(albedo=0.5, intensity=50.0):
    """A closed box [-1, 1]^3 of matte walls (one albedo) with a point light
    at (0.1, 0.2, 0.3) of the given intensity: every photon path hits a wall,
    and with a grey Lambertian albedo the reference's Russian roulette keeps
    each photon's weight at 4 pi I."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import Material, PointLight, RenderPrimitive
    bv, bt = scenes._box_inward()
    prims = [RenderPrimitive(TriangleMesh(bv, bt), 0)]
    return prims, [Material(kd=(albedo,) * 3)], [PointLight((0.1, 0.2, 0.3), (intensity,) * 3)]


def medium_cases():
    """Homogeneous-medium renders: {name: (prims, materials, point_lights,
    camera, medium)} -- the grey box with a point light filled with a
    scattering medium, the same with an emitting non-scattering medium, and
    the direct-lighting box (area light) with the configuration's medium
    (sigma_a 0.05, sigma_s 0.2, g 0.3)."""
    from skwarka_gb300.render import Camera, Medium
    prims, mats, lights = photon_box_scene(0.5, 5.0)
    cam = Camera.look_at((0.0, 0.0, -0.9), (0.0, 0.0, 1.0), (0, 1, 0), np.radians(70), 32, 32)
    out = {"point_scatter": (prims, mats, lights, cam, Medium(sigma_a=(0.1, 0.05, 0.02), sigma_s=(0.4, 0.3, 0.2),
                                                              g=0.3, step=0.05)),
           "point_emit": (prims, mats, lights, cam, Medium(sigma_a=(0.2, 0.2, 0.2), sigma_s=(0, 0, 0),
                                                           emission=(0.3, 0.2, 0.1), step=0.05))}
    bp, bm, bcam = scenes.direct_lighting_box()
    out["box_area"] = (bp, bm, [], bcam(32, 32), Medium(sigma_a=(0.05,) * 3, sigma_s=(0.2,) * 3, g=0.3, step=0.05))
    out["box_absorb"] = (bp, bm, [], bcam(32, 32), Medium(sigma_a=(0.25,) * 3, sigma_s=(0, 0, 0), g=0.3, step=0.05))
    return out


def measured_plane_scenes(measured):
    """The plane scenes of material_plane_scenes with the measured BRDF
    `measured` (a skwarka_gb300.render.MeasuredBRDF) as the plane's material."""
    from skwarka_gb300.render import MEASURED, Material
    base = material_plane_scenes()
    m = Material(kind=MEASURED, measured=measured)
    out = {}
    for light in ("area", "point"):
        prims, mats, lights, cam = base[light + "_matte"]
        out[light + "_measured"] = (prims, [m] + mats[1:], lights, cam)
    return out


def two_light_scene():
    """The direct-lighting box with a second, smaller and brighter quad light
    on the -x wall facing +x: (prims, materials, camera 32 x 32), for the
    light choice among several area lights."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.render import RenderPrimitive
    prims, mats, cam = scenes.direct_lighting_box()
    lv = np.array([[-0.98, -0.2, -0.1], [-0.98, 0.2, -0.1], [-0.98, 0.2, 0.1], [-0.98, -0.2, 0.1]], np.float32)
    lt = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    a, b, c = lv[lt[0]]
    assert np.cross(b - a, c - a)[0] > 0  # emits towards +x
    prims = prims + [RenderPrimitive(TriangleMesh(lv, lt), 2, emission=(30.0, 20.0, 10.0))]
    return prims, mats, cam(32, 32)


def caustic_cases(seed=41):
    """A 4 x 4 plane (z = 0) under a weak point light, with a seeded caustic
    photon map and empty direct and indirect maps: 30,000 photons on the
    plane, 70 % uniform in a disk of radius 0.6 around the origin and 30 %
    uniform over [-2, 2]^2 (so lookups outside the disk find fewer than k),
    incident directions from the upper hemisphere, weights
    U[0.5, 1.5] x (0.8, 0.6, 0.4), 200,000 caustic paths (the caustic term
    is then about twice the direct lighting).  Cases: matte
    and plastic planes with (k, radius) = (50, 0.1); the matte plane with
    (200, 0.05), whose k-NN heaps live in global scratch.  Returns {name:
    (prims, materials, lights, camera, maps, paths, k, radius)}; a 32 x 32
    camera looks down at the disk at about 25 degrees from the normal."""
    from skwarka_gb300.accel import TriangleMesh
    from skwarka_gb300.kdtree import compress_directions
    from skwarka_gb300.photon import PHOTON_DTYPE
    from skwarka_gb300.render import PLASTIC, Camera, Material, PointLight, RenderPrimitive
    rng = np.random.default_rng(seed)
    n = 30_000
    n_disk = int(0.7 * n)
    r = 0.6 * np.sqrt(rng.uniform(size=n_disk))
    a = rng.uniform(0.0, 2.0 * np.pi, size=n_disk)
    pos = np.zeros((n, 3))
    pos[:n_disk, 0], pos[:n_disk, 1] = r * np.cos(a), r * np.sin(a)
    pos[n_disk:, :2] = rng.uniform(-2.0, 2.0, size=(n - n_disk, 2))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:, 2] = np.abs(d[:, 2])
    caustic = np.zeros(n, PHOTON_DTYPE)
    caustic["position"] = pos.astype(np.float32)
    caustic["weight"] = (rng.uniform(0.5, 1.5, size=(n, 1)) * np.array([0.8, 0.6, 0.4])).astype(np.float32)
    caustic["incident"] = compress_directions(d)
    caustic["normal"] = compress_directions(np.tile([0.0, 0.0, 1.0], (n, 1)))
    empty = np.zeros(0, PHOTON_DTYPE)
    maps, paths = [caustic, empty, empty], [200_000, 0, 0]
    s = 2.0
    plane = TriangleMesh(np.array([[-s, -s, 0], [s, -s, 0], [s, s, 0], [-s, s, 0]], np.float32),
                         np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    cam = Camera.look_at((0.0, -0.6, 1.4), (0.0, 0.0, 0.0), (0, 1, 0), np.radians(60.0), 32, 32)
    lights = [PointLight((0.3, 0.2, 2.0), (0.05, 0.05, 0.05))]
    matte = Material(kd=(0.7, 0.6, 0.5))
    plastic = Material(kind=PLASTIC, kd=(0.4, 0.3, 0.2), ks=(0.5, 0.5, 0.5), roughness=0.1)
    return {"matte_k50": ([RenderPrimitive(plane, 0)], [matte], lights, cam, maps, paths, 50, 0.1),
            "plastic_k50": ([RenderPrimitive(plane, 0)], [plastic], lights, cam, maps, paths, 50, 0.1),
            "matte_k200": ([RenderPrimitive(plane, 0)], [matte], lights, cam, maps, paths, 200, 0.05)}


def specular_scene(material, lights="area", resolution=(48, 32)):
    """skwarka_gb300.scenes.glass_sphere_scene: a sphere of `material` above a
    matte floor under an area light ("area") or a point light ("point")."""
    return scenes.glass_sphere_scene(material, lights, resolution)


def specular_cases():
    """{name: (prims, materials, point_lights, camera)} of specular_scene:
    clear glass (r = t = 1, index 1.5) under the area light and under the
    point light, tinted glass (t = (0.9, 0.6, 0.3), index 1.33), and a
    reflection-only dielectric of index 8 (a Fresnel mirror, r = (0.9, 0.8,
    0.7))."""
    from skwarka_gb300.render import TRANSPARENT, Material
    glass = Material(kind=TRANSPARENT, kd=(1.0, 1.0, 1.0), ks=(1.0, 1.0, 1.0), refractive_index=1.5)
    tinted = Material(kind=TRANSPARENT, kd=(1.0, 1.0, 1.0), ks=(0.9, 0.6, 0.3), refractive_index=1.33)
    mirror = Material(kind=TRANSPARENT, kd=(0.9, 0.8, 0.7), ks=(0.0, 0.0, 0.0), refractive_index=8.0)
    return {"glass_area": specular_scene(glass, "area"),
            "glass_point": specular_scene(glass, "point"),
            "tinted_area": specular_scene(tinted, "area"),
            "mirror_area": specular_scene(mirror, "area")}


def specular_medium():
    """A scattering, absorbing medium around the glass sphere and the lit
    floor (box [-1.5, 1.5]^2 x [0, 1.3], sigma_a 0.1, sigma_s 0.3, HG g 0.3,
    march step 0.05)."""
    from skwarka_gb300.render import Medium
    return Medium(lo=(-1.5, -1.5, 0.0), hi=(1.5, 1.5, 1.3), sigma_a=(0.1, 0.1, 0.1), sigma_s=(0.3, 0.3, 0.3),
                  g=0.3, step=0.05)


def material_cases():
    """{name: (prims, materials, point_lights, camera)} for SubstrateMaterial,
    UberMaterial and MixMaterial: the plane of material_plane_scenes() under
    its area light with a substrate (smooth and rough), an opaque uber with a
    specular reflection (the light's mirror image in the plane), and a mix of
    matte and plastic; and the sphere of specular_scene() as a half-opaque
    uber (its specular transmission, reflection, diffuse and glossy parts)
    and as a mix of clear glass and matte; and the two-roughness substrate
    on the plane (no uvs, and uvs) and on the sphere (vertex tangents)."""
    from skwarka_gb300.render import MATTE, MIX, PLASTIC, SUBSTRATE, TRANSPARENT, UBER, Material
    planes = material_plane_scenes()
    prims, mats, pls, cam = planes["area_matte"]
    out = {}
    plane_mats = {
        "substrate": [Material(kind=SUBSTRATE, kd=(0.6, 0.45, 0.3), ks=(0.25, 0.25, 0.25), roughness=0.1)],
        "substrate_rough": [Material(kind=SUBSTRATE, kd=(0.6, 0.45, 0.3), ks=(0.25, 0.25, 0.25), roughness=0.5)],
        "uber_opaque": [Material(kind=UBER, kd=(0.4, 0.3, 0.2), ks=(0.3, 0.3, 0.3), kr=(0.2, 0.2, 0.2),
                                 roughness=0.1, refractive_index=1.5)],
        "mix_matte_plastic": [Material(kind=MIX, mix=(1, 2), mix_scale=(0.3, 0.5, 0.7)),
                              Material(kind=MATTE, kd=(0.8, 0.6, 0.4)),
                              Material(kind=PLASTIC, kd=(0.2, 0.3, 0.5), ks=(0.5, 0.5, 0.5), roughness=0.1)],
    }
    for name, ms in plane_mats.items():
        # the plane takes material 0; the light's black matte goes last
        out["plane_" + name] = ([prims[0].__class__(prims[0].mesh, 0), prims[1].__class__(
            prims[1].mesh, len(ms), emission=prims[1].emission)], ms + [Material(kd=(0.0, 0.0, 0.0))], pls, cam)
    uber = Material(kind=UBER, kd=(0.3, 0.3, 0.3), ks=(0.2, 0.2, 0.2), kr=(0.3, 0.3, 0.3), roughness=0.2,
                    opacity=(0.5, 0.6, 0.7), refractive_index=1.5)
    out["sphere_uber"] = specular_scene(uber, "area")
    glass = Material(kind=TRANSPARENT, kd=(1.0, 1.0, 1.0), ks=(1.0, 1.0, 1.0), refractive_index=1.5)
    sp, sm, sl, sc = specular_scene(glass, "area")
    # the sphere (material 1) becomes a mix of glass (appended) and a matte
    n = len(sm)
    mix = Material(kind=MIX, mix=(n, n + 1), mix_scale=(0.6, 0.6, 0.6))
    out["sphere_mix_glass_matte"] = (sp, [sm[0], mix] + list(sm[2:]) + [glass, Material(kd=(0.7, 0.2, 0.2))], sl, sc)
    # the two-roughness substrate (AnisotropicDistribution) under each source
    # of the shading tangent: CoordinateSystem of the normal (the plane
    # without uvs), triangle uvs (the plane, u along a diagonal), and vertex
    # tangents (the sphere, Sphere::BuildMesh's (0, 0, 1) x v)
    aniso = Material(kind=SUBSTRATE, kd=(0.5, 0.4, 0.3), ks=(0.3, 0.3, 0.3), roughness=0.04, v_roughness=0.6)
    out["plane_substrate_aniso"] = ([prims[0].__class__(prims[0].mesh, 0), prims[1].__class__(
        prims[1].mesh, 1, emission=prims[1].emission)], [aniso, Material(kd=(0.0, 0.0, 0.0))], pls, cam)
    uv = np.array([[0.0, 0.0, 0.7, 0.7, 0.0, 1.0]] * len(prims[0].mesh.triangles), np.float32)
    out["plane_substrate_aniso_uv"] = ([prims[0].__class__(prims[0].mesh, 0, triangle_uvs=uv), prims[1].__class__(
        prims[1].mesh, 1, emission=prims[1].emission)], [aniso, Material(kd=(0.0, 0.0, 0.0))], pls, cam)
    ap, am, al, ac = specular_scene(aniso, "area")
    sv = (ap[1].mesh.vertices.astype(np.float64) - [0.0, 0.0, 0.45]) / 0.4
    tan = np.cross(np.array([0.0, 0.0, 1.0]), sv)
    ln = np.linalg.norm(tan, axis=1)
    tan = np.where(ln[:, None] > 0, tan / np.maximum(ln, 1e-300)[:, None], [1.0, 0.0, 0.0])
    ap = [ap[0], ap[1].__class__(ap[1].mesh, 1, vertex_tangents=tan.astype(np.float32))] + list(ap[2:])
    out["sphere_substrate_aniso"] = (ap, am, al, ac)
    return out

