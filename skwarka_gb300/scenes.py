"""Seeded synthetic scenes and ray sets for the benchmarks and parity tests.

The same arrays feed the CUDA path and the CPU oracle, so both see identical
float32 geometry and rays.

* ``sphere_mesh(n)`` -- the reference's tessellated sphere
  (Shapes/Sphere.cpp:42-197): a tetrahedron whose triangles are split 4-way
  ``n`` times, edge midpoints pushed to the unit sphere, 4 * 4**n triangles.
  Vertex and triangle order follow the reference: new vertices in order of
  first use, each triangle replaced by its four children in place.
* ``displaced_sphere`` -- that sphere with a seeded radial gradient-noise
  displacement (the ray-query workload: n = 9 gives 1,048,576 triangles).
* ``random_triangles`` -- small triangles with uniform centroids.
* ``uniform_rays`` -- origins uniform in a box, directions uniform on S^2.
"""
from __future__ import annotations

import math

import numpy as np


def sphere_mesh(subdivisions: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit sphere: (float64 (nv, 3) vertices, int32 (4*4**n, 3) triangles)."""
    base = math.sqrt(8.0) / 3.0
    c, s = math.cos(2.0 * math.pi / 3.0), math.sin(2.0 * math.pi / 3.0)
    verts = [np.array([[0.0, 0.0, 1.0], [base, 0.0, -1.0 / 3.0], [base * c, base * s, -1.0 / 3.0],
                       [base * c, -base * s, -1.0 / 3.0]])]
    nv = 4
    tris = np.array([[1, 3, 2], [1, 0, 3], [1, 2, 0], [0, 2, 3]], dtype=np.int64)
    allv = verts[0]
    for _ in range(subdivisions):
        m = tris.shape[0]
        a = tris[:, [0, 1, 2]].reshape(-1)
        b = tris[:, [1, 2, 0]].reshape(-1)
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo * (1 << 32) + hi
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")          # unique edges by first use
        rank = np.empty_like(order)
        rank[order] = np.arange(order.size)
        mid_index = nv + rank[inv.reshape(-1)]             # new vertex id per (tri, edge)
        ea, eb = a[first[order]], b[first[order]]
        mid = (allv[ea] + allv[eb]) * 0.5
        length = np.sqrt(mid[:, 0] * mid[:, 0] + mid[:, 1] * mid[:, 1] + mid[:, 2] * mid[:, 2])
        mid = mid * (1.0 / length)[:, None]
        allv = np.concatenate([allv, mid])
        nv += mid.shape[0]
        mi = mid_index.reshape(m, 3)  # (m01, m12, m20)
        i0, i1, i2 = tris[:, 0], tris[:, 1], tris[:, 2]
        m01, m12, m20 = mi[:, 0], mi[:, 1], mi[:, 2]
        tris = np.stack([
            np.stack([i0, m01, m20], 1), np.stack([i1, m12, m01], 1),
            np.stack([i2, m20, m12], 1), np.stack([m01, m12, m20], 1)], 1).reshape(-1, 3)
    return allv, tris.astype(np.int32)


def _gradient_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3-D gradient (Perlin-style) noise in about [-1, 1]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm])
    g = rng.normal(size=(256, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    pi &= 255

    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    u, v, w = fade(pf[:, 0]), fade(pf[:, 1]), fade(pf[:, 2])
    out = np.zeros(p.shape[0])
    acc = {}
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                h = perm[perm[perm[pi[:, 0] + dx] + pi[:, 1] + dy] + pi[:, 2] + dz]
                d = pf - np.array([dx, dy, dz], dtype=np.float64)
                acc[(dx, dy, dz)] = np.einsum("ij,ij->i", g[h], d)
    x00 = acc[(0, 0, 0)] * (1 - u) + acc[(1, 0, 0)] * u
    x10 = acc[(0, 1, 0)] * (1 - u) + acc[(1, 1, 0)] * u
    x01 = acc[(0, 0, 1)] * (1 - u) + acc[(1, 0, 1)] * u
    x11 = acc[(0, 1, 1)] * (1 - u) + acc[(1, 1, 1)] * u
    y0 = x00 * (1 - v) + x10 * v
    y1 = x01 * (1 - v) + x11 * v
    out = y0 * (1 - w) + y1 * w
    return np.clip(out * 1.8, -1.0, 1.0)


def displaced_sphere(subdivisions: int = 9, radius: float = 1.0, amplitude: float = 0.05, frequency: float = 4.0,
                     seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Sphere of the given radius with radial displacement amplitude*noise."""
    v, t = sphere_mesh(subdivisions)
    n = _gradient_noise(v * frequency + 17.0, seed)
    r = radius * (1.0 + amplitude * n)
    return (v * r[:, None]).astype(np.float32), t


def random_triangles(n: int = 50_000, edge: float = 0.01, lo: float = 0.0, hi: float = 1.0,
                     seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """n independent triangles with centroids uniform in [lo, hi]^3 and mean edge ~ `edge`."""
    rng = np.random.default_rng(seed + 1000)
    c = rng.uniform(lo, hi, size=(n, 1, 3))
    u = rng.normal(size=(n, 3, 3))
    u /= np.linalg.norm(u, axis=2, keepdims=True)
    v = (c + u * (edge * 0.75)).astype(np.float32).reshape(-1, 3)
    t = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return v, t


def uniform_rays(n: int, lo, hi, seed: int, tmax_range: tuple[float, float] | None = None) -> np.ndarray:
    """(n, 8) float32 rays: origin uniform in [lo, hi], direction uniform on
    S^2 (normalised in double, then rounded), tmin = 0, tmax = inf or
    uniform in tmax_range."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3:6] = d
    r[:, 6] = 0.0
    if tmax_range is None:
        r[:, 7] = np.inf
    else:
        r[:, 7] = rng.uniform(tmax_range[0], tmax_range[1], size=n)
    return r


def ray_query_scene(sphere_subdivisions: int = 9, n_random: int = 50_000, seed: int = 3):
    """Displaced unit sphere (4*4**n triangles) plus `n_random` small random
    triangles in the unit cube: list of (vertices float32, triangles int32)."""
    sv, st = displaced_sphere(sphere_subdivisions, 1.0, 0.05, 4.0, seed)
    meshes = [(sv, st)]
    if n_random:
        meshes.append(random_triangles(n_random, 0.01, 0.0, 1.0, seed))
    return meshes


def scene_bounds(meshes) -> tuple[np.ndarray, np.ndarray]:
    lo = np.min([v.min(0) for v, _ in meshes], axis=0)
    hi = np.max([v.max(0) for v, _ in meshes], axis=0)
    return lo.astype(np.float64), hi.astype(np.float64)


# ------------------------------------------------------------ render scenes --

def _box_inward(lo=-1.0, hi=1.0):
    """Closed axis-aligned box of 12 triangles whose geometric normals
    ((v1 - v0) x (v2 - v0)) point into the box."""
    c = np.array([[x, y, z] for x in (lo, hi) for y in (lo, hi) for z in (lo, hi)], np.float32)
    idx = lambda x, y, z: x * 4 + y * 2 + z  # noqa: E731
    faces = [  # quad corners; the normal noted is the inward one
        [idx(0, 0, 0), idx(0, 0, 1), idx(0, 1, 1), idx(0, 1, 0)],  # x = lo, normal +x
        [idx(1, 0, 0), idx(1, 1, 0), idx(1, 1, 1), idx(1, 0, 1)],  # x = hi, normal -x
        [idx(0, 0, 0), idx(1, 0, 0), idx(1, 0, 1), idx(0, 0, 1)],  # y = lo, normal +y
        [idx(0, 1, 0), idx(0, 1, 1), idx(1, 1, 1), idx(1, 1, 0)],  # y = hi, normal -y
        [idx(0, 0, 0), idx(0, 1, 0), idx(1, 1, 0), idx(1, 0, 0)],  # z = lo, normal +z
        [idx(0, 0, 1), idx(1, 0, 1), idx(1, 1, 1), idx(0, 1, 1)],  # z = hi, normal -z
    ]
    tris = []
    for a, b, cc, d in faces:  # listed outward-facing; reversed to face inward
        tris += [[a, cc, b], [a, d, cc]]
    return c, np.array(tris, np.int32)


def _jittered_sphere(subdivisions, center, radius, rng, jitter=0.01):
    v, t = sphere_mesh(subdivisions)
    r = radius * (1.0 + rng.uniform(-jitter, jitter, size=(v.shape[0], 1)))
    return (v * r + np.asarray(center)).astype(np.float32), t, v.astype(np.float32)


def direct_lighting_box(seed: int = 1, sphere_subdivisions=(6, 5)):
    """The plain direct-lighting configuration: a closed box of 12 triangles
    (matte walls, per-wall albedo uniform in [0.2, 0.8], seed+1), two
    tessellated spheres (4*4^6 + 4*4^5 = 20,480 triangles, radius jittered by
    +-1 %, plastic Kd 0.5 Ks 0.3 roughness 0.1, shading normals from the
    sphere), and a 2-triangle quad area light of radiance 10 under the
    ceiling.  Returns (prims, materials, camera-at(width, height) factory)."""
    from .accel import TriangleMesh
    from .render import Camera, Material, PLASTIC, RenderPrimitive
    rng = np.random.default_rng(seed)
    arng = np.random.default_rng(seed + 1)
    bv, bt = _box_inward()
    wall = arng.uniform(0.2, 0.8, size=(6, 3)).astype(np.float32)
    albedo = np.repeat(wall, 2, axis=0)
    s1v, s1t, s1n = _jittered_sphere(sphere_subdivisions[0], (-0.35, -0.6, 0.25), 0.38, rng)
    s2v, s2t, s2n = _jittered_sphere(sphere_subdivisions[1], (0.45, -0.68, -0.2), 0.3, rng)
    lv = np.array([[-0.3, 0.98, -0.3], [0.3, 0.98, -0.3], [0.3, 0.98, 0.3], [-0.3, 0.98, 0.3]], np.float32)
    lt = np.array([[0, 1, 2], [0, 2, 3]], np.int32)  # normal (v1-v0)x(v2-v0) = -y: emits downwards
    materials = [Material(kd=(0.5, 0.5, 0.5)),  # walls (per-triangle albedo overrides kd)
                 Material(kind=PLASTIC, kd=(0.5, 0.5, 0.5), ks=(0.3, 0.3, 0.3), roughness=0.1),
                 Material(kd=(0.0, 0.0, 0.0))]   # the light's own surface
    prims = [RenderPrimitive(TriangleMesh(bv, bt), 0, triangle_albedo=albedo),
             RenderPrimitive(TriangleMesh(s1v, s1t), 1, vertex_normals=s1n),
             RenderPrimitive(TriangleMesh(s2v, s2t), 1, vertex_normals=s2n),
             RenderPrimitive(TriangleMesh(lv, lt), 2, emission=(10.0, 10.0, 10.0))]

    def camera(width=256, height=256):
        return Camera.look_at((0.0, 0.1, -0.95), (0.0, -0.3, 1.0), (0.0, 1.0, 0.0), np.radians(75.0), width, height)

    return prims, materials, camera


def batching_scene(seed: int = 4, levels=(6,) * 12 + (3,) * 20, with_light: bool = True):
    """The 200k-triangle procedural scene: the 12-triangle box, 32 spheres
    (12 of 4*4^6 and 20 of 4*4^3 triangles = 201,728 + 12) of radius
    U[0.05, 0.2] at random positions inside the box, each matte, plastic or
    metal (seeded), shading normals from the sphere, per-wall matte albedo
    U[0.2, 0.8], and the box's quad light of radiance 10 under the ceiling.
    Returns (prims, materials)."""
    from .accel import TriangleMesh
    from .render import METAL, PLASTIC, Material, RenderPrimitive
    rng = np.random.default_rng(seed)
    bv, bt = _box_inward()
    wall = rng.uniform(0.2, 0.8, size=(6, 3)).astype(np.float32)
    materials = [Material(kd=(0.5, 0.5, 0.5)),                                             # 0 walls
                 Material(kd=(0.0, 0.0, 0.0)),                                             # 1 light surface
                 Material(kd=(0.7, 0.5, 0.3)),                                             # 2 matte
                 Material(kind=PLASTIC, kd=(0.3, 0.4, 0.6), ks=(0.4, 0.4, 0.4), roughness=0.15),  # 3 plastic
                 Material(kind=METAL, eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2), roughness=0.2)]   # 4 metal
    prims = [RenderPrimitive(TriangleMesh(bv, bt), 0, triangle_albedo=np.repeat(wall, 2, axis=0))]
    for lvl in levels:
        r = float(rng.uniform(0.05, 0.2))
        c = rng.uniform(-0.75, 0.75, size=3)
        v, t, n = _jittered_sphere(lvl, c, r, rng)
        prims.append(RenderPrimitive(TriangleMesh(v, t), int(rng.integers(2, 5)), vertex_normals=n))
    if with_light:
        lv = np.array([[-0.3, 0.98, -0.3], [0.3, 0.98, -0.3], [0.3, 0.98, 0.3], [-0.3, 0.98, 0.3]], np.float32)
        lt = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
        prims.append(RenderPrimitive(TriangleMesh(lv, lt), 1, emission=(10.0, 10.0, 10.0)))
    return prims, materials


def batching_views(n: int = 64, seed: int = 5, lo: int = 64, hi: int = 1024):
    """n cameras inside the box looking at random points, with square films
    whose side is log-uniform in [lo, hi] and a field of view in [40, 90]
    degrees."""
    from .render import Camera
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(n):
        side = int(round(lo * (hi / lo) ** rng.uniform()))
        eye = rng.uniform(-0.85, 0.85, size=3)
        eye[1] = rng.uniform(-0.2, 0.8)
        target = rng.uniform(-0.9, 0.9, size=3)
        target[1] = rng.uniform(-1.0, 0.2)
        fov = np.radians(rng.uniform(40.0, 90.0))
        cams.append(Camera.look_at(tuple(eye), tuple(target), (0.0, 1.0, 0.0), float(fov), side, side))
    return cams


def photon_scene(sphere_subdivisions: int = 9, n_random: int = 50_000, seed: int = 3, albedo: float = 0.6,
                 intensity: float = 50.0, light=(1.2, 0.9, 0.7)):
    """The photon-mapping configuration: the ray-query scene (1M-triangle
    displaced sphere + 50k random triangles) with matte albedo 0.6 and a
    point light of intensity 50 outside the sphere.  Returns (prims,
    materials, point_lights, camera(width, height) factory)."""
    from .accel import TriangleMesh
    from .render import Camera, Material, PointLight, RenderPrimitive
    meshes = ray_query_scene(sphere_subdivisions, n_random, seed)
    prims = [RenderPrimitive(TriangleMesh(v, t), 0) for v, t in meshes]

    def camera(width=512, height=512):
        return Camera.look_at((2.2, 1.8, 1.6), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), np.radians(38.0), width, height)

    return prims, [Material(kd=(albedo,) * 3)], [PointLight(tuple(light), (intensity,) * 3)], camera


def camera_rays(camera, spp_x: int, spp_y: int, seed: int = 0) -> np.ndarray:
    """Stratified, jittered pinhole rays of a Camera (PerspectiveCamera
    convention, as the renderer's): float32 (h * w * spp, 8), pixel-major."""
    rng = np.random.default_rng(seed)
    w, h = camera.width, camera.height
    spp = spp_x * spp_y
    j = np.arange(spp)
    px = np.arange(w * h)
    x, y = (px % w)[:, None], (px // w)[:, None]
    ix = x + ((j % spp_x)[None, :] + rng.uniform(size=(w * h, spp))) / spp_x
    iy = y + ((j // spp_x)[None, :] + rng.uniform(size=(w * h, spp))) / spp_y
    xt = np.tan(camera.x_view_angle / 2.0)
    yt = xt * h / w
    cx = (2.0 * xt * (ix - w * 0.5) / w).reshape(-1)
    cy = (2.0 * yt * (iy - h * 0.5) / h).reshape(-1)
    m = np.asarray(camera.camera_to_world, np.float64).reshape(4, 4)
    d = np.stack([cx, cy, np.ones_like(cx)], 1) @ m[:3, :3].T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((d.shape[0], 8), np.float32)
    r[:, :3] = m[:3, 3]
    r[:, 3:6] = d
    r[:, 7] = np.inf
    return r


def merl_table(seed: int = 7, kd=(0.35, 0.25, 0.15), ks=(0.5, 0.5, 0.5), exponent: float = 40.0,
               noise: float = 0.02) -> bytes:
    """A measured-style BRDF in the MERL binary layout (3 int32 dims, then 3
    channels of 90 x 90 x 180 doubles, stored divided by the loader's channel
    scales 1/1500, 1.15/1500, 1.66/1500): a seeded microfacet formula --
    Lambertian kd plus a normalised Blinn lobe in the half-vector angle with
    Schlick's Fresnel in the difference angle -- times 1 + N(0, noise), at
    the centre of every (theta_h, theta_d, phi_d) bin (theta_h bins are
    quadratic, as in the format)."""
    rng = np.random.default_rng(seed)
    ih = (np.arange(90) + 0.5) / 90.0
    th = ih * ih * (np.pi / 2)
    td = (np.arange(90) + 0.5) * (np.pi / 2) / 90.0
    TH, TD = np.meshgrid(th, td, indexing="ij")
    fres = 0.04 + 0.96 * (1.0 - np.cos(TD)) ** 5
    lobe = (exponent + 2.0) / (8.0 * np.pi) * np.cos(TH) ** exponent * fres
    out = []
    scales = (1.0 / 1500, 1.15 / 1500, 1.66 / 1500)
    for c in range(3):
        f = kd[c] / np.pi + ks[c] * lobe
        f = np.repeat(f[:, :, None], 180, axis=2) * (1.0 + noise * rng.normal(size=(90, 90, 180)))
        out.append((np.maximum(f, 0.0) / scales[c]).astype("<f8").reshape(-1))
    return np.array([90, 90, 180], "<i4").tobytes() + b"".join(o.tobytes() for o in out)


def glass_sphere_scene(material, lights="area", resolution=(48, 32)):
    """A sphere (radius 0.4, 4 * 4**4 flat outward-facing triangles) above a
    10 x 10 matte floor (albedo (0.7, 0.6, 0.5)), lit by a 0.6 x 0.6 quad
    light of radiance 10 at height 2 (lights="area") or a point light of
    intensity 3 at (0.2, -0.1, 1.6) (lights="point"); `material` is the
    sphere's skwarka_gb300.render.Material.  Returns (prims, materials,
    point_lights, camera): the camera looks at the sphere from above and to
    the side, so the floor is seen directly and through the sphere."""
    from .accel import TriangleMesh
    from .render import Camera, Material, PointLight, RenderPrimitive
    v, t = sphere_mesh(4)
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    outward = (np.cross(b - a, c - a) * (a + b + c)).sum(1) > 0
    t = np.where(outward[:, None], t, t[:, [0, 2, 1]]).astype(np.int32)
    sphere = TriangleMesh((v * 0.4 + np.array([0.0, 0.0, 0.45])).astype(np.float32), t)
    s = 5.0
    floor = TriangleMesh(np.array([[-s, -s, 0], [s, -s, 0], [s, s, 0], [-s, s, 0]], np.float32),
                         np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    prims = [RenderPrimitive(floor, 0), RenderPrimitive(sphere, 1)]
    mats = [Material(kd=(0.7, 0.6, 0.5)), material]
    pls = []
    if lights == "area":
        q = 0.3
        lv = np.array([[-q, -q, 2], [q, -q, 2], [q, q, 2], [-q, q, 2]], np.float32)
        prims.append(RenderPrimitive(TriangleMesh(lv, np.array([[0, 2, 1], [0, 3, 2]], np.int32)), 2,
                                     emission=(10.0, 10.0, 10.0)))
        mats.append(Material(kd=(0.0, 0.0, 0.0)))
    else:
        pls = [PointLight((0.2, -0.1, 1.6), (3.0, 3.0, 3.0))]
    w, h = resolution
    cam = Camera.look_at((1.3, -1.1, 1.2), (0.0, 0.0, 0.35), (0, 0, 1), np.radians(55.0), w, h)
    return prims, mats, pls, cam
