"""Host-side mirror of the reference's direct-lighting render setup.

``RenderPrimitive`` / ``Material`` / ``PointLight`` describe a scene like the
reference's Primitive + Material + light sources; ``RenderScene`` builds it on
the GPU (``Scene``, Raytracer/Core/Scene.h:107-113) and ``render_direct``
renders an image the way ``SamplerBasedRenderer`` with a ``StratifiedSampler``,
``DirectLightingLTEIntegrator``, pinhole ``PerspectiveCamera`` and a
box-filtered ``ImageFilm`` does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .accel import Context, TriangleMesh, default_context

MATTE, PLASTIC, METAL, MEASURED, TRANSPARENT, SUBSTRATE, UBER, MIX = 0, 1, 2, 3, 4, 5, 6, 7


class MeasuredBRDF:
    """A tabulated BRDF in the MERL binary layout (skw_merl): the file image
    is converted and its sampling tables built on the host, then uploaded."""

    def __init__(self, data: bytes, ctx: "Context | None" = None, device: bool = True):
        """device=False builds the host tables only (no GPU needed; the host
        entry points work, a scene cannot use it)."""
        self.data = bytes(data)
        self.ctx = (ctx or default_context()) if device else None
        ch = self.ctx.handle if self.ctx is not None else None
        h = C.c_void_p()
        _lib.check(_lib.load().skw_merl_create(ch, self.data, len(self.data), C.byref(h)), ch)
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_merl_destroy(h)
            self.handle = None

    def export(self):
        """(half table (1458000, 3) uint16, segmentations (90, 1173) float32)."""
        import numpy as np
        t = np.empty((90 * 90 * 180, 3), np.uint16)
        sg = np.zeros((90, 1173), np.float32)
        _lib.check(_lib.load().skw_merl_export(self.handle, t.ctypes.data, sg.ctypes.data))
        return t, sg

    def eval_host(self, wi, wo):
        import numpy as np
        wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
        wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
        f = np.empty_like(wi)
        pdf = np.empty(len(wi))
        _lib.check(_lib.load().skw_merl_eval_host(self.handle, wi.ctypes.data, wo.ctypes.data, len(wi), f.ctypes.data,
                                                  pdf.ctypes.data))
        return f, pdf

    def sample_host(self, wi, u):
        import numpy as np
        wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, np.float64).reshape(-1, 2)
        wo, f = np.empty_like(wi), np.empty_like(wi)
        pdf = np.empty(len(wi))
        _lib.check(_lib.load().skw_merl_sample_host(self.handle, wi.ctypes.data, u.ctypes.data, len(wi), wo.ctypes.data,
                                                    f.ctypes.data, pdf.ctypes.data))
        return wo, f, pdf


@dataclass
class Material:
    kind: int = MATTE
    kd: tuple = (0.5, 0.5, 0.5)
    ks: tuple = (0.0, 0.0, 0.0)
    roughness: float = 0.1
    sigma: float = 0.0
    eta: tuple = (1.0, 1.0, 1.0)
    k: tuple = (0.0, 0.0, 0.0)
    measured: "MeasuredBRDF | None" = None
    refractive_index: float = 1.5
    kr: tuple = (0.0, 0.0, 0.0)         # UBER: specular reflectance
    opacity: tuple = (1.0, 1.0, 1.0)    # UBER: opacity (1: opaque)
    mix: tuple = (-1, -1)               # MIX: indices of the two mixed materials
    mix_scale: tuple = (0.5, 0.5, 0.5)  # MIX: the first material's scale
    v_roughness: float = 0.0            # SUBSTRATE: > 0 the two-roughness (anisotropic) form


@dataclass
class RenderPrimitive:
    mesh: TriangleMesh
    material: int
    mesh_to_world: np.ndarray | None = None
    vertex_normals: np.ndarray | None = None
    triangle_albedo: np.ndarray | None = None
    emission: tuple = (0.0, 0.0, 0.0)
    vertex_tangents: np.ndarray | None = None  # (nv, 3) mesh-space tangents (the BSDF frame's first axis)
    triangle_uvs: np.ndarray | None = None     # (nt, 6) per-triangle uvs, when no vertex tangents


@dataclass
class Medium:
    """Homogeneous participating medium in an axis-aligned box with a
    Henyey-Greenstein phase function (HomogeneousVolumeRegion, HGPhaseFunction);
    step is the ray-march step (DirectLightingLTEIntegratorParams::m_media_step_size)."""
    lo: tuple = (-1.0, -1.0, -1.0)
    hi: tuple = (1.0, 1.0, 1.0)
    sigma_a: tuple = (0.05, 0.05, 0.05)
    sigma_s: tuple = (0.2, 0.2, 0.2)
    emission: tuple = (0.0, 0.0, 0.0)
    g: float = 0.3
    step: float = 0.05


@dataclass
class PointLight:
    position: tuple
    intensity: tuple


@dataclass
class Camera:
    camera_to_world: np.ndarray
    x_view_angle: float
    width: int
    height: int

    @staticmethod
    def look_at(eye, target, up, x_view_angle, width, height) -> "Camera":
        """Camera x -> image right, camera y -> image down, camera z -> forward."""
        eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
        f = target - eye
        f /= np.linalg.norm(f)
        r = np.cross(f, up)
        r /= np.linalg.norm(r)
        d = np.cross(f, r)
        m = np.eye(4)
        m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, d, f, eye
        return Camera(m, float(x_view_angle), int(width), int(height))


class skw_material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("kd", C.c_float * 3), ("ks", C.c_float * 3), ("roughness", C.c_float),
                ("sigma", C.c_float), ("eta", C.c_float * 3), ("k", C.c_float * 3), ("measured", C.c_void_p),
                ("refractive_index", C.c_float), ("kr", C.c_float * 3), ("opacity", C.c_float * 3),
                ("mix", C.c_int32 * 2), ("mix_scale", C.c_float * 3), ("v_roughness", C.c_float)]


class skw_render_primitive(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("mesh_to_world", C.c_void_p), ("material", C.c_int32),
                ("vertex_normals", C.c_void_p), ("triangle_albedo", C.c_void_p), ("emission", C.c_float * 3),
                ("vertex_tangents", C.c_void_p), ("triangle_uvs", C.c_void_p)]


class skw_point_light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("intensity", C.c_float * 3)]


class skw_camera(C.Structure):
    _fields_ = [("camera_to_world", C.c_double * 16), ("x_view_angle", C.c_double), ("width", C.c_int32),
                ("height", C.c_int32)]


class skw_render_params(C.Structure):
    _fields_ = [("spp_x", C.c_int32), ("spp_y", C.c_int32), ("light_samples", C.c_int32), ("seed", C.c_uint64),
                ("sampler", C.c_int32)]


STRATIFIED, LD = 0, 1  # SKW_SAMPLER_STRATIFIED (StratifiedSampler), SKW_SAMPLER_LD (LDSampler)


def c_material(m: Material, measured_handle=None) -> skw_material:
    """measured_handle overrides the handle of m.measured (the reference
    driver passes its own)."""
    h = measured_handle
    if h is None and m.measured is not None:
        h = m.measured.handle
    return skw_material(m.kind, (C.c_float * 3)(*m.kd), (C.c_float * 3)(*m.ks), m.roughness, m.sigma,
                        (C.c_float * 3)(*m.eta), (C.c_float * 3)(*m.k), h, m.refractive_index,
                        (C.c_float * 3)(*m.kr), (C.c_float * 3)(*m.opacity), (C.c_int32 * 2)(*m.mix),
                        (C.c_float * 3)(*m.mix_scale), m.v_roughness)


def c_camera(cam: Camera) -> skw_camera:
    return skw_camera((C.c_double * 16)(*np.asarray(cam.camera_to_world, np.float64).reshape(-1)), cam.x_view_angle,
                      cam.width, cam.height)


def c_prims(prims: list[RenderPrimitive]):
    """(skw_mesh array, skw_render_primitive array, keep-alive list)."""
    keep, meshes, mesh_ids = [], [], {}
    for p in prims:
        if id(p.mesh) not in mesh_ids:
            mesh_ids[id(p.mesh)] = len(meshes)
            meshes.append(p.mesh)
    cm = (_lib.skw_mesh * max(len(meshes), 1))()
    for i, m in enumerate(meshes):
        cm[i] = _lib.skw_mesh(m.vertices.ctypes.data, m.vertices.shape[0], m.triangles.ctypes.data, m.triangles.shape[0])
    cp = (skw_render_primitive * max(len(prims), 1))()
    for i, p in enumerate(prims):
        xf = None if p.mesh_to_world is None else np.ascontiguousarray(p.mesh_to_world, np.float64).reshape(4, 4)
        vn = None if p.vertex_normals is None else np.ascontiguousarray(p.vertex_normals, np.float32).reshape(-1, 3)
        ta = None if p.triangle_albedo is None else np.ascontiguousarray(p.triangle_albedo, np.float32).reshape(-1, 3)
        vt = None if p.vertex_tangents is None else np.ascontiguousarray(p.vertex_tangents, np.float32).reshape(-1, 3)
        uv = None if p.triangle_uvs is None else np.ascontiguousarray(p.triangle_uvs, np.float32).reshape(-1, 6)
        keep += [xf, vn, ta, vt, uv]
        cp[i] = skw_render_primitive(mesh_ids[id(p.mesh)], None if xf is None else xf.ctypes.data, p.material,
                                     None if vn is None else vn.ctypes.data, None if ta is None else ta.ctypes.data,
                                     (C.c_float * 3)(*p.emission), None if vt is None else vt.ctypes.data,
                                     None if uv is None else uv.ctypes.data)
    return cm, len(meshes), cp, keep


class skw_medium(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3),
                ("emission", C.c_float * 3), ("g", C.c_float), ("step", C.c_float)]


class skw_batch_config(C.Structure):
    _fields_ = [("samples_per_pass", C.c_int64), ("stack_cap", C.c_int32), ("trace_ctas_per_sm", C.c_int32),
                ("shade_block", C.c_int32), ("overlap", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RenderScene:
    def __init__(self, prims: list[RenderPrimitive], materials: list[Material], point_lights=(),
                 ctx: Context | None = None, medium: "Medium | None" = None):
        self.ctx = ctx or default_context()
        lib = _lib.load()
        cm, nm, cp, self._keep = c_prims(prims)
        mats = (skw_material * max(len(materials), 1))(*[c_material(m) for m in materials])
        pls = (skw_point_light * max(len(point_lights), 1))(
            *[skw_point_light((C.c_float * 3)(*l.position), (C.c_float * 3)(*l.intensity)) for l in point_lights])
        h = C.c_void_p()
        _lib.check(lib.skw_scene_create(self.ctx.handle, cm, nm, cp, len(prims), mats, len(materials), pls,
                                        len(point_lights), C.byref(h)), self.ctx.handle)
        self.handle = h
        self.prims, self.materials, self.point_lights = prims, materials, list(point_lights)
        if medium is not None:
            self.set_medium(medium)

    def set_medium(self, medium: "Medium | None") -> None:
        m = None
        if medium is not None:
            m = skw_medium((C.c_float * 3)(*medium.lo), (C.c_float * 3)(*medium.hi), (C.c_float * 3)(*medium.sigma_a),
                           (C.c_float * 3)(*medium.sigma_s), (C.c_float * 3)(*medium.emission), medium.g, medium.step)
        _lib.check(_lib.load().skw_scene_set_medium(self.handle, None if m is None else C.byref(m)), self.ctx.handle)

    def hit_geometry(self, rays, hits, stream=None):
        """(n, 12) float64 CUDA tensor: point, geometric normal, shading
        normal, b1, b2, t of closest hits (rays (n, 8) float32 and hits (n, 4)
        int32 as skw_intersect returns them for this scene's accelerator)."""
        import torch
        n = rays.shape[0]
        out = torch.empty((n, 12), dtype=torch.float64, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(_lib.load().skw_scene_hit_geometry(self.handle, rays.data_ptr(), hits.data_ptr(), n,
                                                      out.data_ptr(), s), self.ctx.handle)
        return out

    def accelerator(self):
        """The scene's own accelerator (skw_scene_accel; owned by the scene)
        for ray queries on the scene's primitives."""
        from .accel import TriangleAccelerator
        a = TriangleAccelerator.__new__(TriangleAccelerator)
        a.ctx, a.primitives, a._owner = self.ctx, self.prims, self
        a.handle = C.c_void_p(_lib.load().skw_scene_accel(self.handle))
        a._borrowed = True
        return a

    def intersection(self, rays_d, hits_d, diffs=None, stream=None):
        """The whole Intersection of closest hits (skw_scene_intersection):
        rays_d (n, 8) float64 CUDA tensor of double rays, hits_d the (n, 2)
        float64 skw_hit_d records skw_intersect_d returned for them on this
        scene's accelerator, diffs (optional) (n, 12) float64: origin_dx,
        direction_dx, origin_dy, direction_dy.  Returns an (n, 36) float64
        CUDA tensor in skw_intersection layout: point, geometric normal,
        shading normal, uv, point_dx, point_dy, normal_dx, normal_dy, duv_dx,
        duv_dy, tangent, cross, dot, t, then prim and tri as int32 bits."""
        import torch
        n = rays_d.shape[0]
        rd = torch.zeros((n, 21), dtype=torch.float64, device=rays_d.device)
        rd[:, :8] = rays_d
        if diffs is not None:
            rd[:, 8:20] = diffs
            rd[:, 20] = torch.tensor([1], dtype=torch.int64).view(torch.float64).item()
        out = torch.empty((n, 36), dtype=torch.float64, device=rays_d.device)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(_lib.load().skw_scene_intersection(self.handle, rd.data_ptr(), hits_d.data_ptr(), n,
                                                      out.data_ptr(), s), self.ctx.handle)
        return out

    def next_rays(self, rays, hits, directions, stream=None):
        """Outgoing rays as the renders make them (skw_scene_next_rays): from
        the float hit points of closest hits (rays (n, 8) float32, hits (n, 4)
        int32 from skw_intersect on this scene's accelerator) in the given
        (n, 3) float32 directions, tmin = GetNextMinT.  (n, 8) float32."""
        import torch
        n = rays.shape[0]
        out = torch.empty((n, 8), dtype=torch.float32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        d = directions.contiguous()
        _lib.check(_lib.load().skw_scene_next_rays(self.handle, rays.data_ptr(), hits.data_ptr(), d.data_ptr(), n,
                                                   out.data_ptr(), s), self.ctx.handle)
        return out

    def set_max_specular_depth(self, depth: int) -> None:
        """DirectLightingLTEIntegratorParams::m_max_specular_depth (default 10, at most 11)."""
        _lib.check(_lib.load().skw_scene_set_max_specular_depth(self.handle, int(depth)), self.ctx.handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_scene_destroy(h)
            self.handle = None

    def render_direct(self, camera: Camera, spp_x: int = 2, spp_y: int = 2, light_samples: int = 1, seed: int = 0,
                      out=None, stream=None, sampler: int = STRATIFIED):
        """Renders into a CUDA float32 tensor (height, width, 3) and returns it.
        sampler=LD: LDSampler with spp_x * spp_y samples per pixel."""
        import torch
        if out is None:
            out = torch.empty((camera.height, camera.width, 3), dtype=torch.float32, device="cuda")
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        cam = c_camera(camera)
        par = skw_render_params(spp_x, spp_y, light_samples, seed, sampler)
        _lib.check(_lib.load().skw_render_direct(self.handle, C.byref(cam), C.byref(par), out.data_ptr(), s),
                   self.ctx.handle)
        return out


class RenderBatch:
    """Many cameras of one RenderScene rendered as one wavefront (one CUDA
    graph launch per run).  View v gets seed = seeds[v] (default seed + v)
    and renders exactly what RenderScene.render_direct renders with that
    seed."""

    def __init__(self, scene: RenderScene, cameras: list[Camera], spp_x: int = 2, spp_y: int = 2,
                 light_samples: int = 1, seed: int = 0, seeds=None, config: dict | None = None,
                 sampler: int = STRATIFIED):
        import numpy as np
        lib = _lib.load()
        self.scene, self.cameras = scene, list(cameras)
        cams = (skw_camera * len(cameras))(*[c_camera(c) for c in cameras])
        par = skw_render_params(spp_x, spp_y, light_samples, seed, sampler)
        self._seeds = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
        cfg = None
        if config is not None:
            cfg = skw_batch_config(**config)
        h = C.c_void_p()
        _lib.check(lib.skw_render_batch_create(scene.handle, cams, len(cameras), C.byref(par),
                                               None if self._seeds is None else self._seeds.ctypes.data,
                                               None if cfg is None else C.byref(cfg), C.byref(h)), scene.ctx.handle)
        self.handle = h
        self.n_floats = int(lib.skw_render_batch_film_floats(h))
        self.offsets = [int(lib.skw_render_batch_film_offset(h, v)) for v in range(len(cameras))]

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_render_batch_destroy(h)
            self.handle = None

    def config(self) -> dict:
        c = skw_batch_config()
        _lib.check(_lib.load().skw_render_batch_get_config(self.handle, C.byref(c)), self.scene.ctx.handle)
        return c.as_dict()

    def new_films(self):
        import torch
        return torch.empty(self.n_floats, dtype=torch.float32, device="cuda")

    def run(self, films=None, stream=None):
        """Renders all views into the packed float buffer `films` (CUDA) and
        returns it; view(films, v) is view v's (h, w, 3) image."""
        import torch
        if films is None:
            films = self.new_films()
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(_lib.load().skw_render_batch_run(self.handle, films.data_ptr(), s), self.scene.ctx.handle)
        return films

    def view(self, films, v: int):
        c = self.cameras[v]
        o = self.offsets[v]
        return films[o:o + c.width * c.height * 3].view(c.height, c.width, 3)

    def autotune(self, stream=None) -> tuple[dict, float, int]:
        """Times candidate configurations on the GPU and installs the best:
        (config, ms per run, candidates timed)."""
        import torch
        scratch = self.new_films()
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        best, ms, n = skw_batch_config(), C.c_float(), C.c_int32()
        _lib.check(_lib.load().skw_render_batch_autotune(self.handle, scratch.data_ptr(), s, C.byref(best),
                                                         C.byref(ms), C.byref(n)), self.scene.ctx.handle)
        return best.as_dict(), float(ms.value), int(n.value)
