"""Photon maps on the GPU (C ABI: skw_photon_*).

PhotonMap.shoot traces photon paths through a RenderScene on the GPU
(PhotonLTEIntegrator::ShootPhotons); PhotonMap.from_arrays builds the maps
from given photons.  Either way the three photon kd-trees and the irradiance
photon map are built as the reference builds them."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .accel import Context, default_context

# skw_photon: position, weight, incident direction id, geometric normal id.
PHOTON_DTYPE = np.dtype([("position", "<f4", 3), ("weight", "<f4", 3), ("incident", "<u2"), ("normal", "<u2")])
assert PHOTON_DTYPE.itemsize == 28


class skw_photon_params(C.Structure):
    _fields_ = [("paths", C.c_int64), ("max_bounces", C.c_int32), ("rr_probability", C.c_float), ("seed", C.c_uint64)]


class skw_photon_map_info(C.Structure):
    _fields_ = [("n_caustic", C.c_int64), ("n_direct", C.c_int64), ("n_indirect", C.c_int64),
                ("n_irradiance", C.c_int64), ("paths_caustic", C.c_int64), ("paths_direct", C.c_int64),
                ("paths_indirect", C.c_int64), ("max_irradiance_lookup_dist", C.c_double), ("scene_area", C.c_double),
                ("shoot_ms", C.c_double), ("build_ms", C.c_double), ("trees_on_gpu", C.c_int32)]


class PhotonMap:
    MAPS = ("caustic", "direct", "indirect")

    def __init__(self, handle, ctx: Context):
        self.handle, self.ctx = handle, ctx

    @classmethod
    def from_arrays(cls, maps, paths, scene_area: float, ctx: Context | None = None) -> "PhotonMap":
        ctx = ctx or default_context()
        arrs = [np.ascontiguousarray(m, PHOTON_DTYPE) for m in maps]
        ptrs = (C.c_void_p * 3)(*[a.ctypes.data for a in arrs])
        n = np.array([len(a) for a in arrs], np.int64)
        p = np.array(paths, np.int64)
        h = C.c_void_p()
        _lib.check(_lib.load().skw_photon_map_create(ctx.handle, ptrs, n.ctypes.data, p.ctypes.data,
                                                     float(scene_area), C.byref(h)), ctx.handle)
        return cls(h, ctx)

    @classmethod
    def shoot(cls, scene, paths: int, max_bounces: int = 64, rr_probability: float = 0.0, seed: int = 0) -> "PhotonMap":
        h = C.c_void_p()
        par = skw_photon_params(int(paths), int(max_bounces), float(rr_probability), int(seed))
        _lib.check(_lib.load().skw_photon_shoot(scene.handle, C.byref(par), C.byref(h)), scene.ctx.handle)
        return cls(h, scene.ctx)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_photon_map_destroy(h)
            self.handle = None

    def info(self) -> dict:
        i = skw_photon_map_info()
        _lib.check(_lib.load().skw_photon_map_get_info(self.handle, C.byref(i)), self.ctx.handle)
        return {k: getattr(i, k) for k, _ in i._fields_}

    def export(self, which: str) -> np.ndarray:
        w = self.MAPS.index(which)
        n = self.info()["n_" + which]
        out = np.empty(n, PHOTON_DTYPE)
        _lib.check(_lib.load().skw_photon_map_export(self.handle, w, out.ctypes.data if n else None), self.ctx.handle)
        return out

    def irradiance_photons(self):
        """(positions, external, internal irradiance, normal ids) in kd-tree order."""
        n = self.info()["n_irradiance"]
        pos, ext, intr = (np.empty((n, 3), np.float32) for _ in range(3))
        nrm = np.empty(n, np.uint16)
        _lib.check(_lib.load().skw_photon_map_export_irradiance(
            self.handle, pos.ctypes.data, ext.ctypes.data, intr.ctypes.data, nrm.ctypes.data), self.ctx.handle)
        return pos, ext, intr, nrm


class skw_photon_render_params(C.Structure):
    _fields_ = [("gather_samples", C.c_int32), ("caustic_lookup", C.c_int32), ("max_caustic_dist", C.c_double)]


def render_photon(scene, photon_map: PhotonMap, camera, spp_x: int = 2, spp_y: int = 2, light_samples: int = 1,
                  gather_samples: int = 16, seed: int = 0, out=None, stream=None, caustic_lookup: int = 50,
                  max_caustic_dist: float = 0.1, sampler: int = 0):
    """Photon-mapping render (emission + direct lighting + caustic-map
    radiance + final gather) into a CUDA float32 tensor (h, w, 3).
    caustic_lookup / max_caustic_dist: the caustic estimate's photon count
    and radius (PhotonLTEIntegratorParams); used when the map has caustic
    photons.  sampler: render.STRATIFIED or render.LD."""
    import torch
    from .render import c_camera, skw_render_params
    if out is None:
        out = torch.empty((camera.height, camera.width, 3), dtype=torch.float32, device="cuda")
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    cam = c_camera(camera)
    par = skw_render_params(spp_x, spp_y, light_samples, seed, sampler)
    pp = skw_photon_render_params(gather_samples, caustic_lookup, max_caustic_dist)
    _lib.check(_lib.load().skw_render_photon(scene.handle, photon_map.handle, C.byref(cam), C.byref(par), C.byref(pp),
                                             out.data_ptr(), s), scene.ctx.handle)
    return out


def scene_total_area(scene) -> float:
    return float(_lib.load().skw_scene_total_area(scene.handle))
