"""ctypes access to the oracle (test infrastructure only).

``Oracle`` wraps ``oracle/_build/libskw_oracle.so`` (the CPU restatement in
``oracle/skw_oracle.cpp``); ``Reference`` wraps ``oracle/_ref/libskw_ref.so``
(the reference's own sources, built by ``oracle/build_ref.py``) and is None
where that library is absent.  Only tests, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` use this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "libskw_oracle.so"
REF_LIB = HERE / "_ref" / "libskw_ref.so"

_P = C.c_void_p
_i64 = C.c_int64


def _ptr(a):
    return None if a is None else a.ctypes.data


def _declare(lib, table):
    for name, res, args in table:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_ORACLE_SIGS = [
    ("oracle_accel_create", _P, [_P, _P, _P, _i64]),
    ("oracle_accel_destroy", None, [_P]),
    ("oracle_accel_num_nodes", _i64, [_P]),
    ("oracle_accel_export", None, [_P, _P, _P, _P, _P]),
    ("oracle_intersect", None, [_P, _P, _i64, _P, _P, _P, _P, _P, C.c_int]),
    ("oracle_intersect_test", None, [_P, _P, _i64, _P, _P, _P, C.c_int]),
    ("oracle_intersect_d", None, [_P, _P, _i64, _P, _P, _P, C.c_int]),
    ("oracle_intersect_test_d", None, [_P, _P, _i64, _P, C.c_int]),
    ("oracle_brute_force", None, [_P, _P, _P, _i64, _P, _i64, _P, _P, _P, C.c_int]),
    ("oracle_kdtree_create", _P, [_P, _P, _i64, _P, _P]),
    ("oracle_kdtree_destroy", None, [_P]),
    ("oracle_knn", None, [_P, _P, _P, _i64, C.c_int32, C.c_double, C.c_double, _P, _P, _P, _P, C.c_int]),
    ("oracle_compressed_direction_table", None, [_P]),
    ("oracle_nearest", None, [_P, _P, _P, _i64, C.c_double, C.c_double, _P, C.c_int]),
]

_REF_SIGS = [
    ("skw_ref_accel_create", _P, [C.c_int, _P, C.c_int, _P, _P, _P, _P, _P]),
    ("skw_ref_accel_destroy", None, [_P]),
    ("skw_ref_intersect", None, [_P, _P, _i64, _P, _P, _P, C.c_int]),
    ("skw_ref_intersect_test", None, [_P, _P, _i64, _P, C.c_int]),
    ("skw_ref_accel_create_normals", _P, [C.c_int, _P, C.c_int, _P, _P, _P, _P, _P, _P]),
    ("skw_ref_accel_num_instances", _i64, [_P]),
    ("skw_ref_accel_export_instances", None, [_P, _P, _P, _P]),
    ("skw_ref_accel_meshes_ascending", C.c_int, [_P]),
    ("skw_ref_accel_mesh_rank", None, [_P, _P]),
    ("skw_ref_intersect_d", None, [_P, _P, _i64, _P, _P, _P, C.c_int]),
    ("skw_ref_intersect_test_d", None, [_P, _P, _i64, _P, C.c_int]),
    ("skw_ref_intersection", None, [_P, _P, _P, _i64, _P, _P, _P, C.c_int]),
    ("skw_ref_accel_num_nodes", _i64, [_P]),
    ("skw_ref_accel_num_triangles", _i64, [_P]),
    ("skw_ref_accel_export", None, [_P, _P, _P, _P, _P, _P]),
    ("skw_ref_kdtree_create", _P, [_P, _P, _P, _i64, _P, _P]),
    ("skw_ref_kdtree_destroy", None, [_P]),
    ("skw_ref_knn", None, [_P, _P, _P, _i64, C.c_int32, C.c_double, C.c_double, _P, _P, _P, C.c_int]),
    ("skw_ref_nearest", None, [_P, _P, _i64, C.c_double, _P, C.c_int]),
    ("skw_ref_compressed_direction_table", None, [_P]),
    ("skw_ref_compress_direction", C.c_uint16, [C.c_double, C.c_double, C.c_double]),
    ("skw_ref_render_direct", C.c_int, [C.c_int, _P, _P, _P, _P, C.c_int, _P, C.c_int, _P, C.c_int, _P, _P,
                                        C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P,
                                        C.c_int]),
    ("skw_ref_luminance_weights", None, [_P]),
    ("skw_ref_pbrt_rgb", None, [C.c_int, _P, _i64, _P]),
    ("skw_ref_render_photon", C.c_int, [C.c_int, _P, _P, _P, _P, C.c_int, _P, _P, C.c_int, _P, _P, C.c_double,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i64, C.c_int, C.c_int,
                                        C.c_double, _P, _P, _P]),
    ("skw_ref_photon_irradiance", C.c_int, [_P, _P, _P, C.c_double, _P, _P, _P, _P, _P, _P]),
    ("skw_ref_shoot_photons", C.c_int, [C.c_int, _P, _P, _P, _P, C.c_int, _P, _P, C.c_int, _P, _i64, _P, _P, _P]),
    ("skw_ref_render_photon_maps", C.c_int, [C.c_int, _P, _P, _P, _P, C.c_int, _P, _P, C.c_int, _P, _P, _P, _P, _P,
                                             C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_double, _P, _P, _P]),
    ("skw_ref_merl_create", _P, [C.c_char_p, _i64]),
    ("skw_ref_merl_destroy", None, [_P]),
    ("skw_ref_merl_export", None, [_P, _P, _P]),
    ("skw_ref_merl_eval", None, [_P, _P, _P, _i64, _P, _P]),
    ("skw_ref_merl_sample", None, [_P, _P, _P, _i64, _P, _P, _P]),
]


def world_triangles(meshes):
    """Flatten [(vertices, triangles)] with identity transforms into the
    reference's triangle order: (tris float32 (n, 9), prim int32, tri int32)."""
    tv, pr, ti = [], [], []
    for p, (v, t) in enumerate(meshes):
        v = np.asarray(v, np.float32)
        t = np.asarray(t, np.int64)
        ok = ((t >= 0) & (t < len(v))).all(1) & (t[:, 0] != t[:, 1]) & (t[:, 0] != t[:, 2]) & (t[:, 1] != t[:, 2])
        t = t[ok]
        tv.append(v[t].reshape(-1, 9))
        pr.append(np.full(len(t), p, np.int32))
        ti.append(np.arange(len(t), dtype=np.int32))
    return (np.ascontiguousarray(np.concatenate(tv)), np.concatenate(pr), np.concatenate(ti))


class Oracle:
    def __init__(self):
        if not ORACLE_LIB.exists():
            from . import build
            build.build_oracle()
        self.lib = _declare(C.CDLL(str(ORACLE_LIB)), _ORACLE_SIGS)

    # -- accelerator --
    def accel(self, meshes):
        tris, prim, tidx = world_triangles(meshes)
        return OracleAccel(self.lib, tris, prim, tidx)

    def brute_force(self, tris, prim, tidx, rays, threads=0):
        n = rays.shape[0]
        p, t, th = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.float64)
        self.lib.oracle_brute_force(_ptr(tris), _ptr(prim), _ptr(tidx), tris.shape[0], _ptr(rays), n, _ptr(p),
                                    _ptr(t), _ptr(th), threads)
        return p, t, th

    # -- photon kd-tree --
    def kdtree(self, pos, normal_ids=None):
        return OracleKD(self.lib, pos, normal_ids)

    def direction_table(self):
        out = np.empty((1 << 16, 3), np.float64)
        self.lib.oracle_compressed_direction_table(_ptr(out))
        return out


class OracleAccel:
    def __init__(self, lib, tris, prim, tidx):
        self.lib = lib
        self.tris, self.prim, self.tidx = tris, prim, tidx
        self.h = lib.oracle_accel_create(_ptr(tris), _ptr(prim), _ptr(tidx), tris.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_accel_destroy(self.h)
            self.h = None

    def export(self):
        nn = self.lib.oracle_accel_num_nodes(self.h)
        bbox = np.empty((nn, 6), np.float32)
        info = np.empty((nn, 8), np.int32)
        tp = np.empty(max(self.tris.shape[0], 1), np.int32)
        ti = np.empty(max(self.tris.shape[0], 1), np.int32)
        self.lib.oracle_accel_export(self.h, _ptr(bbox), _ptr(info), _ptr(tp), _ptr(ti))
        return bbox, info, tp[:self.tris.shape[0]], ti[:self.tris.shape[0]]

    def intersect(self, rays, counters=False, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        p, t, th = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.float64)
        nv = np.empty(n, np.int32) if counters else None
        nt = np.empty(n, np.int32) if counters else None
        self.lib.oracle_intersect(self.h, _ptr(rays), n, _ptr(p), _ptr(t), _ptr(th), _ptr(nv), _ptr(nt), threads)
        out = {"prim": p, "tri": t, "t": th}
        if counters:
            out.update(nodes=nv, tris=nt)
        return out

    def intersect_d(self, rays, threads=0):
        """Closest hits of double rays ((n, 8) float64)."""
        rays = np.ascontiguousarray(rays, np.float64)
        n = rays.shape[0]
        p, t, th = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.float64)
        self.lib.oracle_intersect_d(self.h, _ptr(rays), n, _ptr(p), _ptr(t), _ptr(th), threads)
        return {"prim": p, "tri": t, "t": th}

    def intersect_test_d(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float64)
        occ = np.empty(rays.shape[0], np.uint8)
        self.lib.oracle_intersect_test_d(self.h, _ptr(rays), rays.shape[0], _ptr(occ), threads)
        return occ

    def intersect_test(self, rays, counters=False, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        nv = np.empty(n, np.int32) if counters else None
        nt = np.empty(n, np.int32) if counters else None
        self.lib.oracle_intersect_test(self.h, _ptr(rays), n, _ptr(occ), _ptr(nv), _ptr(nt), threads)
        if counters:
            return occ, nv, nt
        return occ


class OracleKD:
    def __init__(self, lib, pos, normal_ids=None):
        self.lib = lib
        self.pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        self.nids = None if normal_ids is None else np.ascontiguousarray(normal_ids, np.uint16)
        n = self.pos.shape[0]
        self.perm = np.empty(n, np.int32)
        self.nodes = np.empty((n, 2), np.uint32)
        self.h = lib.oracle_kdtree_create(_ptr(self.pos), _ptr(self.nids), n, _ptr(self.perm), _ptr(self.nodes))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_kdtree_destroy(self.h)
            self.h = None

    def knn(self, q, qn, k, max_dist, cos_threshold=-1.0, counters=False, threads=0):
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        qn = None if qn is None else np.ascontiguousarray(qn, np.float64).reshape(-1, 3)
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int32)
        d2 = np.empty((nq, k), np.float64)
        cnt = np.empty(nq, np.int32)
        vis = np.empty(nq, np.int32) if counters else None
        self.lib.oracle_knn(self.h, _ptr(q), _ptr(qn), nq, k, max_dist, cos_threshold, _ptr(idx), _ptr(d2), _ptr(cnt),
                            _ptr(vis), threads)
        out = {"idx": idx, "d2": d2, "count": cnt}
        if counters:
            out["visited"] = vis
        return out

    def nearest(self, q, qn, max_dist, cos_threshold=-1.0, threads=0):
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        qn = None if qn is None else np.ascontiguousarray(qn, np.float64).reshape(-1, 3)
        out = np.empty(q.shape[0], np.int32)
        self.lib.oracle_nearest(self.h, _ptr(q), _ptr(qn), q.shape[0], max_dist, cos_threshold, _ptr(out), threads)
        return out


class Reference:
    """The reference's own code (oracle/_ref/libskw_ref.so)."""

    def __init__(self):
        self.lib = _declare(C.CDLL(str(REF_LIB)), _REF_SIGS)

    @staticmethod
    def available() -> bool:
        return REF_LIB.exists()

    def accel(self, meshes, normals=None, mesh_of=None, xforms=None):
        return RefAccel(self.lib, meshes, normals, mesh_of, xforms)

    def pbrt_rgb(self, kind: int, rgb) -> np.ndarray:
        """The PBRT importer's colour conversion of float RGB triples (kind 0
        a reflectance, 1 an emission): (n, 3) float64."""
        x = np.ascontiguousarray(np.asarray(rgb, np.float32).reshape(-1, 3))
        out = np.zeros(x.shape, np.float64)
        self.lib.skw_ref_pbrt_rgb(kind, x.ctypes.data, x.shape[0], out.ctypes.data)
        return out

    def kdtree(self, pos, normal_ids=None, dir_ids=None):
        return RefKD(self.lib, pos, normal_ids, dir_ids)

    def direction_table(self):
        out = np.empty((1 << 16, 3), np.float64)
        self.lib.skw_ref_compressed_direction_table(_ptr(out))
        return out

    def _merl(self, measured):
        """The reference's MERLMeasuredData for a MeasuredBRDF (cached)."""
        cache = self.__dict__.setdefault("_merl_cache", {})
        key = id(measured)
        if key not in cache:
            cache[key] = (measured, self.lib.skw_ref_merl_create(measured.data, len(measured.data)))
        return cache[key][1]

    def merl(self, data: bytes):
        return RefMerl(self.lib, data)

    def photon_irradiance(self, maps, paths, scene_area):
        """The reference's _ConstructIrradiancePhotonMap on the given photon
        maps (structured arrays of PHOTON_DTYPE: caustic, direct, indirect)
        with their path counts: (positions, external, internal irradiance,
        normal ids -- in its kd-tree order -- and the max lookup distance)."""
        from skwarka_gb300.photon import PHOTON_DTYPE
        arrs = [np.ascontiguousarray(m, PHOTON_DTYPE) for m in maps]
        ptrs = (C.c_void_p * 3)(*[a.ctypes.data for a in arrs])
        n = np.array([len(a) for a in arrs], np.int64)
        pth = np.array(paths, np.int64)
        cap = len(arrs[2]) // 10 + 1
        pos, ext, intr = (np.zeros((cap, 3), np.float32) for _ in range(3))
        nrm = np.zeros(cap, np.uint16)
        k, md = np.zeros(1, np.int64), np.zeros(1)
        self.lib.skw_ref_photon_irradiance(ptrs, _ptr(n), _ptr(pth), float(scene_area), _ptr(k), _ptr(pos), _ptr(ext),
                                           _ptr(intr), _ptr(nrm), _ptr(md))
        k = int(k[0])
        return pos[:k], ext[:k], intr[:k], nrm[:k], float(md[0])

    def render_photon(self, prims, materials, point_lights, camera, spp_x, spp_y, n_paths, light_samples=1,
                      gather_samples=16, caustic_lookup=50, max_caustic_dist=0.1):
        """The reference's photon-mapping render (PhotonLTEIntegrator:
        ShootPhotons(n_paths), then the sampler-based render with final
        gathering): (film, {"shoot_s", "render_s", "caustic", "direct",
        "indirect", "irradiance"})."""
        from skwarka_gb300.render import c_material, c_prims
        cm, nm, cp, keep = c_prims(prims)
        verts = (C.c_void_p * nm)(*[cm[i].vertices for i in range(nm)])
        tris = (C.c_void_p * nm)(*[cm[i].triangles for i in range(nm)])
        nv = np.array([cm[i].n_vertices for i in range(nm)], np.int64)
        nt = np.array([cm[i].n_triangles for i in range(nm)], np.int64)
        mats = (type(c_material(materials[0])) * len(materials))(
            *[c_material(m, self._merl(m.measured) if m.measured is not None else None) for m in materials])
        pl = np.array([list(l.position) + list(l.intensity) for l in point_lights], np.float32).reshape(-1, 6)
        c2w = np.ascontiguousarray(camera.camera_to_world, np.float64).reshape(-1)
        film = np.zeros((max(camera.height, 1), max(camera.width, 1), 3), np.float32)
        info = np.zeros(4, np.int64)
        sec = np.zeros(2)
        self.lib.skw_ref_render_photon(nm, verts, _ptr(nv), tris, _ptr(nt), len(prims), C.addressof(cp),
                                       C.addressof(mats), len(point_lights), _ptr(pl) if len(pl) else None, _ptr(c2w),
                                       camera.x_view_angle, camera.width, camera.height, spp_x, spp_y, light_samples,
                                       int(n_paths), gather_samples, caustic_lookup, max_caustic_dist, _ptr(film),
                                       _ptr(info), _ptr(sec))
        return film, {"shoot_s": float(sec[0]), "render_s": float(sec[1]), "caustic": int(info[0]),
                      "direct": int(info[1]), "indirect": int(info[2]), "irradiance": int(info[3])}

    def shoot_photons(self, prims, materials, point_lights, n_paths, cap=4_000_000):
        """The reference's PhotonLTEIntegrator::ShootPhotons(n_paths): the
        positions (float32 (n, 3), kd-tree order) of its caustic, direct and
        indirect photons."""
        from skwarka_gb300.render import c_material, c_prims
        cm, nm, cp, keep = c_prims(prims)
        verts = (C.c_void_p * nm)(*[cm[i].vertices for i in range(nm)])
        tris = (C.c_void_p * nm)(*[cm[i].triangles for i in range(nm)])
        nv = np.array([cm[i].n_vertices for i in range(nm)], np.int64)
        nt = np.array([cm[i].n_triangles for i in range(nm)], np.int64)
        mats = (type(c_material(materials[0])) * len(materials))(
            *[c_material(m, self._merl(m.measured) if m.measured is not None else None) for m in materials])
        pl = np.array([list(l.position) + list(l.intensity) for l in point_lights], np.float32).reshape(-1, 6)
        bufs = [np.zeros((cap, 3), np.float32) for _ in range(3)]
        ptrs = (C.c_void_p * 3)(*[b.ctypes.data for b in bufs])
        caps = np.full(3, cap, np.int64)
        n = np.zeros(3, np.int64)
        self.lib.skw_ref_shoot_photons(nm, verts, _ptr(nv), tris, _ptr(nt), len(prims), C.addressof(cp),
                                       C.addressof(mats), len(point_lights), _ptr(pl) if len(pl) else None,
                                       int(n_paths), ptrs, _ptr(caps), _ptr(n))
        return [b[:min(int(k), cap)] for b, k in zip(bufs, n)]

    def render_photon_maps(self, prims, materials, point_lights, camera, spp_x, spp_y, maps, paths, light_samples=1,
                           gather_samples=16, caustic_lookup=50, max_caustic_dist=0.1):
        """The reference's photon-mapping render with the given photon maps
        (structured arrays of PHOTON_DTYPE: caustic, direct, indirect, with
        their path counts) in place of ShootPhotons: (film, {"render_s",
        "caustic", "direct", "indirect", "irradiance"})."""
        from skwarka_gb300.photon import PHOTON_DTYPE
        from skwarka_gb300.render import c_material, c_prims
        cm, nm, cp, keep = c_prims(prims)
        verts = (C.c_void_p * nm)(*[cm[i].vertices for i in range(nm)])
        tris = (C.c_void_p * nm)(*[cm[i].triangles for i in range(nm)])
        nv = np.array([cm[i].n_vertices for i in range(nm)], np.int64)
        nt = np.array([cm[i].n_triangles for i in range(nm)], np.int64)
        mats = (type(c_material(materials[0])) * len(materials))(
            *[c_material(m, self._merl(m.measured) if m.measured is not None else None) for m in materials])
        pl = np.array([list(l.position) + list(l.intensity) for l in point_lights], np.float32).reshape(-1, 6)
        arrs = [np.ascontiguousarray(m, PHOTON_DTYPE) for m in maps]
        ptrs = (C.c_void_p * 3)(*[a.ctypes.data for a in arrs])
        n = np.array([len(a) for a in arrs], np.int64)
        pth = np.array(paths, np.int64)
        c2w = np.ascontiguousarray(camera.camera_to_world, np.float64).reshape(-1)
        film = np.zeros((camera.height, camera.width, 3), np.float32)
        info = np.zeros(4, np.int64)
        sec = np.zeros(1)
        self.lib.skw_ref_render_photon_maps(nm, verts, _ptr(nv), tris, _ptr(nt), len(prims), C.addressof(cp),
                                            C.addressof(mats), len(point_lights), _ptr(pl) if len(pl) else None, ptrs,
                                            _ptr(n), _ptr(pth), _ptr(c2w), camera.x_view_angle, camera.width,
                                            camera.height, spp_x, spp_y, light_samples, gather_samples,
                                            caustic_lookup, max_caustic_dist, _ptr(film), _ptr(info), _ptr(sec))
        return film, {"render_s": float(sec[0]), "caustic": int(info[0]), "direct": int(info[1]),
                      "indirect": int(info[2]), "irradiance": int(info[3])}

    def render_direct(self, prims, materials, point_lights, camera, spp_x, spp_y, light_samples=1, medium=None,
                      ld=False):
        """The reference's own direct-lighting render of a scene described with
        skwarka_gb300.render types: (film (h, w, 3) float32, seconds).
        medium: skwarka_gb300.render.Medium or None; ld: LDSampler with
        spp_x * spp_y samples per pixel instead of the StratifiedSampler."""
        from skwarka_gb300.render import c_material, c_prims
        cm, nm, cp, keep = c_prims(prims)
        verts = (C.c_void_p * nm)(*[cm[i].vertices for i in range(nm)])
        tris = (C.c_void_p * nm)(*[cm[i].triangles for i in range(nm)])
        nv = np.array([cm[i].n_vertices for i in range(nm)], np.int64)
        nt = np.array([cm[i].n_triangles for i in range(nm)], np.int64)
        mats = (type(c_material(materials[0])) * len(materials))(
            *[c_material(m, self._merl(m.measured) if m.measured is not None else None) for m in materials])
        pl = np.array([list(l.position) + list(l.intensity) for l in point_lights], np.float32).reshape(-1, 6)
        c2w = np.ascontiguousarray(camera.camera_to_world, np.float64).reshape(-1)
        film = np.zeros((camera.height, camera.width, 3), np.float32)
        sec = np.zeros(1)
        med = None
        if medium is not None:
            med = np.array(list(medium.lo) + list(medium.hi) + list(medium.emission) + list(medium.sigma_a)
                           + list(medium.sigma_s) + [medium.g, medium.step], np.float64)
        self.lib.skw_ref_render_direct(nm, verts, _ptr(nv), tris, _ptr(nt), len(prims), C.addressof(cp), len(materials),
                                       C.addressof(mats), len(point_lights), _ptr(pl) if len(pl) else None, _ptr(c2w),
                                       camera.x_view_angle, camera.width, camera.height, spp_x, spp_y, light_samples,
                                       _ptr(film), _ptr(sec), None if med is None else _ptr(med), int(bool(ld)))
        return film, float(sec[0])


class RefAccel:
    def __init__(self, lib, meshes, normals=None, mesh_of=None, xforms=None):
        """meshes: [(vertices, triangles)]; normals: optional per-mesh vertex
        normals (or None entries); mesh_of: the mesh of each primitive
        (default one primitive per mesh); xforms: optional (n_prims, 4, 4)
        mesh-to-world matrices."""
        self.lib = lib
        self._v = [np.ascontiguousarray(v, np.float32) for v, _ in meshes]
        self._t = [np.ascontiguousarray(t, np.int32) for _, t in meshes]
        nm = len(meshes)
        vp = (C.c_void_p * nm)(*[v.ctypes.data for v in self._v])
        tp = (C.c_void_p * nm)(*[t.ctypes.data for t in self._t])
        nv = np.array([v.shape[0] for v in self._v], np.int64)
        nt = np.array([t.shape[0] for t in self._t], np.int64)
        self._mesh_of = np.arange(nm, dtype=np.int32) if mesh_of is None else np.ascontiguousarray(mesh_of, np.int32)
        npr = len(self._mesh_of)
        self._x = None if xforms is None else np.ascontiguousarray(xforms, np.float64).reshape(npr, 16)
        if normals is None:
            self.h = lib.skw_ref_accel_create(npr, _ptr(self._mesh_of), nm, vp, _ptr(nv), tp, _ptr(nt),
                                              _ptr(self._x))
        else:
            self._n = [None if n is None else np.ascontiguousarray(n, np.float32) for n in normals]
            np_ = (C.c_void_p * nm)(*[None if n is None else n.ctypes.data for n in self._n])
            self.h = lib.skw_ref_accel_create_normals(npr, _ptr(self._mesh_of), nm, vp, _ptr(nv), tp, _ptr(nt), np_,
                                                      _ptr(self._x))
        self.n_tris = lib.skw_ref_accel_num_triangles(self.h)

    def instances(self):
        """(primitive int32 (n,), world_to_mesh float64 (n, 4, 4), subtree
        triangles int32 (n,)) in the accelerator's final instance order."""
        n = self.lib.skw_ref_accel_num_instances(self.h)
        p, m, c = np.zeros(n, np.int32), np.zeros((n, 4, 4)), np.zeros(n, np.int32)
        if n:
            self.lib.skw_ref_accel_export_instances(self.h, _ptr(p), _ptr(m), _ptr(c))
        return p, m, c

    def mesh_rank(self, n_meshes):
        """Rank of each mesh (numbered in order of first use) in the
        reference's address order of meshes."""
        r = np.zeros(n_meshes, np.int32)
        self.lib.skw_ref_accel_mesh_rank(self.h, _ptr(r))
        return r

    def meshes_ascending(self) -> bool:
        """The meshes' addresses ascend in creation order (the reference
        orders shared meshes by address)."""
        return bool(self.lib.skw_ref_accel_meshes_ascending(self.h))

    def intersect_d(self, rays, threads=0):
        """TriangleAccelerator::Intersect of double rays ((n, 8) float64)."""
        rays = np.ascontiguousarray(rays, np.float64)
        n = rays.shape[0]
        p, t, th = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.float64)
        self.lib.skw_ref_intersect_d(self.h, _ptr(rays), n, _ptr(p), _ptr(t), _ptr(th), threads)
        return {"prim": p, "tri": t, "t": th}

    def intersect_test_d(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float64)
        occ = np.empty(rays.shape[0], np.uint8)
        self.lib.skw_ref_intersect_test_d(self.h, _ptr(rays), rays.shape[0], _ptr(occ), threads)
        return occ

    def intersection(self, rays, diffs=None, next_dirs=None, threads=0):
        """The whole Intersection of each double ray ((n, 40) float64, see
        skw_ref_intersection) and, with next_dirs, GetNextMinT per hit."""
        rays = np.ascontiguousarray(rays, np.float64)
        n = rays.shape[0]
        d = None if diffs is None else np.ascontiguousarray(diffs, np.float64)
        nd = None if next_dirs is None else np.ascontiguousarray(next_dirs, np.float64)
        out = np.empty((n, 40), np.float64)
        nt = np.empty(n, np.float64) if nd is not None else None
        self.lib.skw_ref_intersection(self.h, _ptr(rays), _ptr(d), n, _ptr(out), _ptr(nd), _ptr(nt), threads)
        return (out, nt) if nd is not None else out

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.skw_ref_accel_destroy(self.h)
            self.h = None

    def export(self):
        nn = self.lib.skw_ref_accel_num_nodes(self.h)
        bbox = np.empty((nn, 6), np.float32)
        info = np.empty((nn, 8), np.int32)
        tp = np.empty(max(self.n_tris, 1), np.int32)
        ti = np.empty(max(self.n_tris, 1), np.int32)
        tr = np.empty((max(self.n_tris, 1), 9), np.float32)
        self.lib.skw_ref_accel_export(self.h, _ptr(bbox), _ptr(info), _ptr(tp), _ptr(ti), _ptr(tr))
        return bbox, info, tp[:self.n_tris], ti[:self.n_tris]

    def intersect(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        p, t, th = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.float64)
        self.lib.skw_ref_intersect(self.h, _ptr(rays), n, _ptr(p), _ptr(t), _ptr(th), threads)
        return {"prim": p, "tri": t, "t": th}

    def intersect_test(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        self.lib.skw_ref_intersect_test(self.h, _ptr(rays), n, _ptr(occ), threads)
        return occ


class RefKD:
    def __init__(self, lib, pos, normal_ids=None, dir_ids=None):
        self.lib = lib
        self.pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        n = self.pos.shape[0]
        self.nids = None if normal_ids is None else np.ascontiguousarray(normal_ids, np.uint16)
        self.dids = None if dir_ids is None else np.ascontiguousarray(dir_ids, np.uint16)
        self.perm = np.empty(n, np.int32)
        self.nodes = np.empty((n, 2), np.uint32)
        self.h = lib.skw_ref_kdtree_create(_ptr(self.pos), _ptr(self.nids), _ptr(self.dids), n, _ptr(self.perm),
                                           _ptr(self.nodes))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.skw_ref_kdtree_destroy(self.h)
            self.h = None

    def knn(self, q, qn, k, max_dist, cos_threshold=-1.0, threads=0):
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        qn = None if qn is None else np.ascontiguousarray(qn, np.float64).reshape(-1, 3)
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int32)
        d2 = np.empty((nq, k), np.float64)
        cnt = np.empty(nq, np.int32)
        self.lib.skw_ref_knn(self.h, _ptr(q), _ptr(qn), nq, k, max_dist, cos_threshold, _ptr(idx), _ptr(d2), _ptr(cnt),
                             threads)
        return {"idx": idx, "d2": d2, "count": cnt}

    def nearest(self, q, max_dist, threads=0):
        q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
        out = np.empty(q.shape[0], np.int32)
        self.lib.skw_ref_nearest(self.h, _ptr(q), q.shape[0], max_dist, _ptr(out), threads)
        return out


class RefMerl:
    """The reference's MERLMeasuredData / MERLMeasured on a file image."""

    def __init__(self, lib, data: bytes):
        self.lib = lib
        self.h = lib.skw_ref_merl_create(data, len(data))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.skw_ref_merl_destroy(self.h)
            self.h = None

    def export(self):
        t = np.empty((90 * 90 * 180, 3), np.uint16)
        sg = np.zeros((90, 1173), np.float32)
        self.lib.skw_ref_merl_export(self.h, _ptr(t), _ptr(sg))
        return t, sg

    def eval(self, wi, wo):
        wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
        wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
        f, pdf = np.empty_like(wi), np.empty(len(wi))
        self.lib.skw_ref_merl_eval(self.h, _ptr(wi), _ptr(wo), len(wi), _ptr(f), _ptr(pdf))
        return f, pdf

    def sample(self, wi, u):
        wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, np.float64).reshape(-1, 2)
        wo, f, pdf = np.empty_like(wi), np.empty_like(wi), np.empty(len(wi))
        self.lib.skw_ref_merl_sample(self.h, _ptr(wi), _ptr(u), len(wi), _ptr(wo), _ptr(f), _ptr(pdf))
        return wo, f, pdf
