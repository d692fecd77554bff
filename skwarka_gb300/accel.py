"""Host-side mirror of the reference's scene / accelerator interface.

``TriangleMesh``, ``Primitive`` and ``TriangleAccelerator`` follow the
reference classes of the same names (Raytracer/Core/TriangleMesh.h:82,
Primitive.h:48, TriangleAccelerator.h:35-57); the queries are batched:
``intersect`` answers ``TriangleAccelerator::Intersect`` for many rays at once
(closest hit: primitive index, mesh triangle index, t) and
``intersect_test`` answers ``IntersectTest`` (any hit in [tmin, tmax]).

Rays are ``(n, 8)`` float32 arrays ``ox oy oz dx dy dz tmin tmax``.  CUDA
tensors are processed in place on the current stream (device path); numpy
arrays go through the library's host-buffer entry points (copies included).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib


class Context:
    """One skw_ctx bound to a CUDA device."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.skw_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def launch_count(self) -> int:
        return int(_lib.load().skw_launch_count(self.handle))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_ctx_destroy(h)
            self.handle = None


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


@dataclass
class TriangleMesh:
    """float32 (nv, 3) vertices and int32 (nt, 3) vertex-index triangles."""
    vertices: np.ndarray
    triangles: np.ndarray

    def __post_init__(self):
        self.vertices = np.ascontiguousarray(self.vertices, dtype=np.float32).reshape(-1, 3)
        self.triangles = np.ascontiguousarray(self.triangles, dtype=np.int32).reshape(-1, 3)


@dataclass
class Primitive:
    """A mesh with an optional row-major 4x4 mesh-to-world matrix."""
    mesh: TriangleMesh
    mesh_to_world: np.ndarray | None = None
    material: object = field(default=None)

    def __post_init__(self):
        if self.mesh_to_world is not None:
            self.mesh_to_world = np.ascontiguousarray(self.mesh_to_world, dtype=np.float64).reshape(4, 4)


class TriangleAccelerator:
    """Ternary bbox kd-tree over the primitives' triangles, resident on the GPU."""

    def __init__(self, primitives: list[Primitive], ctx: Context | None = None):
        self.ctx = ctx or default_context()
        lib = _lib.load()
        meshes, mesh_ids, prims = [], {}, []
        for p in primitives:
            key = id(p.mesh)
            if key not in mesh_ids:
                mesh_ids[key] = len(meshes)
                meshes.append(p.mesh)
            prims.append(p)
        self._keep = []
        cm = (_lib.skw_mesh * max(len(meshes), 1))()
        for i, m in enumerate(meshes):
            cm[i] = _lib.skw_mesh(m.vertices.ctypes.data, m.vertices.shape[0], m.triangles.ctypes.data,
                                  m.triangles.shape[0])
        cp = (_lib.skw_primitive * max(len(prims), 1))()
        for i, p in enumerate(prims):
            xf = p.mesh_to_world.ctypes.data if p.mesh_to_world is not None else None
            cp[i] = _lib.skw_primitive(mesh_ids[id(p.mesh)], xf)
        h = C.c_void_p()
        _lib.check(lib.skw_accel_create(self.ctx.handle, cm, len(meshes), cp, len(prims), C.byref(h)),
                   self.ctx.handle)
        self.handle = h
        self.primitives = primitives
        info = _lib.skw_accel_info()
        _lib.check(lib.skw_accel_get_info(h, C.byref(info)), self.ctx.handle)
        self.info = {
            "n_triangles": info.n_triangles, "n_nodes": info.n_nodes, "n_leaves": info.n_leaves,
            "max_depth": info.max_depth, "stack_need": info.stack_need, "bounds": list(info.bounds),
            "build_ms": info.build_ms, "device_bytes": info.device_bytes,
            "built_on_device": bool(info.built_on_device),
        }

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and not getattr(self, "_borrowed", False):
            _lib.load().skw_accel_destroy(h)
        self.handle = None

    def rays_traced(self) -> int:
        """Rays traced so far by every launch on this accelerator (waits for the device)."""
        v = C.c_uint64()
        _lib.check(_lib.load().skw_accel_rays_traced(self.handle, C.byref(v)), self.ctx.handle)
        return int(v.value)

    def export(self):
        """(nodes uint32 (n_nodes, 8), tri_prim int32, tri_index int32) of the flattened tree."""
        nn, nt = self.info["n_nodes"], self.info["n_triangles"]
        nodes = np.zeros((nn, 8), np.uint32)
        tp = np.zeros(max(nt, 1), np.int32)
        ti = np.zeros(max(nt, 1), np.int32)
        _lib.check(_lib.load().skw_accel_export(self.handle, nodes.ctypes.data, tp.ctypes.data, ti.ctypes.data),
                   self.ctx.handle)
        return nodes, tp[:nt], ti[:nt]

    # ------------------------------------------------------------ queries --
    def intersect(self, rays, stream=None):
        """Closest hits.  CUDA tensor (n, 8) -> int32 CUDA tensor (n, 4) holding
        (t as float bits, prim, tri, flags); numpy -> dict of numpy arrays."""
        if isinstance(rays, np.ndarray):
            r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
            hits = np.zeros((r.shape[0], 4), np.int32)
            _lib.check(_lib.load().skw_intersect_host(self.handle, r.ctypes.data, r.shape[0], hits.ctypes.data),
                       self.ctx.handle)
            return unpack_hits(hits)
        import torch
        assert rays.is_cuda and rays.dtype == torch.float32 and rays.is_contiguous() and rays.shape[-1] == 8
        n = rays.numel() // 8
        hits = torch.empty((n, 4), dtype=torch.int32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        _lib.check(_lib.load().skw_intersect(self.handle, rays.data_ptr(), n, hits.data_ptr(), s), self.ctx.handle)
        return hits

    def intersect_d(self, rays, stream=None):
        """Closest hits of double rays (skw_ray_d: (n, 8) float64 ox oy oz dx dy
        dz tmin tmax), the reference's exact t.  numpy in -> dict of numpy
        (prim, tri, t); CUDA tensor in -> (n, 2) float64 CUDA tensor of
        skw_hit_d records (t, then prim and tri as the bits of the second
        double; unpack_hits_d reads them)."""
        lib = _lib.load()
        if isinstance(rays, np.ndarray):
            r = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 8)
            hits = np.zeros((r.shape[0], 2), np.float64)
            _lib.check(lib.skw_intersect_d_host(self.handle, r.ctypes.data, r.shape[0], hits.ctypes.data),
                       self.ctx.handle)
            return unpack_hits_d(hits)
        import torch
        assert rays.is_cuda and rays.dtype == torch.float64 and rays.is_contiguous() and rays.shape[-1] == 8
        n = rays.numel() // 8
        hits = torch.empty((n, 2), dtype=torch.float64, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        _lib.check(lib.skw_intersect_d(self.handle, rays.data_ptr(), n, hits.data_ptr(), s), self.ctx.handle)
        return hits

    def intersect_test_d(self, rays, stream=None):
        """Any hit of double rays: uint8 0/1 per ray (numpy in -> numpy out)."""
        lib = _lib.load()
        if isinstance(rays, np.ndarray):
            r = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 8)
            occ = np.zeros(r.shape[0], np.uint8)
            _lib.check(lib.skw_intersect_test_d_host(self.handle, r.ctypes.data, r.shape[0], occ.ctypes.data),
                       self.ctx.handle)
            return occ
        import torch
        n = rays.numel() // 8
        occ = torch.empty((n,), dtype=torch.uint8, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        _lib.check(lib.skw_intersect_test_d(self.handle, rays.data_ptr(), n, occ.data_ptr(), s), self.ctx.handle)
        return occ

    def intersect_test(self, rays, stream=None):
        """Any hit in [tmin, tmax]: uint8 0/1 per ray (numpy in -> numpy out)."""
        if isinstance(rays, np.ndarray):
            r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
            occ = np.zeros(r.shape[0], np.uint8)
            _lib.check(_lib.load().skw_intersect_test_host(self.handle, r.ctypes.data, r.shape[0], occ.ctypes.data),
                       self.ctx.handle)
            return occ
        import torch
        assert rays.is_cuda and rays.dtype == torch.float32 and rays.is_contiguous() and rays.shape[-1] == 8
        n = rays.numel() // 8
        occ = torch.empty((n,), dtype=torch.uint8, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        _lib.check(_lib.load().skw_intersect_test(self.handle, rays.data_ptr(), n, occ.data_ptr(), s),
                   self.ctx.handle)
        return occ


def unpack_hits(hits) -> dict:
    """Split an (n, 4) int32 hit array (numpy or tensor) into t/prim/tri/flags."""
    if not isinstance(hits, np.ndarray):
        hits = hits.cpu().numpy()
    hits = np.ascontiguousarray(hits, dtype=np.int32)
    return {"t": hits[:, 0].view(np.float32).copy(), "prim": hits[:, 1].copy(), "tri": hits[:, 2].copy(),
            "flags": hits[:, 3].view(np.uint32).copy()}


def build_flat_tree(primitives: list[Primitive], threads: int = 0, device: Context | None = None,
                    min_device_triangles: int = 0) -> dict:
    """Tree build, flattened into the device layout as numpy arrays -- nodes
    uint32 (n, 8), tris float32 (n, 9), tri_prim, tri_index -- plus
    max_depth.  On the host (no GPU needed), or with ``device`` given on that
    context's GPU (``on_device`` in the result tells whether the GPU built it:
    instancing, or fewer than ``min_device_triangles`` triangles, builds on
    the host)."""
    lib = _lib.load()
    meshes, mesh_ids = [], {}
    for p in primitives:
        if id(p.mesh) not in mesh_ids:
            mesh_ids[id(p.mesh)] = len(meshes)
            meshes.append(p.mesh)
    cm = (_lib.skw_mesh * max(len(meshes), 1))()
    for i, m in enumerate(meshes):
        cm[i] = _lib.skw_mesh(m.vertices.ctypes.data, m.vertices.shape[0], m.triangles.ctypes.data,
                              m.triangles.shape[0])
    cp = (_lib.skw_primitive * max(len(primitives), 1))()
    for i, p in enumerate(primitives):
        xf = p.mesh_to_world.ctypes.data if p.mesh_to_world is not None else None
        cp[i] = _lib.skw_primitive(mesh_ids[id(p.mesh)], xf)
    h = C.c_void_p()
    on_dev = C.c_int32(0)
    if device is not None:
        _lib.check(lib.skw_flat_tree_build_device(device.handle, cm, len(meshes), cp, len(primitives),
                                                  min_device_triangles, C.byref(h), C.byref(on_dev)), device.handle)
    else:
        err = C.create_string_buffer(256)
        rc = lib.skw_flat_tree_build(cm, len(meshes), cp, len(primitives), threads, C.byref(h), err, 256)
        if rc != _lib.SKW_OK:
            raise _lib.SkwError(rc, err.value.decode())
    try:
        nn, nt, md = C.c_int64(), C.c_int64(), C.c_int32()
        _lib.check(lib.skw_flat_tree_sizes(h, C.byref(nn), C.byref(nt), C.byref(md)))
        nodes = np.zeros((nn.value, 8), np.uint32)
        tris = np.zeros((max(nt.value, 1), 9), np.float32)
        tp = np.zeros(max(nt.value, 1), np.int32)
        ti = np.zeros(max(nt.value, 1), np.int32)
        _lib.check(lib.skw_flat_tree_export(h, nodes.ctypes.data, tris.ctypes.data, tp.ctypes.data, ti.ctypes.data))
        ni, ns = C.c_int64(), C.c_int64()
        _lib.check(lib.skw_flat_tree_instances(h, C.byref(ni), None, None, None, C.byref(ns), None))
        ip = np.zeros(max(ni.value, 1), np.int32)
        ir = np.zeros(max(ni.value, 1), np.uint32)
        im = np.zeros((max(ni.value, 1), 4, 4), np.float64)
        sr = np.zeros(max(ns.value, 1), np.uint32)
        _lib.check(lib.skw_flat_tree_instances(h, None, ip.ctypes.data, ir.ctypes.data, im.ctypes.data, None,
                                               sr.ctypes.data))
        ext = {}
        for i in np.nonzero((nodes[:, 7] & 3 == 0) & (nodes[:, 7] & 0x80 != 0))[0]:
            r = np.zeros(4, np.uint32)
            _lib.check(lib.skw_flat_tree_leaf_ranges(h, int(nodes[i, 6]), r.ctypes.data))
            ext[int(i)] = tuple(int(x) for x in r)
    finally:
        lib.skw_flat_tree_destroy(h)
    n = nt.value
    return {"nodes": nodes, "tris": tris[:n], "tri_prim": tp[:n], "tri_index": ti[:n], "max_depth": md.value,
            "inst_prim": ip[:ni.value], "inst_root": ir[:ni.value], "inst_world_to_mesh": im[:ni.value],
            "subtree_roots": sr[:ns.value], "leaf_ranges": ext, "on_device": bool(on_dev.value)}


def unpack_hits_d(hits) -> dict:
    """skw_hit_d records ((n, 2) float64, numpy or CUDA) -> dict of numpy
    arrays: prim, tri (int32) and t (float64)."""
    h = hits.cpu().numpy() if hasattr(hits, "cpu") else np.asarray(hits)
    h = np.ascontiguousarray(h, np.float64).reshape(-1, 2)
    ids = h[:, 1].copy().view(np.int32).reshape(-1, 2)
    return {"prim": ids[:, 0].copy(), "tri": ids[:, 1].copy(), "t": h[:, 0].copy()}
