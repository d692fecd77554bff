"""Host-side mirror of the reference's photon kd-tree interface.

``PhotonKDTree`` stands in for ``KDTree<Photon>`` (Raytracer/Core/KDTree.h):
construction permutes the photons into tree order exactly as the reference
does, and the batched ``get_nearest_points`` / ``get_nearest_point`` answer
``GetNearestPoints`` / ``GetNearestPoint`` (optionally with the photon
normal/tangent-plane filter, PhotonInternalTypes.h:113-137) for many queries
at once.  Returned indices are tree positions, like the reference's pointers
into its permuted array; ``perm`` maps them to input order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .accel import Context, default_context


def compress_direction(v) -> int:
    """16-bit id of a unit vector (CompressedDirection)."""
    return int(_lib.load().skw_compress_direction(float(v[0]), float(v[1]), float(v[2])))


def compress_directions(vs: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    return np.array([lib.skw_compress_direction(float(a), float(b), float(c)) for a, b, c in np.asarray(vs)],
                    np.uint16)


def direction_table() -> np.ndarray:
    out = np.empty((1 << 16, 3), np.float64)
    _lib.check(_lib.load().skw_direction_table(out.ctypes.data))
    return out


def build_host(positions: np.ndarray, threads: int = 0):
    """Host-only build (no GPU): (perm int32 (n,), node_words uint32 (n, 2))."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    perm = np.empty(n, np.int32)
    nodes = np.empty((n, 2), np.uint32)
    _lib.check(_lib.load().skw_kdtree_build_host(pos.ctypes.data, n, threads, perm.ctypes.data, nodes.ctypes.data))
    return perm, nodes


def repair_host(positions: np.ndarray, ties, perm: np.ndarray, nodes: np.ndarray):
    """The host half of the GPU build: (perm, node_words) of a tree equal to
    the reference's except below the tie nodes at tree positions `ties`,
    remade there (the paths from the root to them and their subtrees) as the
    host build makes them.  Returns new arrays."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    t = np.ascontiguousarray(ties, np.int32)
    p = np.array(perm, np.int32, copy=True)
    w = np.array(nodes, np.uint32, copy=True).reshape(n, 2)
    _lib.check(_lib.load().skw_kdtree_repair_host(pos.ctypes.data, n, t.ctypes.data if len(t) else None, len(t),
                                                   p.ctypes.data, w.ctypes.data))
    return p, w


def build_device(positions: np.ndarray, ctx: Context | None = None):
    """The GPU build: (perm int32 (n,), node_words uint32 (n, 2), median_tie
    int), equal to build_host's outputs; median_tie counts the nodes whose
    median ties on its split axis (their subtrees are remade on the host)."""
    ctx = ctx or default_context()
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    perm = np.empty(n, np.int32)
    nodes = np.empty((n, 2), np.uint32)
    tie = C.c_int32()
    _lib.check(_lib.load().skw_kdtree_build_device(ctx.handle, pos.ctypes.data, n, perm.ctypes.data,
                                                    nodes.ctypes.data, C.byref(tie)), ctx.handle)
    return perm, nodes, int(tie.value)


class PhotonKDTree:
    def __init__(self, positions: np.ndarray, normal_ids: np.ndarray | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        nid = None if normal_ids is None else np.ascontiguousarray(normal_ids, np.uint16)
        h = C.c_void_p()
        lib = _lib.load()
        _lib.check(lib.skw_kdtree_create(self.ctx.handle, pos.ctypes.data, None if nid is None else nid.ctypes.data,
                                         pos.shape[0], C.byref(h)), self.ctx.handle)
        self.handle = h
        self.n = pos.shape[0]
        self.perm = np.empty(self.n, np.int32)
        _lib.check(lib.skw_kdtree_permutation(h, self.perm.ctypes.data if self.n else None), self.ctx.handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.load().skw_kdtree_destroy(h)
            self.handle = None

    def get_nearest_points(self, q, qn, k: int, max_dist: float = np.inf, cos_threshold: float = -1.0, stream=None):
        """numpy in -> dict of numpy (idx (nq, k), d2 (nq, k), count (nq,)) via
        the host-buffer entry point; CUDA float64 tensors in -> tensors out."""
        lib = _lib.load()
        if isinstance(q, np.ndarray):
            q = np.ascontiguousarray(q, np.float64).reshape(-1, 3)
            qn = None if qn is None else np.ascontiguousarray(qn, np.float64).reshape(-1, 3)
            nq = q.shape[0]
            idx = np.empty((nq, k), np.int32)
            d2 = np.empty((nq, k), np.float64)
            cnt = np.empty(nq, np.int32)
            _lib.check(lib.skw_knn_host(self.handle, q.ctypes.data, None if qn is None else qn.ctypes.data, nq, k,
                                        max_dist, cos_threshold, idx.ctypes.data, d2.ctypes.data, cnt.ctypes.data),
                       self.ctx.handle)
            return {"idx": idx, "d2": d2, "count": cnt}
        import torch
        nq = q.numel() // 3
        idx = torch.empty((nq, k), dtype=torch.int32, device=q.device)
        d2 = torch.empty((nq, k), dtype=torch.float64, device=q.device)
        cnt = torch.empty((nq,), dtype=torch.int32, device=q.device)
        s = stream if stream is not None else torch.cuda.current_stream(q.device).cuda_stream
        _lib.check(lib.skw_knn(self.handle, q.data_ptr(), None if qn is None else qn.data_ptr(), nq, k, max_dist,
                               cos_threshold, idx.data_ptr(), d2.data_ptr(), cnt.data_ptr(), s), self.ctx.handle)
        return {"idx": idx, "d2": d2, "count": cnt}

    def get_nearest_point(self, q, qn=None, max_dist: float = np.inf, cos_threshold: float = -1.0, stream=None):
        """CUDA float64 (nq, 3) tensor -> int32 tensor of tree positions (-1: none)."""
        import torch
        nq = q.numel() // 3
        out = torch.empty((nq,), dtype=torch.int32, device=q.device)
        s = stream if stream is not None else torch.cuda.current_stream(q.device).cuda_stream
        _lib.check(_lib.load().skw_nearest(self.handle, q.data_ptr(), None if qn is None else qn.data_ptr(), nq,
                                           max_dist, cos_threshold, out.data_ptr(), s), self.ctx.handle)
        return out
