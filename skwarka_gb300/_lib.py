"""ctypes binding of the in-tree C ABI library (include/skw.h).

Loading fails loudly: there is no CPU fallback.  The library is built by
``skwarka_gb300.build.build()`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libskw.so"

SKW_OK = 0
STATUS_NAMES = {
    0: "SKW_OK", 1: "SKW_ERR_ARG", 2: "SKW_ERR_CUDA", 3: "SKW_ERR_OOM", 4: "SKW_ERR_BUDGET",
    5: "SKW_ERR_STACK_OVERFLOW", 6: "SKW_ERR_UNSUPPORTED", 7: "SKW_ERR_NO_DEVICE",
}


class SkwError(RuntimeError):
    """A nonzero skw_status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class skw_mesh(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_int64),
                ("triangles", C.c_void_p), ("n_triangles", C.c_int64)]


class skw_primitive(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("mesh_to_world", C.c_void_p)]


class skw_accel_info(C.Structure):
    _fields_ = [("n_triangles", C.c_int64), ("n_nodes", C.c_int64), ("n_leaves", C.c_int64),
                ("max_depth", C.c_int32), ("stack_need", C.c_int32), ("bounds", C.c_float * 6),
                ("build_ms", C.c_double), ("device_bytes", C.c_int64), ("built_on_device", C.c_int32)]


# (name, restype, argtypes) for every symbol include/skw.h declares.
_P = C.c_void_p
SIGNATURES = [
    ("skw_version", C.c_int, []),
    ("skw_ctx_create", C.c_int, [C.c_int, C.POINTER(_P)]),
    ("skw_ctx_destroy", None, [_P]),
    ("skw_last_error", C.c_char_p, [_P]),
    ("skw_launch_count", C.c_int64, [_P]),
    ("skw_ctx_host_buffers_in_place", C.c_int, [_P]),
    ("skw_flat_tree_build", C.c_int, [C.POINTER(skw_mesh), C.c_int32, C.POINTER(skw_primitive), C.c_int32, C.c_int,
                                      C.POINTER(_P), C.c_char_p, C.c_size_t]),
    ("skw_flat_tree_build_device", C.c_int, [_P, C.POINTER(skw_mesh), C.c_int32, C.POINTER(skw_primitive), C.c_int32,
                                             C.c_int64, C.POINTER(_P), C.POINTER(C.c_int32)]),
    ("skw_flat_tree_destroy", None, [_P]),
    ("skw_flat_tree_sizes", C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    ("skw_flat_tree_export", C.c_int, [_P, _P, _P, _P, _P]),
    ("skw_flat_tree_instances", C.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    ("skw_flat_tree_leaf_ranges", C.c_int, [_P, C.c_uint32, _P]),
    ("skw_accel_create_from_flat", C.c_int, [_P, _P, C.POINTER(_P)]),
    ("skw_accel_create", C.c_int, [_P, C.POINTER(skw_mesh), C.c_int32, C.POINTER(skw_primitive), C.c_int32,
                                   C.POINTER(_P)]),
    ("skw_accel_destroy", None, [_P]),
    ("skw_accel_get_info", C.c_int, [_P, C.POINTER(skw_accel_info)]),
    ("skw_accel_rays_traced", C.c_int, [_P, C.POINTER(C.c_uint64)]),
    ("skw_accel_export", C.c_int, [_P, _P, _P, _P]),
    ("skw_intersect", C.c_int, [_P, _P, C.c_int64, _P, _P]),
    ("skw_intersect_test", C.c_int, [_P, _P, C.c_int64, _P, _P]),
    ("skw_intersect_host", C.c_int, [_P, _P, C.c_int64, _P]),
    ("skw_intersect_test_host", C.c_int, [_P, _P, C.c_int64, _P]),
    ("skw_intersect_d", C.c_int, [_P, _P, C.c_int64, _P, _P]),
    ("skw_intersect_test_d", C.c_int, [_P, _P, C.c_int64, _P, _P]),
    ("skw_intersect_d_host", C.c_int, [_P, _P, C.c_int64, _P]),
    ("skw_intersect_test_d_host", C.c_int, [_P, _P, C.c_int64, _P]),
    ("skw_compress_direction", C.c_uint16, [C.c_double, C.c_double, C.c_double]),
    ("skw_direction_table", C.c_int, [_P]),
    ("skw_kdtree_build_host", C.c_int, [_P, C.c_int64, C.c_int, _P, _P]),
    ("skw_kdtree_repair_host", C.c_int, [_P, C.c_int64, _P, C.c_int64, _P, _P]),
    ("skw_kdtree_build_device", C.c_int, [_P, _P, C.c_int64, _P, _P, C.POINTER(C.c_int32)]),
    ("skw_kdtree_create", C.c_int, [_P, _P, _P, C.c_int64, C.POINTER(_P)]),
    ("skw_kdtree_destroy", None, [_P]),
    ("skw_kdtree_size", C.c_int, [_P, C.POINTER(C.c_int64)]),
    ("skw_kdtree_permutation", C.c_int, [_P, _P]),
    ("skw_knn", C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, _P, _P, _P, _P]),
    ("skw_knn_noalloc", C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, _P, _P, _P, _P]),
    ("skw_knn_host", C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, C.c_double, C.c_double, _P, _P, _P]),
    ("skw_scene_create", C.c_int, [_P, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                   C.c_void_p, C.c_int32, C.POINTER(_P)]),
    ("skw_scene_destroy", None, [_P]),
    ("skw_scene_accel", _P, [_P]),
    ("skw_render_direct", C.c_int, [_P, C.c_void_p, C.c_void_p, _P, _P]),
    ("skw_photon_map_create", C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.POINTER(_P)]),
    ("skw_photon_shoot", C.c_int, [_P, C.c_void_p, C.POINTER(_P)]),
    ("skw_photon_map_destroy", None, [_P]),
    ("skw_photon_map_get_info", C.c_int, [_P, C.c_void_p]),
    ("skw_photon_map_export", C.c_int, [_P, C.c_int32, C.c_void_p]),
    ("skw_photon_map_export_irradiance", C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("skw_scene_total_area", C.c_double, [_P]),
    ("skw_merl_create", C.c_int, [_P, C.c_void_p, C.c_int64, C.POINTER(_P)]),
    ("skw_merl_destroy", None, [_P]),
    ("skw_merl_export", C.c_int, [_P, _P, _P]),
    ("skw_merl_eval_host", C.c_int, [_P, _P, _P, C.c_int64, _P, _P]),
    ("skw_merl_sample_host", C.c_int, [_P, _P, _P, C.c_int64, _P, _P, _P]),
    ("skw_scene_set_medium", C.c_int, [_P, C.c_void_p]),
    ("skw_scene_set_max_specular_depth", C.c_int, [_P, C.c_int32]),
    ("skw_scene_hit_geometry", C.c_int, [_P, _P, _P, C.c_int64, _P, _P]),
    ("skw_scene_intersection", C.c_int, [_P, _P, _P, C.c_int64, _P, _P]),
    ("skw_next_min_t", C.c_double, [_P, _P]),
    ("skw_scene_next_rays", C.c_int, [_P, _P, _P, _P, C.c_int64, _P, _P]),
    ("skw_render_photon", C.c_int, [_P, _P, C.c_void_p, C.c_void_p, C.c_void_p, _P, _P]),
    ("skw_scene_n_triangles", C.c_int64, [_P]),
    ("skw_scene_set_triangle_albedo", C.c_int, [_P, _P, _P]),
    ("skw_scene_set_emission_scale", C.c_int, [_P, C.c_float]),
    ("skw_render_direct_adjoint", C.c_int, [_P, C.c_void_p, C.c_void_p, _P, _P, _P, _P]),
    ("skw_render_batch_create", C.c_int, [_P, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(_P)]),
    ("skw_render_batch_destroy", None, [_P]),
    ("skw_render_batch_film_floats", C.c_int64, [_P]),
    ("skw_render_batch_film_offset", C.c_int64, [_P, C.c_int32]),
    ("skw_render_batch_get_config", C.c_int, [_P, C.c_void_p]),
    ("skw_render_batch_run", C.c_int, [_P, _P, _P]),
    ("skw_render_batch_autotune", C.c_int, [_P, _P, _P, C.c_void_p, C.POINTER(C.c_float),
                                            C.POINTER(C.c_int32)]),
    ("skw_nearest", C.c_int, [_P, _P, _P, C.c_int64, C.c_double, C.c_double, _P, _P]),
]

_lib = None


def load() -> C.CDLL:
    """Load libskw.so (once) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, ctx=None) -> None:
    if rc != SKW_OK:
        msg = load().skw_last_error(ctx).decode() if ctx else ""
        raise SkwError(rc, msg)
