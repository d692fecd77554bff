"""The C-ABI library loads and exports every entry point include/skw.h
declares; argument errors come back as status codes.  No GPU needed."""
import ctypes as C
import re
from pathlib import Path

import pytest

from skwarka_gb300 import _lib

HEADER_DIR = Path(__file__).resolve().parent.parent / "include"


def declared_functions():
    names = set()
    for h in HEADER_DIR.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(skw_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_symbols_exported(built):
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built):
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_version_and_null_args(built):
    lib = _lib.load()
    assert lib.skw_version() >= 100
    assert lib.skw_ctx_create(0, None) == 1  # SKW_ERR_ARG
    assert lib.skw_accel_get_info(None, None) == 1
    assert lib.skw_flat_tree_build(None, 0, None, 0, 0, None, None, 0) == 1
    assert lib.skw_scene_set_max_specular_depth(None, 3) == 1
    assert lib.skw_scene_hit_geometry(None, None, None, 0, None, None) == 1
    assert lib.skw_scene_set_medium(None, None) == 1


def test_ctx_without_gpu_reports_no_device(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.skw_ctx_create(0, C.byref(h)) == 7  # SKW_ERR_NO_DEVICE
