"""Builds the in-tree shared library ``skwarka_gb300/_lib/libskw.so``.

CUDA translation units are compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host translation units with
g++.  Host code is compiled with ``-ffp-contract=off`` so that the
kd-tree builder rounds identically on x86-64 and aarch64.  Translation units
compile in parallel; a unit is rebuilt when it or any header is newer than its
object file, or when the flags change.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = OUT / "obj"
LIB = OUT / "libskw.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]
# Extra device-compiler flags, e.g. the kernels' tuning macros
# (SKW_KNN_BLOCK, SKW_TRAV_SCAP, ...) for a sweep; a change rebuilds every unit.
NVCC_FLAGS += os.environ.get("SKW_NVCC_EXTRA", "").split()
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall", "-Wno-unused-function",
             "-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(CUDA_HOME / "include")]


def _units() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path, hdr_mtime: float, flags_changed: bool) -> Path:
    obj = OBJ / (src.name + ".o")
    if (not flags_changed and obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime)):
        return obj
    if src.suffix == ".cu":
        cmd = [NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    """Compile every translation unit and link libskw.so; returns its path."""
    if not Path(NVCC).exists() and shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build skwarka_gb300")
    OBJ.mkdir(parents=True, exist_ok=True)
    stamp = OBJ / ".flags"
    flags_sig = " ".join(NVCC_FLAGS + CXX_FLAGS)
    flags_changed = not stamp.exists() or stamp.read_text() != flags_sig
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    hdr_mtime = max((h.stat().st_mtime for h in headers), default=0.0)
    units = _units()
    with ThreadPoolExecutor(max_workers=max(1, min(len(units), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_mtime, flags_changed), units))
    stamp.write_text(flags_sig)
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest or flags_changed:
        cmd = [NVCC, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
