"""Recipe that compiles the reference renderer's own C++ sources into
``oracle/_ref/libskw_ref.so`` -- test infrastructure, never product code.

What it does:

1. Staging (only where the reference tree is mounted): copies the
   ``Source/RayLibs/{Common,Math,Raytracer,Shapes}`` sources into
   ``oracle/_ref/src`` and applies the mechanical, semantics-preserving
   rewrites g++ needs (the reference targets MSVC 2013):

   * ``X.swap(std::vector<T>())`` (binds a temporary to a non-const
     reference, an MSVC extension) becomes ``std::vector<T>().swap(X)``
     (``Raytracer/Core/TriangleAccelerator.cpp:145-146``,
     ``Raytracer/LTEIntegrators/PhotonLTEIntegrator/PhotonShootingPipeline.cpp:347,357,367``);
   * ``Texture()`` in the constructors of the texture class templates becomes
     ``Texture<T>()`` (``Raytracer/Textures/{Constant,Mix,Scale,Windy,Wrinkled}Texture.h``);
   * a ``MAth`` -> ``Math`` alias for a case typo
     (``PhotonInternalTypes.h:23``);
   * the unit tests' ``VolumeRegionMock`` constructor takes its spectra by
     const reference (``UnitTests/Mocks/VolumeRegionMock.h:30``; the tests
     pass temporaries).

   The staged copy (plus the reference's unit tests and its vendored CxxTest
   4.4, which the drop-in tests compile against the GPU accelerator) is
   git-ignored; it exists so that the same build can be repeated on a
   machine without the reference tree.
2. Shim headers (``oracle/ref_shims``) stand in for Windows, the MSVC debug
   CRT, Boost (``mt19937``, ``intrusive_ptr``) and TBB (a real thread pool).
   The MSVC-style ``<a\\b.h>`` includes are satisfied by files whose names
   contain a literal backslash, generated into ``oracle/_ref/shims``.
3. Compiles every translation unit except the three that need FreeImage or
   do not compile upstream (``ImageEnvironmentalLight.cpp``,
   ``RGBImageSource.cpp``, ``TranslucentMaterial.cpp``; none is on the
   ray-query / light-transport path), plus ``oracle/ref_driver.cpp`` (our
   C-ABI shim over the reference classes), into one shared library.

Usage: ``python oracle/build_ref.py [SKWARKA_SOURCE_ROOT]`` (idempotent;
rebuilds changed files).  The source root defaults to $SKW_REFERENCE_ROOT,
then to a checkout named ``reference`` beside this repository.
"""
from __future__ import annotations

import hashlib
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = OUT / "src"
SHIMS = OUT / "shims"
OBJ = OUT / "obj"
LIB = OUT / "libskw_ref.so"
def reference_root(arg: str | None = None) -> Path:
    """The Skwarka source tree: the given path, else $SKW_REFERENCE_ROOT,
    else a checkout named ``reference`` beside this repository."""
    if arg:
        return Path(arg)
    if os.environ.get("SKW_REFERENCE_ROOT"):
        return Path(os.environ["SKW_REFERENCE_ROOT"])
    return HERE.parent.parent / "reference"


REFERENCE: Path | None = None
SUBDIRS = ("Common", "Math", "Raytracer", "Shapes", "UnitTests")
CXXTEST = OUT / "cxxtest"  # the reference's vendored CxxTest 4.4 (its unit-test framework)
STAGE_VERSION = "staged 3: RayLibs sources, unit tests, CxxTest\n"
EXCLUDE = {"ImageEnvironmentalLight.cpp", "RGBImageSource.cpp", "TranslucentMaterial.cpp", "dllmain.cpp"}
# -ffp-contract=off: no fused multiply-add, so that an aarch64 build rounds
# exactly like the x86-64 (SSE2) build the reference targets.
# -fsigned-char: the reference counts down with `char` loop indices
# (Math/Matrix4x4.h:305, `for (char j=3;j>=0;--j)`), which never ends where
# plain char is unsigned (aarch64); x86-64 char is signed.
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-fpermissive", "-w", "-DNDEBUG", "-DNOMINMAX", "-pthread",
            "-ffp-contract=off", "-fsigned-char"]


def _rewrite(path: Path) -> None:
    text = path.read_text(encoding="latin-1")
    orig = text
    # X.swap(std::vector<T>())  ->  std::vector<T>().swap(X)
    text = re.sub(r"(\w+)\.swap\((std::vector<\w+>)\(\)\)", r"\2().swap(\1)", text)
    if path.parent.name == "Textures" and path.suffix == ".h":
        text = re.sub(r"^Texture\(\),", "Texture<T>(),", text, flags=re.M)
    if path.name == "VolumeRegionMock.h":
        # the unit tests pass temporaries to non-const reference parameters
        # (an MSVC extension): take them by const reference
        text = re.sub(r"(\w+) &i_(emission|absorption|scattering)", r"const \1 &i_\2", text)
    if text != orig:
        path.write_text(text, encoding="latin-1")


def stage() -> None:
    """Copy + patch the reference sources (only where the reference exists)."""
    root = (REFERENCE or reference_root()) / "Source" / "RayLibs"
    if not root.is_dir():
        return
    stamp = SRC / ".staged"
    if stamp.exists() and stamp.read_text() == STAGE_VERSION:
        return
    if SRC.exists():
        shutil.rmtree(SRC)
    if CXXTEST.exists():
        shutil.rmtree(CXXTEST)
    for sub in SUBDIRS:
        shutil.copytree(root / sub, SRC / sub)
    cxx = (REFERENCE or reference_root()) / "ThirdParty" / "cxxtest" / "4.4"
    if cxx.is_dir():
        shutil.copytree(cxx, CXXTEST)
    for p in SRC.rglob("*"):
        if p.suffix in (".h", ".cpp") and p.is_file():
            _rewrite(p)
    (SRC / "MAth").symlink_to("Math")
    stamp.write_text(STAGE_VERSION)


def make_shims() -> None:
    SHIMS.mkdir(parents=True, exist_ok=True)
    src = HERE / "ref_shims"
    for p in src.rglob("*"):
        if p.is_file():
            dst = SHIMS / p.relative_to(src)
            dst.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(p, dst)
    fwd = {
        "boost\\random\\mersenne_twister.hpp": '#include "boost/mt19937.hpp"\n',
        "tbb/atomic.h": '#include "tbb.h"\n',
        "tbb/pipeline.h": '#include "tbb.h"\n',
        "tbb/parallel_invoke.h": '#include "tbb.h"\n',
        "tbb/tick_count.h": '#include "tbb.h"\n',
        "tbb\\enumerable_thread_specific.h": '#include "tbb/tbb.h"\n',
        "tbb\\cache_aligned_allocator.h": '#include "tbb/tbb.h"\n',
        "Common\\Common.h": "#include <Common/Common.h>\n",
    }
    for name, body in fwd.items():
        (SHIMS / name).write_text(body)


def _sources() -> list[Path]:
    out = []
    for sub in SUBDIRS:
        for p in sorted((SRC / sub).rglob("*.cpp")):
            if p.name in EXCLUDE or "UnitTests" in p.parts:
                continue
            out.append(p)
    return out


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    if obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime:
        return
    obj.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", *CXXFLAGS, "-I", str(SHIMS), "-I", str(SRC), "-include", str(SHIMS / "prelude.h"),
           *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle reference build failed on {src}:\n{r.stderr[-4000:]}")


def build(verbose: bool = False) -> Path | None:
    """Build oracle/_ref/libskw_ref.so; returns its path, or None when no
    staged reference sources are available on this machine."""
    stage()
    if not (SRC / ".staged").exists():
        return None
    if (SRC / ".staged").read_text() != STAGE_VERSION:
        raise RuntimeError("the staged reference sources are from an older recipe and the reference tree is absent")
    make_shims()
    # The objects depend on the flags and on every shim header: a change to
    # either rebuilds everything.
    digest = hashlib.sha256(" ".join(CXXFLAGS).encode())
    for p in sorted((HERE / "ref_shims").rglob("*")):
        if p.is_file():
            digest.update(str(p.relative_to(HERE)).encode() + p.read_bytes())
    stamp_text = digest.hexdigest()
    flags_stamp = OBJ / ".flags"
    if OBJ.exists() and (not flags_stamp.exists() or flags_stamp.read_text() != stamp_text):
        shutil.rmtree(OBJ)
    OBJ.mkdir(parents=True, exist_ok=True)
    flags_stamp.write_text(stamp_text)
    srcs = _sources()
    jobs = [(s, OBJ / (str(s.relative_to(SRC)).replace("/", "__") + ".o"), []) for s in srcs]
    jobs.append((HERE / "ref_driver.cpp", OBJ / "ref_driver.o", []))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(lambda j: _compile(*j), jobs))
    objs = [str(j[1]) for j in jobs]
    newest = max(Path(o).stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = ["g++", "-shared", "-pthread", "-o", str(LIB), *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle reference link failed:\n{r.stderr[-4000:]}")
    if verbose:
        print(f"built {LIB} from {len(srcs)} reference translation units")
    return LIB


if __name__ == "__main__":
    if len(sys.argv) > 1:
        REFERENCE = reference_root(sys.argv[1])
    p = build(verbose=True)
    if p is None:
        print("reference sources not available; nothing built", file=sys.stderr)
