"""Builds the reference's own CxxTest unit-test suites against the GPU
drop-in accelerator (skwarka_gb300/adapter: TriangleAccelerator.h / .cpp in
place of the reference's two files), linked with libskw.so.

The reference sources, its unit tests and its vendored CxxTest 4.4 are the
copies oracle/build_ref.py stages under oracle/_ref; this recipe lays an
overlay of that tree with the adapter's header in place of
Raytracer/Core/TriangleAccelerator.h (so that Scene.h and every other
includer see the drop-in), compiles every reference translation unit except
TriangleAccelerator.cpp against it, adds the adapter's .cpp and a CxxTest
runner generated from the chosen suites, and links.  Outputs go to
oracle/_ref/adapter (git-ignored).  Test infrastructure only."""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "oracle" / "_ref"
OUT = REF / "adapter"
ADAPTER = ROOT / "skwarka_gb300" / "adapter"
LIB_DIR = ROOT / "skwarka_gb300" / "_lib"
SUITES_DIR = "UnitTests/MainTests/Raytracer/Core"


def available() -> bool:
    return (REF / "src" / ".staged").exists() and (REF / "cxxtest" / "bin" / "cxxtestgen").exists()


def _overlay() -> Path:
    from oracle import build_ref
    src, ov = REF / "src", OUT / "src"
    stamp = ov / ".overlay"
    want = (src / ".staged").read_text() + (ADAPTER / "TriangleAccelerator.h").read_text()
    if not stamp.exists() or stamp.read_text() != want:
        if ov.exists():
            shutil.rmtree(ov)
        shutil.copytree(src, ov, symlinks=True)
        shutil.copyfile(ADAPTER / "TriangleAccelerator.h", ov / "Raytracer" / "Core" / "TriangleAccelerator.h")
        stamp.write_text(want)
    build_ref.make_shims()
    return ov


def _compile(args):
    src, obj, flags = args
    if obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime:
        return
    obj.parent.mkdir(parents=True, exist_ok=True)
    r = subprocess.run(["g++", *flags, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stderr[-3000:]}")


def build_runner(suites: list[str]) -> Path:
    """Compiles the runner of the given suites (file stems under
    UnitTests/MainTests/Raytracer/Core) against the drop-in; returns its path."""
    from oracle import build_ref
    ov = _overlay()
    cxx = REF / "cxxtest"
    flags = [*build_ref.CXXFLAGS, "-I", str(build_ref.SHIMS), "-I", str(ov), "-I", str(ov / "UnitTests"),
             "-I", str(cxx), "-I", str(ROOT / "include"), "-include", str(build_ref.SHIMS / "prelude.h")]
    digest = hashlib.sha256(" ".join(flags).encode()).hexdigest()[:16]
    obj = OUT / f"obj-{digest}"
    jobs = []
    for s in build_ref._sources():
        if s.name == "TriangleAccelerator.cpp":
            continue
        rel = s.relative_to(build_ref.SRC)
        jobs.append((ov / rel, obj / (str(rel).replace("/", "__") + ".o"), flags))
    jobs.append((ADAPTER / "TriangleAccelerator.cpp", obj / "adapter_TriangleAccelerator.o",
                 flags + ["-I", str(ov / "Raytracer" / "Core")]))
    name = "_".join(suites)
    runner_cpp = OUT / f"runner_{name}.cpp"
    headers = [str(ov / SUITES_DIR / f"{s}.test.h") for s in suites]
    r = subprocess.run([sys.executable, str(cxx / "bin" / "cxxtestgen"), "--error-printer", "-o", str(runner_cpp),
                        *headers], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cxxtestgen failed:\n{r.stderr[-3000:]}")
    jobs.append((runner_cpp, obj / f"runner_{name}.o", flags))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_compile, jobs))
    exe = OUT / f"runner_{name}"
    objs = [str(j[1]) for j in jobs]
    r = subprocess.run(["g++", "-pthread", "-o", str(exe), *objs, "-L", str(LIB_DIR), "-lskw",
                        f"-Wl,-rpath,{LIB_DIR}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-3000:]}")
    return exe


if __name__ == "__main__":
    sys.path.insert(0, str(ROOT))
    print(build_runner(sys.argv[1:] or ["TriangleAccelerator"]))
