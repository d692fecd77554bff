"""The C++ host interface (include/skw.hpp) from a C++ program linked
against the library: tests/cpp/skw_hpp_test.cpp builds accelerators, a
photon kd-tree and a render scene through skwarka's C++ classes and checks
known answers (hits and t on two squares, one of them transformed;
occlusion against tmax; k-NN distances against brute force; a lit floor's
radiance range; a photon shoot's map sizes; an error code)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from skwarka_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def test_cpp_client(gpu, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    lib = Path(_lib.load()._name).parent
    exe = tmp_path / "skw_hpp_test"
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cpp" / "skw_hpp_test.cpp"), "-L", str(lib), "-lskw", "-L", str(CUDA / "lib64"),
           "-lcudart", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{CUDA / 'lib64'}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout.strip())
    assert r.returncode == 0 and "skw.hpp: OK" in r.stdout, r.stdout + r.stderr
