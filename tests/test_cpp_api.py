"""The C++ host interface (include/skw.hpp) compiles cleanly against the C
ABI with a strict g++ (no GPU needed); tests/cpp/skw_hpp_test.cpp is its
client, run on the GPU by test_cpp_api_gpu.py."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA_INC = Path("/usr/local/cuda/include")


def test_skw_hpp_compiles():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
           "-I", str(CUDA_INC), str(ROOT / "tests" / "cpp" / "skw_hpp_test.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
