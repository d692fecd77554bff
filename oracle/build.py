"""Builds the oracle (test infrastructure): ``oracle/_build/libskw_oracle.so``
from ``oracle/skw_oracle.cpp``, and -- where the reference sources are
available -- ``oracle/_ref/libskw_ref.so`` via ``oracle/build_ref.py``."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libskw_oracle.so"
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-Wall"]


def build_oracle() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    src = HERE / "skw_oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        cmd = ["g++", *FLAGS, str(src), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


def build_all(verbose: bool = False):
    lib = build_oracle()
    from . import build_ref  # noqa: WPS433 (sibling module)
    ref = build_ref.build(verbose=verbose)
    if verbose:
        print(f"oracle: {lib}; reference: {ref}")
    return lib, ref


if __name__ == "__main__":
    import sys
    sys.path.insert(0, str(HERE.parent))
    from oracle import build_ref  # noqa: F401
    print(build_oracle())
    print(build_ref.build(verbose=True))
