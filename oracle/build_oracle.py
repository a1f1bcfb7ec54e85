"""Build the CPU oracle (test infrastructure; the product never loads it).

g++ -O2 -ffp-contract=off: IEEE binary32 arithmetic with no fused multiply-add,
so every operation rounds like the WGSL expression it restates.  Output:
``oracle/_build/libmboracle.so``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libmboracle.so"
SRC = HERE / "oracle.cpp"
DEPS = [SRC, HERE / "oracle.h", HERE.parent / "include" / "millionsball.h", Path(__file__)]


def build(force: bool = False) -> Path:
    import fcntl

    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(force)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(force: bool) -> Path:
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in DEPS):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = BUILD / (LIB.name + ".tmp")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
