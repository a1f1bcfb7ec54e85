"""Build recipe for libmillionsball.so (sm_103a) and, separately, the CPU oracle.

The CUDA library is compiled in-tree with plain nvcc (one process per
translation unit, in parallel) and linked into
``bevy_millions_ball_gb300/_build/libmillionsball.so``.  The physics translation
unit is compiled with ``--fmad=false`` so that every float operation rounds like
the shader expression it restates.

The oracle (test infrastructure) is built by ``oracle/build_oracle.py``; this
module only builds the product.
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
BUILD = PKG / "_build"
LIB = BUILD / "libmillionsball.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]
# translation unit -> extra flags
UNITS = {
    "mb_api.cu": [],
    "mb_sort.cu": [],
    "mb_count.cu": [],
    "mb_static.cu": [],
    "mb_segs.cu": [],
    "mb_render.cu": ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
    "mb_batch.cu": [],
    "mb_physics.cu": ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
}
HEADERS = [CSRC / "mb_internal.h", CSRC / "mb_count_dev.cuh", ROOT / "include" / "millionsball.h"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmillionsball")
    return cand


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA translation unit for sm_103a and link the shared library.

    Serialised across processes with a lock file (several ranks may call it)."""
    import fcntl

    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(force, verbose)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(force: bool, verbose: bool) -> Path:
    cc = nvcc()
    objs: list[Path] = []
    jobs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *HEADERS, Path(__file__)]):
            cmd = [cc, *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
                if verbose:
                    print(" ".join(cmd))
                fut.result()
    if force or jobs or _stale(LIB, objs):
        tmp = BUILD / (LIB.name + ".tmp")
        _run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
