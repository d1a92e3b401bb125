"""Build libkapdqmc_gpu.so in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel),
then linked into ``kapdqmc_gb300/libkapdqmc_gpu.so``.  Objects go to
``kapdqmc_gb300/_build/``.  A rebuild happens only when a source or header is
newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libkapdqmc_gpu.so"
INCLUDE = PKG.parent / "include"
UNITS = ["kdq_runtime.cu", "kdq_tu.cu", "kdq_tv.cu", "kdq_tuv.cu", "kdq_tu_mx.cu", "kdq_tv_mx.cu",
         "kdq_tuv_mx.cu", "kdq_grover.cu", "kdq_noalloc.cu", "kdq_cnn.cu",
         "kdq_scee.cu", "kdq_scee_1.cu", "kdq_scee_3.cu", "kdq_scee_6.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()

    def compile_one(u: str) -> Path:
        obj = BUILD / (u.rsplit(".", 1)[0] + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", str(CSRC / u), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
