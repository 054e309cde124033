"""Build recipe for the CUDA library (sm_103a) and the CPU oracle.

Compiles every translation unit of ``csrc/`` in parallel with nvcc for
``sm_103a`` and links ``libmhfem_gb300.so`` in-tree; compiles the oracle
(``oracle/mhfem_oracle.c``) with gcc into ``oracle/liboracle_mhfem.so``.
No cmake, no torch extension machinery: plain nvcc/gcc command lines.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "libmhfem_gb300.so"
ORACLE_DIR = REPO_DIR / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle_mhfem.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")
    return found


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [REPO_DIR / "include" / "mhfem.h"]
    srcs = _sources()
    objs = []
    jobs = []
    for src in srcs:
        obj = BUILD_DIR / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp",
                   "-I", str(REPO_DIR / "include"), "-c", str(src), "-o", str(obj)]
            if src.suffix == ".cu":
                cmd += ["--expt-relaxed-constexpr", "-Xptxas", "-v"] if verbose else ["--expt-relaxed-constexpr"]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        _run([nvcc, "-shared", *ARCH, "-o", str(LIB_PATH), *map(str, objs), "-Xcompiler", "-fopenmp",
              "-lgomp", "-lcudart"])
    return LIB_PATH


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "mhfem_oracle.c"
    hdr = ORACLE_DIR / "mhfem_oracle.h"
    if force or _stale(ORACLE_LIB, [src, hdr]):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-std=c11", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", str(ORACLE_LIB), str(src), "-lm"])
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB_PATH)
    print(ORACLE_LIB)
