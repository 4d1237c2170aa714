"""Build the in-tree CUDA library ``cpmd_gb300/libcpmd_gb300.so`` for sm_103a.

Plain nvcc, one object per translation unit compiled in parallel, then one
shared-library link.  No torch extension machinery: the library exports the
C ABI of ``include/cpmd_gb300.h`` and is loaded with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcpmd_gb300.so"
SOURCES = ["band.cu", "band64.cu", "band32.cu", "linalg.cu", "chol.cu", "ozaki.cu", "nonlocal.cu", "tc_gemm.cu", "energy.cu", "batch.cu", "rortho.cu", "abi.cu", "restart.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-lineinfo", "-Xptxas=-O3",
            "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-math-errno", *ARCH, *extra]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "cpmd_gb300.h"]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = CSRC / s
        obj = BUILD / (s + ".o")
        if force or ptxas_info or _stale(obj, src):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append((src, obj, [cc, *_flags(extra), "-c", str(src), "-o", str(obj)]))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): (src, obj) for src, obj, cmd in jobs}
            for fut in cf.as_completed(futs):
                r = fut.result()
                src, _ = futs[fut]
                if verbose or ptxas_info or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {src.name}")
    objs = [str(BUILD / (s + ".o")) for s in SOURCES]
    if jobs or not LIB.exists() or any(Path(o).stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [cc, "-shared", *ARCH, "-o", str(LIB), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
