"""Builds libcbq.so in-tree: CUDA sources for sm_103a with nvcc, host C++ with g++.

Floating-point flags are part of the contract: the traversal must not contract
a*b+c into FMA (-fmad=false for nvcc, -ffp-contract=off for g++) and must use
IEEE division, or hits stop matching the reference bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "libcbq.so"

CUDA_SOURCES = ["cbq_api.cu", "cbq_flat.cu", "cbq_batch.cu", "cbq_server.cu", "cbq_pathtrace.cu", "cbq_probe.cu",
                "cbq_noalloc.cu"]
CXX_SOURCES = ["cbq_host.cpp", "cbq_builder.cpp"]

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    GENCODE, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
    "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-Wall",
             "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcbq")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    """Compiles every translation unit (in parallel) and links libcbq.so."""
    BUILD_DIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + [PKG_DIR.parent / "include" / "cubiquity_gb300.h"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([nvcc, *NVCC_FLAGS, *(extra_nvcc or []), "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd))
            fut.result()
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        _run([nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
