"""Builds libsph_gb300.so for sm_103a, in-tree under _build/.

nvcc compiles each translation unit of csrc/ in parallel with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then links a shared
library against the CUDA runtime. No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libsph_gb300.so"
SOURCES = ["sph_kernels.cu", "sph_engine.cu", "sph_capi.cu", "sph_static.cu",
           "sph_render.cu", "sph_snapshot.cu", "sph_server.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str, extra) -> pathlib.Path:
    obj = OUT / (pathlib.Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
           "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
           "-I", str(PKG.parent / "include"), *extra, "-c", str(CSRC / src),
           "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    return obj


def build(extra=(), force: bool = False) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    hdrs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list((PKG.parent / "include").glob("*.h"))
    if LIB.exists() and not force:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime < t for p in srcs + hdrs):
            return LIB
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs),
           "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
