"""Build libcmgb300.so (the CUDA kernels and the C ABI) in-tree for sm_103a with nvcc.

    python -m cardiomechanics_gb300.build

Translation units compile in parallel; the library lands in cardiomechanics_gb300/_lib/.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libcmgb300.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math"]
SOURCES = ["cm_kernels.cu", "cm_staged.cu", "cm_multi.cu", "cm_capi.cpp", "cm_params.cpp", "cm_diag.cu", "cm_mlp.cu", "cm_surrogate.cu", "cm_sur_api.cpp", "cm_noalloc.cu", "cm_diffusion.cpp", "cm_backup.cpp", "cm_theta.cu", "cm_theta_api.cpp", "cm_print.cpp"]


def _compile(src: str, extra: list[str]) -> Path:
    obj = OUT / (Path(src).stem + ".o")
    cmd = [NVCC, *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    if src.endswith(".cpp"):
        cmd = [NVCC, *COMMON, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUT.mkdir(exist_ok=True)
    extra = list(extra or [])
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
