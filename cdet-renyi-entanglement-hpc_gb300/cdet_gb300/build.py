"""Compiles the CUDA library libcdet_gb300.so in-tree with nvcc for sm_103a."""
from __future__ import annotations

import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libcdet_gb300.so")
INCLUDE = os.path.join(REPO_ROOT, "include")

SOURCES = ["cdet_kernels.cu", "cdet_dd.cu", "cdet_split.cu", "cdet_capi.cu", "cdet_noalloc.cu",
           "cdet_diagonal.cu", "cdet_mcmcmc.cu", "cdet_mcmcmc_host.cu"]
HEADERS = ["cdet_device.cuh", "cdet_kernels.cuh", "cdet_capi_internal.h"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    # Exact reference arithmetic: no FMA contraction on device or host.
    "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-shared",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CDet CUDA library cannot be built")
    return path


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    built = os.path.getmtime(LIB_PATH)
    inputs = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    inputs.append(os.path.join(INCLUDE, "cdet_gb300.h"))
    return any(os.path.getmtime(p) > built for p in inputs)


def build(force: bool = False, verbose: bool = False) -> str:
    """Builds the library when a source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *NVCC_FLAGS, "-I" + INCLUDE, "-o", tmp] + [os.path.join(CSRC, f) for f in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH
