"""In-tree build of the native library libfednl_gpu.so for sm_103a (GB300).

    python -m ufednl_gb300.build

One nvcc invocation (the CUDA round engine and the host-side local driver), one -gencode; the
output goes to ufednl_gb300/_build/.  Host code is compiled with -ffp-contract=off: gcc contracts
a*b+c into one FMA by default on aarch64 but not on x86-64, and the host parts (the LIBSVM number
parser, the driver's norms) must round the same on both.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
BUILD_DIR = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libfednl_gpu.so")
SOURCES = [os.path.join(PKG, "csrc", "fednl_gpu.cu"), os.path.join(PKG, "csrc", "fednl_mixed.cu"),
           os.path.join(PKG, "csrc", "fednl_local.cpp"), os.path.join(PKG, "csrc", "fednl_serve.cpp")]
DEPS = SOURCES + [os.path.join(PKG, "csrc", f) for f in os.listdir(os.path.join(PKG, "csrc"))] + \
    [os.path.join(REPO, "include", "fednl_gpu.h")]

NVCC_FLAGS = ["-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
              "-Xcompiler", "-fPIC", "-shared", "-Xcompiler", "-fvisibility=default",
              "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfednl_gpu.so")


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in DEPS if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *NVCC_FLAGS, "-I", os.path.join(REPO, "include"), "-o", tmp, *SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
