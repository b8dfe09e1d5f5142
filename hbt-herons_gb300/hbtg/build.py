"""In-tree build of libhbtg.so (CUDA, sm_103a only) with nvcc."""
from __future__ import annotations

import os
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "build")
LIB = os.path.join(BUILD, "libhbtg.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared"]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False):
    """Compiles csrc/*.cu into build/libhbtg.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = sources() + [os.path.join(REPO, "include", "hbt_unbind_gpu.h")]
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = NVCC if os.path.exists(NVCC) else "nvcc"
    units = [os.path.join(CSRC, f) for f in ("unbind.cu", "noalloc.cu", "probe.cu", "mlp.cu")]
    cmd = [nvcc, *ARCH, *FLAGS, "-I", os.path.join(REPO, "include"), *units, "-o", LIB + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(LIB + ".tmp", LIB)
    return LIB
