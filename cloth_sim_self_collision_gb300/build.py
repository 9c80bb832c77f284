"""In-tree build of the CUDA library cloth_sim_self_collision_gb300/lib/libclothgpu.so.

Every translation unit is compiled in parallel for sm_103a only.  Device code
is built with -fmad=false and host code with -ffp-contract=off, so that FP64
results round like the reference's IEEE double code (no fused multiply-add).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libclothgpu.so")
DROPIN_LIB = os.path.join(LIB_DIR, "libclothgpu_dropin.so")
DROPIN_SRC = os.path.join(PKG, "dropin", "clothgpu_dropin.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-pthread"]
SOURCES = ["topology.cpp", "prof.cu", "k_assemble.cu", "k_solve.cu", "k_mixed.cu", "k_collide.cu", "api.cu",
           "k_noalloc.cu", "serve.cu", "frame_graph.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str, extra: list) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cpp"):
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "clothgpu.h"),
                                                                 os.path.abspath(__file__), DROPIN_SRC]
    if not os.path.exists(DROPIN_LIB):
        return True
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list | None = None) -> str:
    """Compiles (if stale) and links the library; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra = list(extra or [])
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the C++ drop-in with the reference's signatures, over the C ABI
    cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-shared", "-o", DROPIN_LIB + ".tmp", DROPIN_SRC,
                                                        "-L" + LIB_DIR, "-lclothgpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the drop-in failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(DROPIN_LIB + ".tmp", DROPIN_LIB)
    if verbose:
        print("built", LIB, "and", DROPIN_LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, extra=[a for a in sys.argv[1:] if a != "--force"])
