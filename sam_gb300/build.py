"""Build the in-tree CUDA library libsam_gpu.so for sm_103a with nvcc.

Each translation unit compiles in parallel; the objects are linked into
sam_gb300/_lib/libsam_gpu.so.  Nothing is installed outside the tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libsam_gpu.so")
SOURCES = ["passes.cu", "passes_f32.cu", "passes_dd_zinv.cu", "passes_dd_yinv.cu", "passes_dd_x.cu", "passes_dd_yfwd.cu",
           "passes_dd_zfwd.cu", "passes_ens.cu", "fields.cu", "diag.cu", "les.cu", "noalloc.cu", "planes.cu", "closure.cu", "sam_gpu.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsam_gpu.so")


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(HERE, "..", "include", "sam_gpu.h"))
    return out


def _compile(src: str) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    newest = max(os.path.getmtime(p) for p in [path, *_deps()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    tmp = obj + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", path, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, obj)
    return obj


def build(force: bool = False) -> str:
    """Compile every CUDA source (in parallel) and link libsam_gpu.so."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJ_DIR):
            os.remove(os.path.join(OBJ_DIR, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(o) for o in objs):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build())
