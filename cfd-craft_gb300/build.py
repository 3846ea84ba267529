"""Compiles the engine library libcfdgpu.so in-tree for sm_103a (no CMake).

Run as a script or call build(). Output: cfd-craft_gb300/_build/libcfdgpu.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcfdgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false / -ffp-contract=off: the plain form rounds every product and sum on
# its own, like the reference (Rust does not contract a*b+c into an FMA).
UNITS = [
    ("engine.cu", ["-fmad=false"]),
    ("mixed.cu", []),  # FP32 inner solve: contraction allowed; its FP64 parts use explicit _rn intrinsics
    ("setup.cpp", []),
]


def _nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return path


def _sources():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "cfdgpu.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in _sources())
        if os.path.getmtime(LIB) >= newest:
            return LIB
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", SRC]

    def compile_unit(unit):
        name, flags = unit
        obj = os.path.join(OUT, name + ".o")
        cmd = [nvcc, "-c", os.path.join(SRC, name), "-o", obj] + common + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {name} failed:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp, "-cudart", "static"] + ARCH + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libcfdgpu.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
