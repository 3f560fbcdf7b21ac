"""Builds libcthermal.so (the CUDA solver library and its C ABI) in-tree.

Host C++ with g++, CUDA with nvcc for sm_103a only, translation units in
parallel, then one shared library linked against the static CUDA runtime, so
the library loads (and lists its symbols) on machines without a GPU.

    python cuda-thermal_gb300/build.py [--force] [--debug]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libcthermal.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the model builder and the host-side arithmetic must round
# exactly as the reference does on every host architecture.
HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-Wall"]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off"]

CPP_SOURCES = ["status.cpp", "model.cpp", "case.cpp"]
CU_SOURCES = ["k_outer.cu", "k_fp64.cu", "k_batch64.cu", "k_mg.cu", "k_dw.cu", "k_batch.cu", "k_sweep_tma.cu", "k_fields.cu", "k_build.cu", "solver.cu", "batch.cu", "noalloc.cu", "k_probe.cu"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith((".h", ".hpp"))]
    return hs


def _compile(src: str, debug: bool) -> str:
    path = os.path.join(SRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    if _newer(obj, [path] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, *CU_FLAGS, "-I", INC, "-I", SRC, "-c", path, "-o", obj]
        if debug:
            cmd += ["-DCT_DEBUG"]
    else:
        cmd = ["g++", *HOST_FLAGS, "-I", INC, "-I", SRC, "-I", "/usr/local/cuda/include",
               "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, debug: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJ_DIR):
            os.remove(os.path.join(OBJ_DIR, f))
    sources = CPP_SOURCES + CU_SOURCES
    with cf.ThreadPoolExecutor(max_workers=len(sources)) as ex:
        objs = list(ex.map(lambda s: _compile(s, debug), sources))
    if not _newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "--cudart", "static", "-o", LIB, *objs,
               "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, debug="--debug" in sys.argv))
