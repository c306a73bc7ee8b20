"""Builds the in-tree shared library libevrsg4.so (CUDA kernels + C ABI).

nvcc compiles every translation unit for sm_103a only, in parallel, into
elvibrot_gb300/libevrsg4.so.  The library is rebuilt when a source is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libevrsg4.so")

SOURCES = ["sg4_device.cu", "sg4_solvers.cu", "sg4_setup.cpp", "sg4_items.cu"]
# translation units: (source, object, extra flags); each item kernel is its
# own unit, per launch geometry (wide, narrow, mid) and kind (small parameter
# block: one context or a field-driven pair; large: multi-context plans;
# small, compiled for type-10 operators only; small, with type-1
# coefficient grids)
UNITS = [("sg4_items.cu", f"sg4_items_g{g}_k{k}.o", [f"-DEVR_GEO={g}", f"-DEVR_KIND={k}"])
         for g in range(3) for k in range(4)] + [
    ("sg4_device.cu", "sg4_device.o", []), ("sg4_solvers.cu", "sg4_solvers.o", []),
    ("sg4_setup.cpp", "sg4_setup.o", [])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libevrsg4.so")


def _deps():
    deps = [os.path.join(CSRC, s) for s in SOURCES]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h") or f.endswith(".cuh")]
    deps.append(os.path.join(INCLUDE, "evr_sg4.h"))
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC, "-Xcompiler", "-fPIC,-O3"]

    def compile_one(unit):
        src, name, flags = unit
        obj = os.path.join(BUILD, name)
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common + flags
        if src.endswith(".cu"):
            cmd += ARCH + ["-lineinfo", "-Xptxas", "-v"] if verbose else ARCH + ["-lineinfo"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), max(4, os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
