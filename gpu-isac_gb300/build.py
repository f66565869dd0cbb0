"""Build recipe of libgpu_aln_pack.so (sm_103a, in-tree).

    python gpu-isac_gb300/build.py [--force] [--verbose] [--checked]

Compiles every translation unit under csrc/ with nvcc in parallel and links
gpu-isac_gb300/lib/libgpu_aln_pack.so, plus gpu_aln_pack.so (the file name the
reference's callers load).  No CMake, no torch extension machinery.
--checked builds the bounds-checked variant (-DGPUISAC_CHECKED: guarded
global accesses skip and record an out-of-range index) into
gpu-isac_gb300/lib/checked/libgpu_aln_pack.so; load it by pointing
GPUISAC_LIBRARY at it.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libgpu_aln_pack.so")
DROPIN = os.path.join(HERE, "lib", "gpu_aln_pack.so")
CHECKED_OBJ = os.path.join(HERE, "lib", "checked", "obj")
CHECKED_LIB = os.path.join(HERE, "lib", "checked", "libgpu_aln_pack.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "gpu_aln_pack.h")]


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib) or (lib == LIB and not os.path.exists(DROPIN)):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None, checked: bool = False) -> str:
    lib, obj_dir = (CHECKED_LIB, CHECKED_OBJ) if checked else (LIB, OBJ)
    if not force and up_to_date(lib):
        return lib
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + (["-DGPUISAC_CHECKED"] if checked else []) + \
        (extra or [])

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if not checked:
        shutil.copyfile(LIB, DROPIN + ".tmp")
        os.replace(DROPIN + ".tmp", DROPIN)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--checked", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, checked=a.checked))
