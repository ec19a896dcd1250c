"""Builds libpencilfft_gb300.so for sm_103a with nvcc, in-tree.

The translation units are compiled in parallel to object files under
``pencilffts.jl_gb300/_build`` and linked into
``pencilffts.jl_gb300/pencilffts_gb300/_lib/libpencilfft_gb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                 # pencilffts.jl_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG_DIR, "_lib")
LIB = os.path.join(LIBDIR, "libpencilfft_gb300.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["pfgb_persist.cu", "pfgb_plan.cu", "pfgb_kernels.cu", "pfgb_noalloc.cu", "pfgb_tc.cu"] + [
    f"pfgb_fast_f32_{op}.cu" for op in ("c2c", "r2c", "c2r", "x00", "d23")] + [
    f"pfgb_fast_{t}_{op}_{iom}.cu" for t in ("dd", "fx")
    for op, ioms in (("c2c", (0, 1, 2, 3)), ("r2c", (0, 2)), ("c2r", (0, 1))) for iom in ioms] + [
    f"pfgb_fast_dd_x00c_{iom}.cu" for iom in (0, 1, 2, 3)] + ["pfgb_fast_dd_x00r_0.cu"] + [
    f"pfgb_fast_dd_d23c_{iom}.cu" for iom in (0, 1, 2, 3)] + ["pfgb_fast_dd_d23r_0.cu"] + [
    f"pfgb_fast_dd_csum_{iom}.cu" for iom in (0, 2)] + ["pfgb_fast_dd_c2ct_0.cu"] + [
    f"pfgb_mr_{t}_{op}_{r0}.cu" for t in ("f32", "dd") for op in ("c2c", "r2c", "c2r") for r0 in (3, 5)] + [
    f"pfgb_bs_{t}_{op}.cu" for t in ("f32", "dd") for op in ("c2c", "r2c", "c2r")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "pencilfft_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I", INCLUDE, "-I", CSRC]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *common, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
