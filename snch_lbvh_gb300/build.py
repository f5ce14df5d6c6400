"""Compile libsnch_gb300.so (the C ABI of include/snch_gb300.h) for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
snch_lbvh_gb300/_lib/libsnch_gb300.so (static cudart). The geometry units are
built with -fmad=false: every float expression is evaluated one IEEE operation
at a time in the reference's order, which is what makes the results equal the
reference's bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libsnch_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, extra flags)
UNITS = [
    ("scan_sort.cu", []),
    ("topology.cu", []),
    ("build.cu", ["-fmad=false"]),
    ("queries.cu", ["-fmad=false"]),
    ("abi.cu", []),
    ("noalloc_sort.cu", []),
    ("mlp.cu", []),
    ("wost.cu", []),
    ("io.cu", []),
    ("scene2d.cu", ["-fmad=false"]),
]
HEADERS = ["common.cuh", "internal.h", "tcgen05.cuh"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsnch_gb300")
    return path


def _inputs():
    files = [os.path.join(CSRC, u) for u, _ in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    files.append(os.path.join(INCLUDE, "snch_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I", INCLUDE, "-I", CSRC] + (extra_flags or [])

    def compile_unit(unit):
        src, flags = unit
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
