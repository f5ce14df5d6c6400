"""The C++ host API (include/snch_gb300.hpp) compiles and links against
libsnch_gb300.so; on a GPU it runs a build + nearest query end to end."""
import os
import subprocess

import pytest

from snch_lbvh_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "scene3_example.cpp")
OUT = os.path.join(ROOT, "tests", "cxx", "_build", "scene3_example")


def compile_example():
    build.build()
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    lib_dir = os.path.dirname(build.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", SRC, "-o", OUT, "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", "-L", lib_dir, "-lsnch_gb300", f"-Wl,-rpath,{lib_dir}",
           "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return OUT


def test_cxx_api_compiles_and_links():
    exe = compile_example()
    r = subprocess.run([exe, "--version"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("snch_gb300"), r.stdout + r.stderr


@pytest.mark.gpu
def test_cxx_api_runs_on_gpu():
    exe = compile_example()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_device_header_compiles_with_default_nvcc_flags(tmp_path):
    """include/snch_device.cuh in a caller's kernels (tests/cxx/device_shim_kernels.cu),
    compiled for sm_103a with nvcc's defaults; the GPU comparison is
    tests/test_gpu_device_shim.py."""
    cmd = [build.nvcc(), "-c", *build.ARCH, "-O3", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cxx", "device_shim_kernels.cu"), "-o", str(tmp_path / "shim.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
