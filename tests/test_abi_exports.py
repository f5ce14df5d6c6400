"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/snch_gb300.h declares. Only argument checks that fail before any CUDA
call run here (no GPU in this suite)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from snch_lbvh_gb300 import _ffi, build


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    L = _ffi.lib()
    assert L.snch_version().decode().startswith("snch_gb300")


def test_every_declared_symbol_is_exported():
    names = _ffi.exported_names()
    core = {"snch_scene_create", "snch_compute_silhouettes", "snch_build_bvh", "snch_get_bvh_view",
            "snch_query_nearest", "snch_query_silhouette", "snch_query_ray", "snch_sample_in_sphere",
            "snch_sample_on_object", "snch_scene_destroy", "snch_last_error"}
    assert core <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT (snch_\w+)", out.stdout))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = _ffi.lib()
    for n in names:
        assert getattr(L, n) is not None


def test_library_is_built_for_sm_103a():
    out = subprocess.run(["cuobjdump", "--list-elf", build.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_argument_errors_before_any_cuda_call():
    L = _ffi.lib()
    h = C.c_void_p()
    v = np.zeros((3, 3), np.float32)
    t = np.array([[0, 1, 2]], np.int32)
    vp = v.ctypes.data_as(C.c_void_p)
    tp = t.ctypes.data_as(C.c_void_p)
    assert L.snch_scene_create(vp, 3, tp, 1, None) == 1
    assert "out_scene" in L.snch_last_error().decode()
    assert L.snch_scene_create(vp, -1, tp, 1, C.byref(h)) == 1
    assert L.snch_scene_create(None, 3, tp, 1, C.byref(h)) == 1
    bad = np.array([[0, 1, 3]], np.int32)
    assert L.snch_scene_create(vp, 3, bad.ctypes.data_as(C.c_void_p), 1, C.byref(h)) == 1
    assert "out of range" in L.snch_last_error().decode()
    assert L.snch_scene_create(vp, 3, tp, 1 << 30, C.byref(h)) == 6
    assert L.snch_build_bvh(None, None) == 1
    assert L.snch_query_nearest(None, None, 0, None, None, None) == 1
    assert L.snch_sort_scratch_bytes(0, 30) == 0
    assert L.snch_sort_scratch_bytes(1000, 30) > 0
    assert L.snch_sort_pairs(None, None, None, None, -1, 30, None, None, None) == 1
    assert L.snch_sort_pairs(None, None, None, None, 10, 33, None, None, None) == 1


def test_snch_error_carries_the_message():
    with pytest.raises(_ffi.SnchError, match="scene is NULL"):
        _ffi.check(_ffi.lib().snch_build_bvh(None, None))


def test_python_constants_match_the_header():
    """Every SNCH_OPT_* and SNCH_DEVICE_* value the header defines has the same
    value under the Python package's name for it (OPT_* in snch_lbvh_gb300,
    DEVICE_* in its _ffi module)."""
    import snch_lbvh_gb300 as snch
    text = open(os.path.join(build.INCLUDE, "snch_gb300.h")).read()
    opts = dict(re.findall(r"#define SNCH_(OPT_\w+) (\d+)\b", text))
    devs = dict(re.findall(r"#define SNCH_(DEVICE_\w+) (\d+)u\b", text))
    assert len(opts) >= 20 and len(devs) >= 6
    for name, value in opts.items():
        assert getattr(snch, name) == int(value), name
    for name, value in devs.items():
        assert getattr(_ffi, name) == int(value), name
