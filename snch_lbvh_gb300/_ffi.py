"""ctypes binding of libsnch_gb300.so (declarations of include/snch_gb300.h).

Loading fails loudly when the library is missing: there is no CPU or
PyTorch fallback behind this package.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

P, I64, I, U32P = C.c_void_p, C.c_int64, C.c_int, C.c_void_p

SNCH_OK = 0
STATUS_NAMES = {0: "SNCH_OK", 1: "SNCH_ERR_INVALID_ARGUMENT", 2: "SNCH_ERR_CUDA", 3: "SNCH_ERR_NOT_BUILT",
                4: "SNCH_ERR_OUT_OF_MEMORY", 5: "SNCH_ERR_DEVICE_STATUS", 6: "SNCH_ERR_TOO_LARGE"}
DEVICE_STACK_OVERFLOW, DEVICE_LOOKBACK_TIMEOUT, DEVICE_HASH_FULL = 1, 2, 4
DEVICE_TREE_DEPTH, DEVICE_COPY_TIMEOUT, DEVICE_WORK_TIMEOUT = 16, 32, 64


class SnchError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class BvhView(C.Structure):
    """snch_bvh_view: byte-compatible with the reference's bvh_device view (bvh.cuh:36-72)."""
    _fields_ = [("num_nodes", C.c_uint32), ("num_objects", C.c_uint32), ("nodes", P), ("aabbs", P),
                ("cones", P), ("objects", P)]


class TraversalView(C.Structure):
    """snch_traversal_view: the tree in this library's 64-byte record layout, read by
    the header-only device functions of include/snch_device.cuh."""
    _fields_ = [("num_triangles", C.c_uint32), ("reserved", C.c_uint32), ("root_box", P), ("inner", P),
                ("inner_cones", P), ("leaves", P), ("edges", P), ("vertices", P), ("triangles", P), ("status", P)]


# name -> (restype, argtypes), parsed from the public header so the binding
# cannot drift from it
def _header_signatures():
    text = open(os.path.join(_build.INCLUDE, "snch_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    sigs = {}
    for m in re.finditer(r"\b(int|size_t|uint64_t|int64_t|const char \*)\s*(snch_\w+)\s*\(([^)]*)\)\s*;", text):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        sigs[name] = (ret, [a.strip() for a in args.split(",") if a.strip() and a.strip() != "void"])
    return sigs


def _ctype(arg: str):
    a = arg.replace("const ", "").strip()
    if "*" in a:
        return P
    t = a.split()[0]
    return {"int64_t": I64, "int": I, "int32_t": C.c_int32, "size_t": C.c_size_t, "snch_scene_t": P, "snch_stream_t": P,
            "uint32_t": C.c_uint32, "uint64_t": C.c_uint64, "float": C.c_float, "snch_mlp_t": P,
            "snch_graph_t": P, "snch_scene2_t": P}[t]


_lib = None


def exported_names() -> list[str]:
    return sorted(_header_signatures())


def lib():
    """Load libsnch_gb300.so, compiling it first if it is missing or stale."""
    global _lib
    if _lib is None:
        path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libsnch_gb300.so missing at {path}")
        L = C.CDLL(path)
        for name, (ret, args) in _header_signatures().items():
            f = getattr(L, name)  # AttributeError = header declares a symbol the library lacks
            f.restype = {"int": I, "size_t": C.c_size_t, "uint64_t": C.c_uint64, "int64_t": I64,
                         "const char *": C.c_char_p}[ret]
            f.argtypes = [_ctype(a) for a in args]
        _lib = L
    return _lib


def check(rc: int):
    if rc != SNCH_OK:
        raise SnchError(rc, lib().snch_last_error().decode())
