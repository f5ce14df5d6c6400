"""Wavefront walk-on-stars driver (snch_wost_trace in the C ABI).

Splits a mesh into a Dirichlet and a Neumann scene by per-face flags and runs
walk-on-stars walkers (Sawhney et al. 2023) for the test problem u(x) = x_0:
every step issues, for every live walker, one nearest-primitive query on the
Dirichlet scene, one nearest-silhouette query, one ray and one
SampleTriangleInSphere draw on the Neumann scene, as batched library calls;
finished walkers are compacted away between steps. With a trained
``LearnedRadius`` (output 0: Dirichlet distance, output 1: Neumann silhouette
distance) the two distance queries are seeded; the walks are identical.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import Scene, _ptr, _stream, _torch
from ._ffi import check, lib

MAX_STEPS = 128


class WostParams(C.Structure):
    _fields_ = [("walkers", C.c_int64), ("max_steps", C.c_int32), ("epsilon", C.c_float),
                ("center", C.c_float * 3), ("radius", C.c_float), ("seed", C.c_uint64),
                ("margin", C.c_float), ("floor_", C.c_float)]


class WostStats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("terminated", C.c_int64), ("live", C.c_int64 * MAX_STEPS),
                ("queries", C.c_int64 * MAX_STEPS), ("step_ms", C.c_float * MAX_STEPS),
                ("query_ms", C.c_float * MAX_STEPS), ("fallback", C.c_uint32 * MAX_STEPS)]


def split_boundary(verts, faces, neumann_flags):
    """(Dirichlet scene, Neumann scene), both built: faces with flag 0 / 1."""
    faces = np.asarray(faces)
    fl = np.asarray(neumann_flags).astype(bool)
    out = []
    for sel in (~fl, fl):
        s = Scene(verts, faces[sel].reshape(-1, 3))
        s.compute_silhouettes()
        s.build_bvh()
        out.append(s)
    return tuple(out)


def trace(dirichlet: Scene, neumann: Scene, walkers: int, max_steps: int = MAX_STEPS, epsilon: float = 1e-3,
          center=(0.0, 0.0, 0.0), radius: float = 0.95, seed: int = 0, model=None, margin: float = 1.5,
          floor: float = 1e-4, stream=None):
    """Runs the walks; returns (estimates [walkers], start points [walkers, 3], stats dict)."""
    torch = _torch()
    est = torch.empty(walkers, device="cuda", dtype=torch.float32)
    start = torch.empty((walkers, 3), device="cuda", dtype=torch.float32)
    p = WostParams(walkers, max_steps, epsilon, (C.c_float * 3)(*center), radius, seed, margin, floor)
    st = WostStats()
    check(lib().snch_wost_trace(dirichlet._h, neumann._h, model._h if model is not None else None, C.byref(p),
                                _ptr(est), _ptr(start), C.byref(st), _stream(stream)))
    k = st.steps
    stats = {"steps": k, "terminated": int(st.terminated), "live": list(st.live[:k]),
             "queries": list(st.queries[:k]), "step_ms": list(st.step_ms[:k]), "query_ms": list(st.query_ms[:k]),
             "fallback": list(st.fallback[:k])}
    return est, start, stats
