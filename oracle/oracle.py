"""ctypes front-end of the CPU oracle (oracle/snch_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU
baseline / reference arm, always as the checker or the timed CPU restatement,
never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

_lib = None


# where the reference checkout lies in the container that generates the golden
# vectors (the GPU machines have none); SNCH_REFERENCE overrides it
REFERENCE_CHECKOUT = "/root/reference"


def build(verbose: bool = False) -> None:
    """Compile the oracle (and, where the reference checkout exists, the reference harness)."""
    env = dict(os.environ)
    if not env.get("SNCH_REFERENCE") and os.path.isdir(REFERENCE_CHECKOUT):
        env["SNCH_REFERENCE"] = REFERENCE_CHECKOUT
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True, env=env)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if verbose:
        print(out.stdout, out.stderr)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


class OrcScene(C.Structure):
    _fields_ = [("num_tris", C.c_int64), ("num_verts", C.c_int64), ("num_edges", C.c_int64),
                ("verts", C.c_void_p), ("tris", C.c_void_p), ("tri_owned", C.c_void_p),
                ("edge_verts", C.c_void_p), ("nodes", C.c_void_p), ("aabbs", C.c_void_p),
                ("cones", C.c_void_p)]


def _declare(L):
    P, I64, I = C.c_void_p, C.c_int64, C.c_int
    L.orc_topology.argtypes = [P, I64, P, P, P]
    L.orc_topology.restype = I64
    L.orc_leaf_aabbs.argtypes = [P, P, I64, P]
    L.orc_leaf_cones.argtypes = [P, P, I64, P, P, P]
    L.orc_build.argtypes = [P, P, I64, P, P, P, P, P, P, P, P]
    L.orc_build.restype = I
    L.orc_query_nearest.argtypes = [P, P, I64, P, P, P, I]
    L.orc_query_silhouette.argtypes = [P, P, P, I64, P, P, P, I]
    L.orc_query_ray.argtypes = [P, P, P, P, I64, P, P, P, P, P, I]
    L.orc_sample_in_sphere.argtypes = [P, P, P, P, I64, P, P, P, I]
    L.orc_sample_on_object.argtypes = [P, P, P, P, I64, P]
    L.orc_brute_nearest_f64.argtypes = [P, P, I64, P, I64, P, P, I]
    L.orc_brute_silhouette_f64.argtypes = [P, P, I64, P, P, I64, P, I]
    L.orc_brute_ray_f64.argtypes = [P, P, I64, P, P, P, I64, P, P, P, I]
    L.orc_max_depth.argtypes = [P, I64]
    L.orc_max_depth.restype = I
    L.orc_leaf_ranks.argtypes = [P, I64, P]
    L.orc_query_overlap.argtypes = [P, P, I64, I64, P, P, I]
    L.orc2_topology.argtypes = [P, I64, I64, P, P]
    L.orc2_build.argtypes = [P, P, I64, P, P, P, P, P, P, P, P]
    L.orc2_build.restype = I
    L.orc2_query_nearest.argtypes = [P, P, I64, P, P]
    L.orc2_query_silhouette.argtypes = [P, P, P, I64, P, P]
    L.orc2_query_ray.argtypes = [P, P, P, P, I64, P, P, P, P]
    L.orc2_sample_in_circle.argtypes = [P, P, P, P, I64, P, P]
    L.orc_query_line.argtypes = [P, P, P, I64, I64, P, P, P, I]


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


class Tree:
    """A scene and its LBVH in the reference's flat layout (bvh.cuh:27-33)."""

    def __init__(self, verts, tris):
        L = lib()
        self.verts = _c(verts, np.float32).reshape(-1, 3)
        self.tris = _c(tris, np.int32).reshape(-1, 3)
        nt = len(self.tris)
        self.tri_edges = np.empty((nt, 3), np.int32)
        self.tri_owned = np.empty((nt, 3), np.int32)
        ev = np.empty((max(3 * nt, 1), 4), np.int32)
        ne = L.orc_topology(_p(self.tris), nt, _p(self.tri_edges), _p(self.tri_owned), _p(ev))
        self.edge_verts = np.ascontiguousarray(ev[:ne])
        nn = max(2 * nt - 1, 0)
        self.morton = np.empty(nt, np.uint32)
        self.sorted_idx = np.empty(nt, np.uint32)
        self.nodes = np.empty((nn, 4), np.uint32)
        self.aabbs = np.empty((nn, 6), np.float32)
        self.cones = np.empty((nn, 5), np.float32)
        self.d1 = np.zeros(nn, np.uint8)
        self.unique = bool(L.orc_build(_p(self.verts), _p(self.tris), nt, _p(self.tri_owned), _p(self.edge_verts),
                                       _p(self.morton), _p(self.sorted_idx), _p(self.nodes), _p(self.aabbs),
                                       _p(self.cones), _p(self.d1)))
        self._s = OrcScene(nt, len(self.verts), ne, _p(self.verts).value, _p(self.tris).value,
                           _p(self.tri_owned).value, _p(self.edge_verts).value, _p(self.nodes).value,
                           _p(self.aabbs).value, _p(self.cones).value)

    @property
    def num_tris(self):
        return len(self.tris)

    def leaf_ranks(self):
        r = np.empty(self.num_tris, np.uint32)
        lib().orc_leaf_ranks(_p(self.nodes), self.num_tris, _p(r))
        return r

    def max_depth(self) -> int:
        return lib().orc_max_depth(_p(self.nodes), self.num_tris)

    def nearest(self, pts, stats=False, nthreads=None):
        pts = _c(pts, np.float32).reshape(-1, 3)
        n = len(pts)
        idx, dist = np.empty(n, np.uint32), np.empty(n, np.float32)
        st = np.empty((n, 3), np.uint32) if stats else None
        lib().orc_query_nearest(C.byref(self._s), _p(pts), n, _p(idx), _p(dist), _p(st),
                                nthreads or nthreads_default())
        return (idx, dist, st) if stats else (idx, dist)

    def silhouette(self, pts, flip=None, stats=False, nthreads=None):
        pts = _c(pts, np.float32).reshape(-1, 3)
        n = len(pts)
        fl = None if flip is None else _c(flip, np.uint8)
        dist, edge = np.empty(n, np.float32), np.empty(n, np.int32)
        st = np.empty((n, 3), np.uint32) if stats else None
        lib().orc_query_silhouette(C.byref(self._s), _p(pts), _p(fl), n, _p(dist), _p(edge), _p(st),
                                   nthreads or nthreads_default())
        return (dist, edge, st) if stats else (dist, edge)

    def ray(self, origins, dirs, tmax, stats=False, nthreads=None):
        o = _c(origins, np.float32).reshape(-1, 3)
        d = _c(dirs, np.float32).reshape(-1, 3)
        tm = _c(tmax, np.float32)
        n = len(o)
        hit, t, uv, idx = np.empty(n, np.uint8), np.empty(n, np.float32), np.empty((n, 2), np.float32), np.empty(n, np.uint32)
        st = np.empty((n, 3), np.uint32) if stats else None
        lib().orc_query_ray(C.byref(self._s), _p(o), _p(d), _p(tm), n, _p(hit), _p(t), _p(uv), _p(idx), _p(st),
                            nthreads or nthreads_default())
        return (hit, t, uv, idx, st) if stats else (hit, t, uv, idx)

    def sample(self, centers, radii, u, stats=False, nthreads=None):
        c = _c(centers, np.float32).reshape(-1, 3)
        r, uu = _c(radii, np.float32), _c(u, np.float32)
        n = len(c)
        idx, pdf = np.empty(n, np.int32), np.empty(n, np.float32)
        st = np.empty((n, 3), np.uint32) if stats else None
        lib().orc_sample_in_sphere(C.byref(self._s), _p(c), _p(r), _p(uu), n, _p(idx), _p(pdf), _p(st),
                                   nthreads or nthreads_default())
        return (idx, pdf, st) if stats else (idx, pdf)

    def overlap(self, boxes, max_out, nthreads=None):
        b = _c(boxes, np.float32).reshape(-1, 6)
        n = len(b)
        idx = np.full((n, max_out), 0xFFFFFFFF, np.uint32)
        cnt = np.empty(n, np.uint32)
        lib().orc_query_overlap(C.byref(self._s), _p(b), n, max_out, _p(idx), _p(cnt), nthreads or nthreads_default())
        return idx, cnt

    def line(self, origins, dirs, max_out, nthreads=None):
        o = _c(origins, np.float32).reshape(-1, 3)
        d = _c(dirs, np.float32).reshape(-1, 3)
        n = len(o)
        idx = np.full((n, max_out), 0xFFFFFFFF, np.uint32)
        t = np.full((n, max_out), np.nan, np.float32)
        cnt = np.empty(n, np.uint32)
        lib().orc_query_line(C.byref(self._s), _p(o), _p(d), n, max_out, _p(idx), _p(t), _p(cnt),
                             nthreads or nthreads_default())
        return idx, t, cnt

    def sample_on_object(self, idx, u, v):
        i, uu, vv = _c(idx, np.int32), _c(u, np.float32), _c(v, np.float32)
        out = np.empty((len(i), 3), np.float32)
        lib().orc_sample_on_object(C.byref(self._s), _p(i), _p(uu), _p(vv), len(i), _p(out))
        return out


def brute_nearest_f64(verts, tris, pts, nthreads=None):
    v, t, p = _c(verts, np.float32), _c(tris, np.int32), _c(pts, np.float32).reshape(-1, 3)
    n = len(p)
    idx, dist = np.empty(n, np.uint32), np.empty(n, np.float64)
    lib().orc_brute_nearest_f64(_p(v), _p(t), len(t.reshape(-1, 3)), _p(p), n, _p(idx), _p(dist),
                                nthreads or nthreads_default())
    return idx, dist


def brute_silhouette_f64(verts, edge_verts, pts, flip=None, nthreads=None):
    v, e, p = _c(verts, np.float32), _c(edge_verts, np.int32), _c(pts, np.float32).reshape(-1, 3)
    n = len(p)
    fl = None if flip is None else _c(flip, np.uint8)
    dist = np.empty(n, np.float64)
    lib().orc_brute_silhouette_f64(_p(v), _p(e), len(e.reshape(-1, 4)), _p(p), _p(fl), n, _p(dist),
                                   nthreads or nthreads_default())
    return dist


def brute_ray_f64(verts, tris, origins, dirs, tmax, nthreads=None):
    v, t = _c(verts, np.float32), _c(tris, np.int32)
    o, d, tm = _c(origins, np.float32).reshape(-1, 3), _c(dirs, np.float32).reshape(-1, 3), _c(tmax, np.float32)
    n = len(o)
    hit, tt, idx = np.empty(n, np.uint8), np.empty(n, np.float64), np.empty(n, np.uint32)
    lib().orc_brute_ray_f64(_p(v), _p(t), len(t.reshape(-1, 3)), _p(o), _p(d), _p(tm), n, _p(hit), _p(tt), _p(idx),
                            nthreads or nthreads_default())
    return hit, tt, idx


class Orc2Scene(C.Structure):
    _fields_ = [("num_segs", C.c_int64), ("num_verts", C.c_int64), ("verts", C.c_void_p), ("segs", C.c_void_p),
                ("seg_owned", C.c_void_p), ("sv", C.c_void_p), ("nodes", C.c_void_p), ("aabbs", C.c_void_p),
                ("cones", C.c_void_p)]


class Tree2:
    """The reference's scene<2> (scene.cuh:287-703): line segments, silhouette
    vertices, the 2D LBVH and the four queries, restated in C (FP32)."""

    def __init__(self, verts, segs):
        L = lib()
        self.verts = _c(verts, np.float32).reshape(-1, 2)
        self.segs = _c(segs, np.int32).reshape(-1, 2)
        n, nv = len(self.segs), len(self.verts)
        self.sv = np.empty((max(nv, 1), 4), np.int32)[:nv]
        self.seg_owned = np.empty((n, 2), np.int32)
        L.orc2_topology(_p(self.segs), n, nv, _p(self.sv), _p(self.seg_owned))
        nn = max(2 * n - 1, 0)
        self.morton = np.empty(n, np.uint32)
        self.sorted_idx = np.empty(n, np.uint32)
        self.nodes = np.empty((nn, 4), np.uint32)
        self.aabbs = np.empty((nn, 4), np.float32)
        self.cones = np.empty((nn, 4), np.float32)
        self.d1 = np.zeros(nn, np.uint8)
        self.unique = bool(L.orc2_build(_p(self.verts), _p(self.segs), n, _p(self.seg_owned), _p(self.sv),
                                        _p(self.morton), _p(self.sorted_idx), _p(self.nodes), _p(self.aabbs),
                                        _p(self.cones), _p(self.d1)))
        self._s = Orc2Scene(n, nv, _p(self.verts).value, _p(self.segs).value, _p(self.seg_owned).value,
                            _p(self.sv).value, _p(self.nodes).value, _p(self.aabbs).value, _p(self.cones).value)

    def nearest(self, pts):
        p = _c(pts, np.float32).reshape(-1, 2)
        idx, dist = np.empty(len(p), np.uint32), np.empty(len(p), np.float32)
        lib().orc2_query_nearest(C.byref(self._s), _p(p), len(p), _p(idx), _p(dist))
        return idx, dist

    def silhouette(self, pts, flip=None):
        p = _c(pts, np.float32).reshape(-1, 2)
        fl = None if flip is None else _c(flip, np.uint8)
        dist, vid = np.empty(len(p), np.float32), np.empty(len(p), np.int32)
        lib().orc2_query_silhouette(C.byref(self._s), _p(p), _p(fl), len(p), _p(dist), _p(vid))
        return dist, vid

    def ray(self, origins, dirs, tmax):
        o, d = _c(origins, np.float32).reshape(-1, 2), _c(dirs, np.float32).reshape(-1, 2)
        tm = _c(tmax, np.float32)
        n = len(o)
        hit, t, sp, idx = np.empty(n, np.uint8), np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n, np.uint32)
        lib().orc2_query_ray(C.byref(self._s), _p(o), _p(d), _p(tm), n, _p(hit), _p(t), _p(sp), _p(idx))
        return hit, t, sp, idx

    def sample(self, centers, radii, u):
        c = _c(centers, np.float32).reshape(-1, 2)
        r, uu = _c(radii, np.float32), _c(u, np.float32)
        idx, pdf = np.empty(len(c), np.int32), np.empty(len(c), np.float32)
        lib().orc2_sample_in_circle(C.byref(self._s), _p(c), _p(r), _p(uu), len(c), _p(idx), _p(pdf))
        return idx, pdf
