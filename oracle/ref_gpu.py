"""The reference's own CUDA queries on GB300 -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_ref/ref_queries_sm103a.cubin (the reference headers compiled
for sm_103a by oracle/Makefile) through oracle/_build/libref_gpu_loader.so and
runs its kernels over a tree built by this project (snch_bvh_view is
byte-compatible with the reference's bvh_device view). Used by the parity
tests and by bench.py's reference arm; unavailable where the cubin was not
built.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_queries_sm103a.cubin")
LOADER = os.path.join(HERE, "_build", "libref_gpu_loader.so")

_lib = None


def available() -> tuple[bool, str]:
    if not os.path.exists(CUBIN):
        return False, f"reference cubin missing ({CUBIN}): it is built only where the reference headers exist"
    if not os.path.exists(LOADER):
        return False, "reference cubin loader not built"
    return True, ""


def lib():
    global _lib
    if _lib is None:
        ok, why = available()
        if not ok:
            raise RuntimeError(why)
        L = C.CDLL(LOADER)
        P, I = C.c_void_p, C.c_int
        L.rg_load.argtypes = [C.c_char_p]
        L.rg_nearest.argtypes = [P, P, I, P, P, P]
        L.rg_silhouette.argtypes = [P, P, P, I, P, P]
        L.rg_silhouette_edge.argtypes = [P, P, P, I, P, P, P]
        L.rg_ray_uv.argtypes = [P, P, P, P, I, P, P, P, P, P]
        L.rg_ray.argtypes = [P, P, P, P, I, P, P, P, P]
        L.rg_sample.argtypes = [P, P, P, P, I, P, P, P]
        rc = L.rg_load(CUBIN.encode())
        if rc != 0:
            raise RuntimeError(f"loading the reference cubin failed: cudaError {rc}")
        _lib = L
    return _lib


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class RefView(C.Structure):
    """lbvh::bvh_device<float, 3, scene<3>::triangle> (bvh.cuh:36-72): counts, then
    node / aabb / cone / object device pointers (40 bytes)."""
    _fields_ = [("num_nodes", C.c_uint32), ("num_objects", C.c_uint32), ("nodes", C.c_void_p),
                ("aabbs", C.c_void_p), ("cones", C.c_void_p), ("objects", C.c_void_p)]


class RefTree:
    """A tree built by the ORACLE (the CPU restatement of the reference's build,
    bvh.cuh:380-613 with the silhouette topology of scene.cuh:1135-1229, equal bit
    for bit to the reference's own build on every golden mesh), uploaded in the
    reference's device layout -- nodes (bvh.cuh:27-33), aabbs upper-first,
    cones, scene<3>::triangle objects (scene.cuh:826-840: vertex ids, owned
    silhouette ids, vertex and edge pointers; 40 B) and silhouette_edge records
    (scene.cuh:708-722: 4 vertex ids and the vertex pointer; 32 B) -- so that the
    reference's own CUDA queries run on a tree this library never touched."""

    def __init__(self, tree):
        import numpy as np
        import torch
        n = tree.num_tris
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        self.verts = dev(tree.verts)
        self.nodes = dev(tree.nodes.view(np.int32))
        self.aabbs = dev(tree.aabbs)
        self.cones = dev(tree.cones)
        vptr = self.verts.data_ptr()
        ne = len(tree.edge_verts)
        e = np.zeros((max(ne, 1), 4), np.int64)  # 32 B per edge
        if ne:
            e[:, :2] = tree.edge_verts.astype(np.int32).view(np.int64)
            e[:, 2] = vptr
        self.edges = dev(e)
        o = np.zeros((max(n, 1), 5), np.int64)  # 40 B per triangle
        if n:
            o[:, :3] = np.concatenate([tree.tris, tree.tri_owned], axis=1).astype(np.int32).view(np.int64)
            o[:, 3] = vptr
            o[:, 4] = self.edges.data_ptr()
        self.objects = dev(o)
        self.view = RefView(2 * n - 1 if n else 0, n, self.nodes.data_ptr(), self.aabbs.data_ptr(),
                            self.cones.data_ptr(), self.objects.data_ptr())


class RefQueries:
    """The reference's query_device kernels over a tree: an snch_lbvh_gb300.Scene
    (through its byte-compatible snch_bvh_view) or a RefTree."""

    def __init__(self, scene):
        self.view = scene.view if isinstance(scene, RefTree) else scene.get_bvh_device_ptr()
        self._keep = scene
        self.L = lib()

    def _s(self, stream):
        import torch
        return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)

    def nearest(self, pts, out=None, stream=None):
        import torch
        n = pts.shape[0]
        idx, dist = out or (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, device="cuda"))
        rc = self.L.rg_nearest(C.byref(self.view), _p(pts), n, _p(idx), _p(dist), self._s(stream))
        assert rc == 0, rc
        return idx, dist

    def silhouette(self, pts, flip=None, out=None, stream=None):
        import torch
        n = pts.shape[0]
        dist = out if out is not None else torch.empty(n, device="cuda")
        rc = self.L.rg_silhouette(C.byref(self.view), _p(pts), _p(flip), n, _p(dist), self._s(stream))
        assert rc == 0, rc
        return dist

    def silhouette_edge(self, pts, flip=None, stream=None):
        """Distance and the silhouette edge the reference's traversal ended on."""
        import torch
        n = pts.shape[0]
        dist = torch.empty(n, device="cuda")
        edge = torch.empty(n, dtype=torch.int32, device="cuda")
        rc = self.L.rg_silhouette_edge(C.byref(self.view), _p(pts), _p(flip), n, _p(dist), _p(edge), self._s(stream))
        assert rc == 0, rc
        return dist, edge

    def ray(self, o, d, tmax, out=None, stream=None):
        import torch
        n = o.shape[0]
        hit, t, idx = out or (torch.empty(n, dtype=torch.uint8, device="cuda"), torch.empty(n, device="cuda"),
                              torch.empty(n, dtype=torch.int32, device="cuda"))
        rc = self.L.rg_ray(C.byref(self.view), _p(o), _p(d), _p(tmax), n, _p(hit), _p(t), _p(idx), self._s(stream))
        assert rc == 0, rc
        return hit, t, idx

    def ray_uv(self, o, d, tmax, stream=None):
        """Closest hit with its barycentric (u, v): hit, t, uv (n, 2), triangle index."""
        import torch
        n = o.shape[0]
        hit = torch.empty(n, dtype=torch.uint8, device="cuda")
        t = torch.empty(n, device="cuda")
        uv = torch.empty((n, 2), device="cuda")
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        rc = self.L.rg_ray_uv(C.byref(self.view), _p(o), _p(d), _p(tmax), n, _p(hit), _p(t), _p(uv), _p(idx),
                              self._s(stream))
        assert rc == 0, rc
        return hit, t, uv, idx

    def sample(self, c, r, u, out=None, stream=None):
        import torch
        n = c.shape[0]
        idx, pdf = out or (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, device="cuda"))
        rc = self.L.rg_sample(C.byref(self.view), _p(c), _p(r), _p(u), n, _p(idx), _p(pdf), self._s(stream))
        assert rc == 0, rc
        return idx, pdf
