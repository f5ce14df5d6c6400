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
        L.rg_ray.argtypes = [P, P, P, P, I, P, P, P, P]
        L.rg_sample.argtypes = [P, P, P, P, I, P, P, P]
        rc = L.rg_load(CUBIN.encode())
        if rc != 0:
            raise RuntimeError(f"loading the reference cubin failed: cudaError {rc}")
        _lib = L
    return _lib


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class RefQueries:
    """The reference's query_device kernels over `scene` (an snch_lbvh_gb300.Scene)."""

    def __init__(self, scene):
        self.view = scene.get_bvh_device_ptr()
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

    def ray(self, o, d, tmax, out=None, stream=None):
        import torch
        n = o.shape[0]
        hit, t, idx = out or (torch.empty(n, dtype=torch.uint8, device="cuda"), torch.empty(n, device="cuda"),
                              torch.empty(n, dtype=torch.int32, device="cuda"))
        rc = self.L.rg_ray(C.byref(self.view), _p(o), _p(d), _p(tmax), n, _p(hit), _p(t), _p(idx), self._s(stream))
        assert rc == 0, rc
        return hit, t, idx

    def sample(self, c, r, u, out=None, stream=None):
        import torch
        n = c.shape[0]
        idx, pdf = out or (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, device="cuda"))
        rc = self.L.rg_sample(C.byref(self.view), _p(c), _p(r), _p(u), n, _p(idx), _p(pdf), self._s(stream))
        assert rc == 0, rc
        return idx, pdf
