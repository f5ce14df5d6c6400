"""Learned search radius for the nearest-primitive and nearest-silhouette queries.

A small MLP (Fourier features of the point, four 64-wide ReLU layers on the
tcgen05 tensor cores, a 2-output head) predicts log(distance to the nearest
triangle) and log(distance to the nearest silhouette edge). Its radius
``exp(prediction) * margin + floor`` seeds ``Scene.query_nearest_seeded`` /
``Scene.query_silhouette_seeded``: the traversal starts with that bound, and
every query whose bounded search finds nothing is re-run unbounded inside the
same call, so results are identical to the plain queries whatever the model
predicts. The reference has no learned bound; this is an addition on top of
its query semantics (include/snch_lbvh/core/query.cuh).

Training data comes from the plain queries themselves (``targets_from_scene``):
the exact distances of a set of sample points.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _dev, _ptr, _stream, _torch
from ._ffi import check, lib

__all__ = ["LearnedRadius", "targets_from_scene", "training_points", "gemm_bf16", "NUM_FREQ", "feature_scales"]

NUM_FREQ = 32


def feature_scales():
    """The frequency multipliers s_k = 2^(k/4) (as float32) of the features
    sin/cos(pi * s_k * u), u the point normalised to [-1, 1]^3 by the box."""
    return np.exp2(0.25 * np.arange(NUM_FREQ)).astype(np.float32)


class LearnedRadius:
    """An MLP radius model over the box [lo, hi] (query points are normalised by it)."""

    def __init__(self, box_lo, box_hi, seed: int = 0):
        self._h = C.c_void_p()
        lo = np.ascontiguousarray(box_lo, np.float32).reshape(3)
        hi = np.ascontiguousarray(box_hi, np.float32).reshape(3)
        check(lib().snch_mlp_create(lo.ctypes.data_as(C.c_void_p), hi.ctypes.data_as(C.c_void_p), C.c_uint64(seed),
                                    C.byref(self._h)))
        self.box_lo, self.box_hi = lo, hi

    def close(self):
        if self._h:
            lib().snch_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def num_params() -> int:
        return int(lib().snch_mlp_num_params())

    @property
    def params(self) -> np.ndarray:
        p = np.empty(self.num_params(), np.float32)
        check(lib().snch_mlp_get_params(self._h, p.ctypes.data_as(C.c_void_p), len(p)))
        return p

    @params.setter
    def params(self, value):
        p = np.ascontiguousarray(value, np.float32).reshape(-1)
        check(lib().snch_mlp_set_params(self._h, p.ctypes.data_as(C.c_void_p), len(p)))

    def gradient(self, points, targets, tau: float = 0.9, stream=None):
        """(gradient, loss) of the mean pinball loss at quantile tau; no update.

        The loss is minimised by the tau-quantile of the target: tau = 0.9 makes
        the predicted radius exceed the true distance for about 90 % of the
        points (the rest fall back to the unbounded search)."""
        torch = _torch()
        p, t = _dev(points, torch.float32, 3), _dev(targets, torch.float32, 2)
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_float()
        check(lib().snch_mlp_gradient(self._h, _ptr(p), _ptr(t), len(p), C.c_float(tau),
                                      g.ctypes.data_as(C.c_void_p), C.byref(loss), _stream(stream)))
        return g, float(loss.value)

    def train(self, points, targets, epochs: int = 1, batch: int = 65536, lr: float = 2e-3, tau: float = 0.9,
              stream=None) -> float:
        """Adam over `epochs` passes; returns the mean loss of the last epoch."""
        torch = _torch()
        p, t = _dev(points, torch.float32, 3), _dev(targets, torch.float32, 2)
        loss = C.c_float()
        check(lib().snch_mlp_train(self._h, _ptr(p), _ptr(t), len(p), epochs, batch, C.c_float(lr), C.c_float(tau),
                                   C.byref(loss), _stream(stream)))
        return float(loss.value)

    def predict(self, points, margin: float = 1.25, floor: float = 0.0, stream=None, out=None, which="both"):
        """Radii (r_near, r_sil) as CUDA tensors; which = "both" | "near" | "sil"."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        n = len(p)
        if out is None:
            rn = torch.empty(n, device=p.device, dtype=torch.float32) if which in ("both", "near") else None
            rs = torch.empty(n, device=p.device, dtype=torch.float32) if which in ("both", "sil") else None
        else:
            rn, rs = out
        check(lib().snch_mlp_predict_radius(self._h, _ptr(p), n, C.c_float(margin), C.c_float(floor), _ptr(rn),
                                            _ptr(rs), _stream(stream)))
        return rn, rs


def training_points(verts, faces, n_uniform: int, n_surface: int, band: float = 0.05, lo=(0, 0, 0), hi=(1, 1, 1),
                    seed: int = 0):
    """Sample points for training: n_uniform U(box) and n_surface near the mesh (a
    uniform point of a random triangle moved along its normal by N(0, (band/3)^2)),
    clipped to the box. float32 [n_uniform + n_surface, 3]."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    u = lo + (hi - lo) * rng.random((n_uniform, 3), dtype=np.float32)
    t = rng.integers(0, len(faces), n_surface)
    a, b, c = (np.asarray(verts, np.float32)[np.asarray(faces)[t, i]] for i in range(3))
    r1, r2 = rng.random(n_surface, dtype=np.float32), rng.random(n_surface, dtype=np.float32)
    s1 = np.sqrt(r1)
    p = a * (1 - s1)[:, None] + b * (s1 * (1 - r2))[:, None] + c * (s1 * r2)[:, None]
    nrm = np.cross(b - a, c - a)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    p = p + nrm * rng.normal(0.0, band / 3.0, (n_surface, 1)).astype(np.float32)
    return np.clip(np.concatenate([u, p.astype(np.float32)]), lo, hi).astype(np.float32)


def targets_from_scene(scene, points, flip=None, stream=None):
    """Training targets [n x 2]: log of the exact nearest-triangle and
    nearest-silhouette distances (NaN where there is no silhouette edge)."""
    torch = _torch()
    p = _dev(points, torch.float32, 3)
    _, dn = scene.query_nearest(p, stream=stream)
    ds, _ = scene.query_silhouette(p, flip, stream=stream)
    t = torch.stack([dn, ds], dim=1)
    t = torch.where(torch.isfinite(t) & (t > 0), t, torch.full_like(t, float("nan")))
    return torch.log(t)


def gemm_bf16(A, B, C_out=None, accumulate=False, status=None, stream=None):
    """C[M x N] (+)= A[M x K] @ B[N x K]^T on the tensor cores (bf16 in, fp32 out)."""
    torch = _torch()
    A, B = A.contiguous(), B.contiguous()  # kept alive until the call returns
    M, K = A.shape
    N = B.shape[0]
    if C_out is None:
        C_out = torch.zeros(M, N, device=A.device, dtype=torch.float32)
    if status is None:
        status = torch.zeros(1, device=A.device, dtype=torch.int32)
    check(lib().snch_gemm_bf16(_ptr(A), _ptr(B), _ptr(C_out), M, N, K, int(accumulate), _ptr(status),
                               _stream(stream)))
    return C_out, status
