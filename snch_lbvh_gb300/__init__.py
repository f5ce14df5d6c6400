"""GB300-native SNCH-LBVH: host-side mirror of the reference's scene API.

``Scene`` follows ``lbvh::scene<3>`` of tyanyuy3125/snch-lbvh
(include/snch_lbvh/scene.cuh:704-1267): construct from vertices and
triangles, ``compute_silhouettes()``, ``build_bvh()``, ``get_bvh_device_ptr()``,
then the four queries of include/snch_lbvh/core/query.cuh and sample.cuh.
Every call goes through the C ABI of libsnch_gb300.so (include/snch_gb300.h);
PyTorch only provides device memory and streams.

Device-buffer calls take CUDA tensors and are asynchronous on the current
torch stream (or ``stream=``); the ``*_host`` forms take NumPy arrays and
return NumPy arrays (copies pipelined inside the library).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _ffi
from ._ffi import BvhView, SnchError, check, lib  # noqa: F401

__all__ = ["Scene", "BatchedScene", "Scene2", "Graph", "SnchError", "BvhView", "lib", "read_obj",
           "cached_memory_bytes", "release_cached_memory"]

INVALID = 0xFFFFFFFF
TRAVERSAL_NEAR_FIRST = 0
TRAVERSAL_REFERENCE_ORDER = 1
OPT_TRAVERSAL, OPT_QUERY_ORDER, OPT_ORDER_MIN_BATCH, OPT_PERSISTENT, OPT_TAIL_CAP = 1, 2, 3, 4, 5
OPT_NODE_WIDTH, OPT_NODE_WIDTH_NEAREST, OPT_NODE_WIDTH_SILHOUETTE = 6, 7, 8
OPT_BLOCK, OPT_BLOCK_NEAREST, OPT_BLOCK_SILHOUETTE = 9, 10, 11
OPT_PACKET, OPT_PACKET_NEAREST, OPT_PACKET_SILHOUETTE = 12, 13, 14
OPT_HOST_CHUNK = 15
OPT_PERSISTENT_NEAREST, OPT_PERSISTENT_SILHOUETTE = 16, 17
OPT_PERSISTENT_RAY = 18
OPT_PACKET_PERSISTENT_MIN = 19
OPT_OUTPUT_SCATTER = 20
OPT_TOP_LEVELS = 21
OPT_RAY_ORDER = 22
OPT_ORDER_BITS = 23


def _torch():
    import torch
    return torch


def _stream(stream):
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _dev(x, dtype, cols=None):
    torch = _torch()
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(np.ascontiguousarray(x))
    x = x.to(device="cuda", dtype=dtype).contiguous()
    if cols is not None:
        x = x.reshape(-1, cols)
    return x


def _host(x, dtype, cols=None):
    a = np.ascontiguousarray(x, dtype=dtype)
    return a.reshape(-1, cols) if cols else a.reshape(-1)


def read_obj(path):
    """scene_loader<3>(path) scene_loader.cuh:86-152: (vertices float32 [V, 3],
    triangles int32 [T, 3], 0-based) of a Wavefront OBJ file."""
    L = lib()
    p = C.cast(C.c_char_p(os.fsencode(path)), C.c_void_p)
    nv, nt = C.c_int64(), C.c_int64()
    check(L.snch_obj_read(p, None, 0, None, 0, C.byref(nv), C.byref(nt)))
    v = np.empty((nv.value, 3), np.float32)
    t = np.empty((nt.value, 3), np.int32)
    check(L.snch_obj_read(p, v.ctypes.data_as(C.c_void_p), nv.value, t.ctypes.data_as(C.c_void_p), nt.value,
                          C.byref(nv), C.byref(nt)))
    return v, t


def cached_memory_bytes():
    """Bytes of released scene arrays this library holds for reuse."""
    return int(lib().snch_cached_memory_bytes())


def release_cached_memory():
    """Return the held scene arrays and the scratch pool to the driver."""
    check(lib().snch_release_cached_memory())


class Scene:
    """lbvh::scene<3>: a triangle mesh, its silhouette edges and its SNCH-LBVH."""

    def __init__(self, vertices, triangles, stream=None):
        self._h = C.c_void_p()
        torch = _torch()
        L = lib()
        if isinstance(vertices, torch.Tensor) and vertices.is_cuda:
            v = vertices.to(torch.float32).contiguous()
            t = triangles.to(device=v.device, dtype=torch.int32).contiguous()
            check(L.snch_scene_create_device(_ptr(v), v.numel() // 3, _ptr(t), t.numel() // 3, C.byref(self._h),
                                             _stream(stream)))
        else:
            v = _host(vertices, np.float32, 3)
            t = _host(triangles, np.int32, 3)
            check(L.snch_scene_create(v.ctypes.data_as(C.c_void_p), len(v), t.ctypes.data_as(C.c_void_p), len(t),
                                      C.byref(self._h)))

    def save(self, path, stream=None):
        """Writes the built scene to a flat binary file (snch_scene_save)."""
        check(lib().snch_scene_save(self._h, C.cast(C.c_char_p(os.fsencode(path)), C.c_void_p), _stream(stream)))

    @classmethod
    def load(cls, path, stream=None):
        """A built Scene read from a file written by save() (no rebuild)."""
        s = cls.__new__(cls)
        s._h = C.c_void_p()
        check(lib().snch_scene_load(C.cast(C.c_char_p(os.fsencode(path)), C.c_void_p), C.byref(s._h),
                                    _stream(stream)))
        return s

    # ------------------------------------------------------------ lifetime
    def close(self):
        if self._h:
            check(lib().snch_scene_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ build
    def compute_silhouettes(self, stream=None):
        """scene<3>::compute_silhouettes() scene.cuh:1167."""
        check(lib().snch_compute_silhouettes(self._h, _stream(stream)))

    def build_bvh(self, stream=None):
        """scene<3>::build_bvh() scene.cuh:1205."""
        check(lib().snch_build_bvh(self._h, _stream(stream)))

    def get_bvh_device_ptr(self) -> BvhView:
        """scene<3>::get_bvh_device_ptr() scene.cuh:1242; raises SnchError("BVH is not built yet.")."""
        v = BvhView()
        check(lib().snch_get_bvh_view(self._h, C.byref(v)))
        return v

    def get_traversal_view(self):
        """The tree in the traversal layout for snch_device.cuh's per-thread queries
        (snch_traversal_view); valid until the scene is rebuilt or destroyed."""
        v = _ffi.TraversalView()
        check(lib().snch_get_traversal_view(self._h, C.byref(v)))
        return v

    def set_traversal(self, mode: int):
        """TRAVERSAL_NEAR_FIRST (default) or TRAVERSAL_REFERENCE_ORDER; same results."""
        check(lib().snch_set_traversal(self._h, int(mode)))

    def set_option(self, option: int, value: int):
        """OPT_TRAVERSAL, OPT_QUERY_ORDER (Morton-sorted batches), OPT_ORDER_MIN_BATCH,
        OPT_PERSISTENT, OPT_TAIL_CAP, OPT_NODE_WIDTH[_NEAREST|_SILHOUETTE] (2, 4 or 8)."""
        check(lib().snch_set_option(self._h, int(option), int(value)))

    def leaf_ranks(self):
        n = self.num_triangles
        r = np.empty(n, np.uint32)
        check(lib().snch_export_leaf_ranks(self._h, r.ctypes.data_as(C.c_void_p)))
        return r

    def info(self):
        nv, nt, ne = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().snch_scene_info(self._h, C.byref(nv), C.byref(nt), C.byref(ne)))
        return nv.value, nt.value, ne.value

    @property
    def num_triangles(self):
        return self.info()[1]

    def device_status(self, reset=True, stream=None) -> int:
        out = C.c_uint32()
        check(lib().snch_get_device_status(self._h, C.byref(out), int(reset), _stream(stream)))
        return out.value

    # ------------------------------------------------------------ exports (parity checks)
    def export_tree(self, stream=None):
        torch = _torch()
        n = self.num_triangles
        nn = max(2 * n - 1, 0)
        d = {k: torch.empty(s, dtype=torch.int32, device="cuda") for k, s in
             [("morton", n), ("sorted_idx", n), ("nodes", (nn, 4))]}
        d["aabbs"] = torch.empty((nn, 6), dtype=torch.float32, device="cuda")
        d["cones"] = torch.empty((nn, 5), dtype=torch.float32, device="cuda")
        check(lib().snch_export_tree(self._h, _ptr(d["morton"]), _ptr(d["sorted_idx"]), _ptr(d["nodes"]),
                                     _ptr(d["aabbs"]), _ptr(d["cones"]), _stream(stream)))
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        out = {k: v.cpu().numpy() for k, v in d.items()}
        for k in ("morton", "sorted_idx", "nodes"):
            out[k] = out[k].view(np.uint32)
        return out

    def export_topology(self, stream=None):
        torch = _torch()
        _, n, ne = self.info()
        te = torch.empty((n, 3), dtype=torch.int32, device="cuda")
        to = torch.empty((n, 3), dtype=torch.int32, device="cuda")
        ev = torch.empty((max(ne, 0), 4), dtype=torch.int32, device="cuda")
        check(lib().snch_export_topology(self._h, _ptr(te), _ptr(to), _ptr(ev), _stream(stream)))
        torch.cuda.synchronize()
        return te.cpu().numpy(), to.cpu().numpy(), ev.cpu().numpy()

    def query_visits(self, kind: str, *inputs, flip=None, stream=None):
        """Per-query work counters {internal nodes, leaves, silhouette edges} of the
        traversal the library runs, for kind in nearest|silhouette|ray|sample."""
        torch = _torch()
        k = {"nearest": 0, "silhouette": 1, "ray": 2, "sample": 3}[kind]
        cols = {0: [3], 1: [3], 2: [3, 3, None], 3: [3, None, None]}[k]
        ins = [_dev(x, torch.float32, c) for x, c in zip(inputs, cols)]
        ins += [None] * (3 - len(ins))
        n = ins[0].shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
        check(lib().snch_query_visits(self._h, k, _ptr(ins[0]), _ptr(ins[1]), _ptr(ins[2]), _ptr(f), n, _ptr(out),
                                      _stream(stream)))
        return out.cpu().numpy().view(np.uint32)

    def query_visits_seeded(self, kind: str, points, radius, flip=None, stream=None):
        """The same counters for the seeded first pass of a nearest / silhouette
        search started at the given radii (queries with nothing inside their
        radius would go to an unbounded pass, not counted here)."""
        torch = _torch()
        k = {"nearest": 0, "silhouette": 1}[kind]
        p = _dev(points, torch.float32, 3)
        r = _dev(radius, torch.float32)
        f = None if flip is None else _dev(flip, torch.uint8)
        n = p.shape[0]
        out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
        check(lib().snch_query_visits_seeded(self._h, k, _ptr(p), _ptr(f), _ptr(r), n, _ptr(out), _stream(stream)))
        return out.cpu().numpy().view(np.uint32)

    def vertices(self):
        """The scene's device vertex buffer as a (V, 3) float32 CUDA tensor view
        (write moved vertices here before the next build_bvh)."""
        torch = _torch()
        ptr = C.c_void_p()
        check(lib().snch_scene_vertices(self._h, C.byref(ptr)))
        nv, _, _ = self.info()
        if nv == 0:
            return torch.zeros((0, 3), dtype=torch.float32, device="cuda")
        return _wrap_device(ptr.value, (nv, 3))

    def capture(self, rebuild=True, near_points=None, near_out=None, sil_points=None, sil_flip=None, sil_out=None,
                near_mesh=None, sil_mesh=None, stream=None):
        """Captures [rebuild +] one nearest and one silhouette batch into a CUDA graph
        (Graph.launch() replays it on the same buffers, which the caller refills)."""
        return Graph(self, rebuild, near_points, near_out, sil_points, sil_flip, sil_out, near_mesh, sil_mesh,
                     stream)

    def get_option(self, option):
        v = C.c_int64()
        check(lib().snch_get_option(self._h, option, C.byref(v)))
        return int(v.value)

    def search_config(self, which: str = "nearest"):
        """(node width, threads per block, OPT_PACKET mode, OPT_PERSISTENT) of the
        nearest or silhouette search."""
        w, b = C.c_int32(), C.c_int32()
        k = {"nearest": 0, "silhouette": 1}[which]
        check(lib().snch_get_search_config(self._h, k, C.byref(w), C.byref(b)))
        return (int(w.value), int(b.value), self.get_option((OPT_PACKET_NEAREST, OPT_PACKET_SILHOUETTE)[k]),
                self.get_option((OPT_PERSISTENT_NEAREST, OPT_PERSISTENT_SILHOUETTE)[k]))

    def node_width(self, which: str = "nearest") -> int:
        return self.search_config(which)[0]

    # (node width, threads per block, OPT_PACKET, OPT_PERSISTENT): warp packets, one query
    # per traversal, persistent work-stealing lanes
    AUTOTUNE_CONFIGS = ((2, 128, 1, 0), (2, 128, 0, 0), (4, 128, 0, 0), (8, 128, 0, 0), (2, 64, 0, 0),
                        (2, 256, 0, 0), (2, 128, 0, 1))

    def autotune(self, near_points=None, sil_points=None, sil_flip=None, near_mesh=None, sil_mesh=None,
                 stream=None):
        """Times the nearest / silhouette searches in each (node width, threads per
        block, packet mode, persistent) of AUTOTUNE_CONFIGS on these sample batches and
        keeps the fastest per type (same distances in every configuration). Returns
        {"nearest": {(width, block, packet, persistent): ms, ...}, "silhouette": {...}}."""
        torch = _torch()
        pn = None if near_points is None else _dev(near_points, torch.float32, 3)
        ps = None if sil_points is None else _dev(sil_points, torch.float32, 3)
        f = None if sil_flip is None else _dev(sil_flip, torch.uint8)
        mn = None if near_mesh is None else _dev(near_mesh, torch.int32)
        ms_ = None if sil_mesh is None else _dev(sil_mesh, torch.int32)
        k = len(self.AUTOTUNE_CONFIGS)
        out = (C.c_float * (2 * k))()
        check(lib().snch_autotune(self._h, _ptr(mn), _ptr(pn), 0 if pn is None else pn.shape[0], _ptr(ms_), _ptr(ps),
                                  _ptr(f), 0 if ps is None else ps.shape[0], C.cast(out, C.c_void_p),
                                  _stream(stream)))
        return {"nearest": dict(zip(self.AUTOTUNE_CONFIGS, out[0:k])),
                "silhouette": dict(zip(self.AUTOTUNE_CONFIGS, out[k:2 * k]))}

    # ------------------------------------------------------------ device-buffer queries
    def query_nearest(self, points, stream=None, out=None):
        """query_device(nearest) query.cuh:239 -> (index int32 [-1 = none], distance)."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        n = p.shape[0]
        idx, dist = out if out is not None else (torch.empty(n, dtype=torch.int32, device="cuda"),
                                                 torch.empty(n, dtype=torch.float32, device="cuda"))
        check(lib().snch_query_nearest(self._h, _ptr(p), n, _ptr(idx), _ptr(dist), _stream(stream)))
        return idx, dist

    def query_nearest_seeded(self, points, radius, stream=None, out=None, num_fallback=None):
        """Nearest query whose search starts at a per-query radius; same results as query_nearest."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        r = _dev(radius, torch.float32)
        n = p.shape[0]
        idx, dist = out if out is not None else (torch.empty(n, dtype=torch.int32, device="cuda"),
                                                 torch.empty(n, dtype=torch.float32, device="cuda"))
        check(lib().snch_query_nearest_seeded(self._h, _ptr(p), _ptr(r), n, _ptr(idx), _ptr(dist), _ptr(num_fallback),
                                              _stream(stream)))
        return idx, dist

    def query_silhouette_seeded(self, points, radius, flip=None, stream=None, out=None, num_fallback=None):
        """Silhouette query whose search starts at a per-query radius; same results as query_silhouette."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        r = _dev(radius, torch.float32)
        n = p.shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        dist, edge = out if out is not None else (torch.empty(n, dtype=torch.float32, device="cuda"),
                                                  torch.empty(n, dtype=torch.int32, device="cuda"))
        check(lib().snch_query_silhouette_seeded(self._h, _ptr(p), _ptr(f), _ptr(r), n, _ptr(dist), _ptr(edge),
                                                 _ptr(num_fallback), _stream(stream)))
        return dist, edge

    def query_silhouette(self, points, flip=None, stream=None, out=None):
        """query_device(nearest_silhouette) query.cuh:326 -> (distance, edge id or -1)."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        n = p.shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        dist, edge = out if out is not None else (torch.empty(n, dtype=torch.float32, device="cuda"),
                                                  torch.empty(n, dtype=torch.int32, device="cuda"))
        check(lib().snch_query_silhouette(self._h, _ptr(p), _ptr(f), n, _ptr(dist), _ptr(edge), _stream(stream)))
        return dist, edge

    def query_overlap(self, boxes, max_per_query=64, stream=None):
        """query_device(overlaps(box)) query.cuh:177: (index [n, max] int32, -1 padded; count [n])."""
        torch = _torch()
        b = _dev(boxes, torch.float32, 6)
        n = b.shape[0]
        idx = torch.full((n, max_per_query), -1, dtype=torch.int32, device="cuda")
        cnt = torch.empty(n, dtype=torch.int32, device="cuda")
        check(lib().snch_query_overlap(self._h, _ptr(b), n, int(max_per_query), _ptr(idx), _ptr(cnt),
                                       _stream(stream)))
        return idx, cnt

    def query_line(self, origins, dirs, max_per_query=64, stream=None):
        """query_device(line_intersect(line)) query.cuh:15: (index [n, max], t [n, max], count [n])."""
        torch = _torch()
        o = _dev(origins, torch.float32, 3)
        d = _dev(dirs, torch.float32, 3)
        n = o.shape[0]
        idx = torch.full((n, max_per_query), -1, dtype=torch.int32, device="cuda")
        tt = torch.full((n, max_per_query), float("nan"), dtype=torch.float32, device="cuda")
        cnt = torch.empty(n, dtype=torch.int32, device="cuda")
        check(lib().snch_query_line(self._h, _ptr(o), _ptr(d), n, int(max_per_query), _ptr(idx), _ptr(tt), _ptr(cnt),
                                    _stream(stream)))
        return idx, tt, cnt

    def query_ray(self, origins, dirs, tmax, stream=None, out=None):
        """query_device(ray_intersect) query.cuh:82 -> (hit uint8, t, uv [n,2], index int32)."""
        torch = _torch()
        o, d = _dev(origins, torch.float32, 3), _dev(dirs, torch.float32, 3)
        tm = _dev(tmax, torch.float32)
        n = o.shape[0]
        if out is None:
            out = (torch.empty(n, dtype=torch.uint8, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"),
                   torch.empty((n, 2), dtype=torch.float32, device="cuda"),
                   torch.empty(n, dtype=torch.int32, device="cuda"))
        hit, t, uv, idx = out
        check(lib().snch_query_ray(self._h, _ptr(o), _ptr(d), _ptr(tm), n, _ptr(hit), _ptr(t), _ptr(uv), _ptr(idx),
                                   _stream(stream)))
        return hit, t, uv, idx

    def query_ray_test(self, origins, dirs, tmax, stream=None, out=None):
        """ray_intersect<TestOnly = true> query.cuh:117-121: occlusion test -> hit uint8."""
        torch = _torch()
        o, d = _dev(origins, torch.float32, 3), _dev(dirs, torch.float32, 3)
        tm = _dev(tmax, torch.float32)
        n = o.shape[0]
        hit = out if out is not None else torch.empty(n, dtype=torch.uint8, device="cuda")
        check(lib().snch_query_ray_test(self._h, _ptr(o), _ptr(d), _ptr(tm), n, _ptr(hit), _stream(stream)))
        return hit

    def sample_in_sphere(self, centers, radii, u, stream=None, out=None):
        """sample_object_in_sphere sample.cuh:26 -> (index or -1, pdf)."""
        torch = _torch()
        c = _dev(centers, torch.float32, 3)
        r, uu = _dev(radii, torch.float32), _dev(u, torch.float32)
        n = c.shape[0]
        idx, pdf = out if out is not None else (torch.empty(n, dtype=torch.int32, device="cuda"),
                                                torch.empty(n, dtype=torch.float32, device="cuda"))
        check(lib().snch_sample_in_sphere(self._h, _ptr(c), _ptr(r), _ptr(uu), n, _ptr(idx), _ptr(pdf),
                                          _stream(stream)))
        return idx, pdf

    def sample_on_object(self, index, u, v, stream=None):
        """sample_on_object sample.cuh:10 -> points [n,3]."""
        torch = _torch()
        i = _dev(index, torch.int32)
        uu, vv = _dev(u, torch.float32), _dev(v, torch.float32)
        out = torch.empty((i.shape[0], 3), dtype=torch.float32, device="cuda")
        check(lib().snch_sample_on_object(self._h, _ptr(i), _ptr(uu), _ptr(vv), i.shape[0], _ptr(out),
                                          _stream(stream)))
        return out

    # ------------------------------------------------------------ host-buffer queries
    def query_nearest_host(self, points, out=None):
        p = _host(points, np.float32, 3)
        n = len(p)
        idx, dist = out if out is not None else (np.empty(n, np.uint32), np.empty(n, np.float32))
        check(lib().snch_query_nearest_host(self._h, p.ctypes.data_as(C.c_void_p), n,
                                            idx.ctypes.data_as(C.c_void_p), dist.ctypes.data_as(C.c_void_p)))
        return idx, dist

    def query_silhouette_host(self, points, flip=None, out=None):
        p = _host(points, np.float32, 3)
        n = len(p)
        f = None if flip is None else _host(flip, np.uint8)
        dist, edge = out if out is not None else (np.empty(n, np.float32), np.empty(n, np.int32))
        check(lib().snch_query_silhouette_host(self._h, p.ctypes.data_as(C.c_void_p),
                                               None if f is None else f.ctypes.data_as(C.c_void_p), n,
                                               dist.ctypes.data_as(C.c_void_p), edge.ctypes.data_as(C.c_void_p)))
        return dist, edge

    def query_ray_host(self, origins, dirs, tmax, out=None):
        o, d, tm = _host(origins, np.float32, 3), _host(dirs, np.float32, 3), _host(tmax, np.float32)
        n = len(o)
        if out is None:
            out = (np.empty(n, np.uint8), np.empty(n, np.float32), np.empty((n, 2), np.float32), np.empty(n, np.uint32))
        hit, t, uv, idx = out
        vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        check(lib().snch_query_ray_host(self._h, vp(o), vp(d), vp(tm), n, vp(hit), vp(t), vp(uv), vp(idx)))
        return hit, t, uv, idx

    def sample_in_sphere_host(self, centers, radii, u, out=None):
        c, r, uu = _host(centers, np.float32, 3), _host(radii, np.float32), _host(u, np.float32)
        n = len(c)
        idx, pdf = out if out is not None else (np.empty(n, np.int32), np.empty(n, np.float32))
        vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        check(lib().snch_sample_in_sphere_host(self._h, vp(c), vp(r), vp(uu), n, vp(idx), vp(pdf)))
        return idx, pdf


def _wrap_device(addr, shape):
    """A float32 CUDA tensor viewing library-owned device memory (no copy)."""
    torch = _torch()
    n = int(np.prod(shape))

    class _Mem:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (int(addr), False), "version": 3}

    return torch.as_tensor(_Mem(), device="cuda").view(*shape)


class Graph:
    """A captured solver step (snch_graph_create): the tensors given at capture are
    the graph's inputs and outputs; refill them in place between launches."""

    def __init__(self, scene, rebuild, near_points, near_out, sil_points, sil_flip, sil_out, near_mesh, sil_mesh,
                 stream):
        torch = _torch()
        self._h = C.c_void_p()
        self._keep = [scene, near_points, near_out, sil_points, sil_flip, sil_out, near_mesh, sil_mesh]
        for x in (near_points, sil_points, sil_flip, near_mesh, sil_mesh):
            assert x is None or (torch.is_tensor(x) and x.is_cuda and x.is_contiguous()), \
                "graph inputs must be contiguous CUDA tensors (their addresses are captured)"
        nn = 0 if near_points is None else near_points.shape[0]
        ns = 0 if sil_points is None else sil_points.shape[0]
        ni, nd = near_out if near_out is not None else (None, None)
        sd, se = sil_out if sil_out is not None else (None, None)
        st = stream if stream is not None else torch.cuda.current_stream()
        if st.cuda_stream == 0:
            raise SnchError(-1, "capture needs a created stream (torch.cuda.Stream()), not the default stream")
        check(lib().snch_graph_create(scene._h, int(bool(rebuild)), _ptr(near_mesh), _ptr(near_points), nn,
                                      _ptr(ni), _ptr(nd), _ptr(sil_mesh), _ptr(sil_points), _ptr(sil_flip), ns,
                                      _ptr(sd), _ptr(se), C.byref(self._h), C.c_void_p(st.cuda_stream)))

    def launch(self, stream=None):
        check(lib().snch_graph_launch(self._h, _stream(stream)))

    def close(self):
        if self._h:
            lib().snch_graph_destroy(self._h)
            self._h = None
            self._keep = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchedScene(Scene):
    """Many independent meshes in one scene: one silhouette pass, one LBVH build
    and one query launch for all of them (snch_batch_* in the C ABI). Each mesh's
    subtree is the tree a ``Scene`` of that mesh alone gets, and the batched
    queries return what that scene's queries return (per-mesh triangle index and
    edge id)."""

    def __init__(self, meshes, stream=None):
        """meshes: sequence of (vertices [nv, 3], triangles [nt, 3]) with per-mesh
        vertex indices; NumPy arrays, or CUDA tensors (all of them)."""
        self._h = C.c_void_p()
        torch = _torch()
        device = len(meshes) > 0 and isinstance(meshes[0][0], torch.Tensor) and meshes[0][0].is_cuda
        vs = np.zeros(len(meshes) + 1, np.int64)
        ts = np.zeros(len(meshes) + 1, np.int64)
        for m, (v, t) in enumerate(meshes):
            vs[m + 1] = vs[m] + len(v)
            ts[m + 1] = ts[m] + len(t)
        self.vert_start, self.tri_start = vs, ts
        L = lib()
        if device:
            v = torch.cat([x.to(torch.float32).reshape(-1, 3) for x, _ in meshes]).contiguous()
            t = torch.cat([y.to(device=v.device, dtype=torch.int32).reshape(-1, 3) for _, y in meshes]).contiguous()
            vp, tp = _ptr(v), _ptr(t)
        else:
            v = np.ascontiguousarray(np.concatenate([np.zeros((0, 3), np.float32)] +
                                                    [_host(x, np.float32, 3) for x, _ in meshes]), np.float32)
            t = np.ascontiguousarray(np.concatenate([np.zeros((0, 3), np.int32)] +
                                                    [_host(y, np.int32, 3) for _, y in meshes]), np.int32)
            vp, tp = v.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p)
        check(L.snch_batch_create(vp, int(vs[-1]), tp, int(ts[-1]), vs.ctypes.data_as(C.c_void_p),
                                  ts.ctypes.data_as(C.c_void_p), len(meshes), int(device), C.byref(self._h),
                                  _stream(stream)))

    @property
    def num_meshes(self) -> int:
        m = C.c_int32()
        check(lib().snch_batch_num_meshes(self._h, C.byref(m)))
        return int(m.value)

    def query_nearest_batch(self, mesh, points, stream=None, out=None):
        """(index within the mesh, int32 [-1 = none], distance) for each (mesh, point)."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        m = _dev(mesh, torch.int32)
        n = p.shape[0]
        idx, dist = out if out is not None else (torch.empty(n, dtype=torch.int32, device="cuda"),
                                                 torch.empty(n, dtype=torch.float32, device="cuda"))
        check(lib().snch_batch_query_nearest(self._h, _ptr(m), _ptr(p), n, _ptr(idx), _ptr(dist), _stream(stream)))
        return idx, dist

    def query_silhouette_batch(self, mesh, points, flip=None, stream=None, out=None):
        """(distance, edge id within the mesh or -1) for each (mesh, point)."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        m = _dev(mesh, torch.int32)
        n = p.shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        dist, edge = out if out is not None else (torch.empty(n, dtype=torch.float32, device="cuda"),
                                                  torch.empty(n, dtype=torch.int32, device="cuda"))
        check(lib().snch_batch_query_silhouette(self._h, _ptr(m), _ptr(p), _ptr(f), n, _ptr(dist), _ptr(edge),
                                                _stream(stream)))
        return dist, edge

    def query_nearest_batch_seeded(self, mesh, points, radius, stream=None, num_fallback=None):
        """query_nearest_batch seeded with per-query radii (same results)."""
        torch = _torch()
        p, m, r = _dev(points, torch.float32, 3), _dev(mesh, torch.int32), _dev(radius, torch.float32)
        n = p.shape[0]
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        check(lib().snch_batch_query_nearest_seeded(self._h, _ptr(m), _ptr(p), _ptr(r), n, _ptr(idx), _ptr(dist),
                                                    _ptr(num_fallback), _stream(stream)))
        return idx, dist

    def query_silhouette_batch_seeded(self, mesh, points, radius, flip=None, stream=None, num_fallback=None):
        """query_silhouette_batch seeded with per-query radii (same results)."""
        torch = _torch()
        p, m, r = _dev(points, torch.float32, 3), _dev(mesh, torch.int32), _dev(radius, torch.float32)
        n = p.shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        edge = torch.empty(n, dtype=torch.int32, device="cuda")
        check(lib().snch_batch_query_silhouette_seeded(self._h, _ptr(m), _ptr(p), _ptr(r), _ptr(f), n, _ptr(dist),
                                                       _ptr(edge), _ptr(num_fallback), _stream(stream)))
        return dist, edge


class Scene2:
    """lbvh::scene<2> (scene.cuh:287-703): line segments with silhouette vertices
    and their SNCH-LBVH; queries on CUDA tensors of 2D points."""

    def __init__(self, vertices, segments):
        self._h = C.c_void_p()
        v = _host(vertices, np.float32, 2)
        s = _host(segments, np.int32, 2)
        check(lib().snch_scene2_create(v.ctypes.data_as(C.c_void_p), len(v), s.ctypes.data_as(C.c_void_p), len(s),
                                       C.byref(self._h)))
        self.num_vertices, self.num_segments = len(v), len(s)

    def close(self):
        if self._h:
            lib().snch_scene2_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, stream=None):
        """compute_silhouettes() + build_bvh() scene.cuh:642-683."""
        check(lib().snch_scene2_build(self._h, _stream(stream)))

    def device_status(self, reset=True, stream=None) -> int:
        b = C.c_uint32()
        check(lib().snch_scene2_get_device_status(self._h, C.byref(b), int(reset), _stream(stream)))
        return int(b.value)

    def export(self, stream=None):
        torch = _torch()
        n, nv = self.num_segments, self.num_vertices
        nn = max(2 * n - 1, 0)
        out = {"sv": torch.empty((nv, 4), dtype=torch.int32, device="cuda"),
               "seg_owned": torch.empty((n, 2), dtype=torch.int32, device="cuda"),
               "morton": torch.empty(n, dtype=torch.int32, device="cuda"),
               "sorted_idx": torch.empty(n, dtype=torch.int32, device="cuda"),
               "nodes": torch.empty((nn, 4), dtype=torch.int32, device="cuda"),
               "aabbs": torch.empty((nn, 4), dtype=torch.float32, device="cuda"),
               "cones": torch.empty((nn, 4), dtype=torch.float32, device="cuda")}
        check(lib().snch_scene2_export(self._h, *[_ptr(out[k]) for k in ("sv", "seg_owned", "morton", "sorted_idx",
                                                                         "nodes", "aabbs", "cones")],
                                       _stream(stream)))
        torch.cuda.synchronize()
        r = {k: x.cpu().numpy() for k, x in out.items()}
        for k in ("morton", "sorted_idx", "nodes"):
            r[k] = r[k].view(np.uint32)
        return r

    def query_nearest(self, points, stream=None):
        torch = _torch()
        p = _dev(points, torch.float32, 2)
        n = p.shape[0]
        idx, dist = torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda")
        check(lib().snch_scene2_query_nearest(self._h, _ptr(p), n, _ptr(idx), _ptr(dist), _stream(stream)))
        return idx, dist

    def query_silhouette(self, points, flip=None, stream=None):
        torch = _torch()
        p = _dev(points, torch.float32, 2)
        n = p.shape[0]
        f = None if flip is None else _dev(flip, torch.uint8)
        dist, vid = torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")
        check(lib().snch_scene2_query_silhouette(self._h, _ptr(p), _ptr(f), n, _ptr(dist), _ptr(vid),
                                                 _stream(stream)))
        return dist, vid

    def query_ray(self, origins, dirs, tmax, stream=None):
        torch = _torch()
        o, d, tm = _dev(origins, torch.float32, 2), _dev(dirs, torch.float32, 2), _dev(tmax, torch.float32)
        n = o.shape[0]
        hit = torch.empty(n, dtype=torch.uint8, device="cuda")
        t, sp = torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda")
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        check(lib().snch_scene2_query_ray(self._h, _ptr(o), _ptr(d), _ptr(tm), n, _ptr(hit), _ptr(t), _ptr(sp),
                                          _ptr(idx), _stream(stream)))
        return hit, t, sp, idx

    def query_ray_test(self, origins, dirs, tmax, stream=None):
        """ray_intersect<TestOnly = true> over segments -> hit uint8."""
        torch = _torch()
        o, d, tm = _dev(origins, torch.float32, 2), _dev(dirs, torch.float32, 2), _dev(tmax, torch.float32)
        hit = torch.empty(o.shape[0], dtype=torch.uint8, device="cuda")
        check(lib().snch_scene2_query_ray_test(self._h, _ptr(o), _ptr(d), _ptr(tm), o.shape[0], _ptr(hit),
                                               _stream(stream)))
        return hit

    def sample_in_circle(self, centers, radii, u, stream=None):
        torch = _torch()
        c, r, uu = _dev(centers, torch.float32, 2), _dev(radii, torch.float32), _dev(u, torch.float32)
        n = c.shape[0]
        idx, pdf = torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda")
        check(lib().snch_scene2_sample_in_circle(self._h, _ptr(c), _ptr(r), _ptr(uu), n, _ptr(idx), _ptr(pdf),
                                                 _stream(stream)))
        return idx, pdf

    def sample_on_object(self, index, u, stream=None):
        torch = _torch()
        i, uu = _dev(index, torch.int32), _dev(u, torch.float32)
        n = i.shape[0]
        out = torch.empty((n, 2), dtype=torch.float32, device="cuda")
        check(lib().snch_scene2_sample_on_object(self._h, _ptr(i), _ptr(uu), n, _ptr(out), _stream(stream)))
        return out
