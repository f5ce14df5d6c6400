"""The header-only device face (include/snch_device.cuh): a caller's own kernels
(tests/cxx/device_shim_kernels.cu, compiled here by nvcc with its default flags,
FMA contraction on) call snch::query_device / sample_object_in_sphere /
sample_on_object per thread in the reference's call forms (query.cuh:82-169,
239-318, 326-423; sample.cuh:10-91), over the view snch_get_traversal_view
returns. Every output must equal the library's own one-thread-per-query kernels
bit for bit: indices, distances, edge ids, hit flags, hit parameters, (u, v),
pdfs and sampled points."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import built_scene
from test_gpu_wide import tie_probes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "device_shim_kernels.cu")
OUT = os.path.join(ROOT, "tests", "cxx", "_build", "libdevice_shim.so")


@pytest.fixture(scope="module")
def shim():
    import torch
    assert torch.cuda.is_available()
    import snch_lbvh_gb300
    from snch_lbvh_gb300 import build
    snch_lbvh_gb300.lib()
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = [build.nvcc(), "-shared", "-Xcompiler", "-fPIC", *build.ARCH, "-O3", "-std=c++17",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    L = C.CDLL(OUT)
    P, I = C.c_void_p, C.c_int
    L.shim_nearest.argtypes = [P, P, I, P, P]
    L.shim_silhouette.argtypes = [P, P, P, I, P, P]
    L.shim_ray.argtypes = [P, P, P, P, I, P, P, P, P, P]
    L.shim_sample.argtypes = [P, P, P, P, P, P, I, P, P, P]
    return L


def _p(t):
    return C.c_void_p(t.data_ptr())


def compare(snch, L, s, pts, flip, rays, spheres):
    import torch
    s.set_option(snch.OPT_PACKET, 0)  # the library's one-thread-per-query kernels
    view = s.get_traversal_view()
    vp = C.byref(view)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    p, fl = cu(pts), cu(flip)
    n = len(pts)
    si, sd = torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, device="cuda")
    assert L.shim_nearest(vp, _p(p), n, _p(si), _p(sd)) == 0
    li, ld = s.query_nearest(p)
    np.testing.assert_array_equal(si.cpu().numpy(), li.cpu().numpy())
    np.testing.assert_array_equal(sd.cpu().numpy().view(np.uint32), ld.cpu().numpy().view(np.uint32))
    ssd, sse = torch.empty(n, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")
    assert L.shim_silhouette(vp, _p(p), _p(fl), n, _p(ssd), _p(sse)) == 0
    lsd, lse = s.query_silhouette(p, fl)
    np.testing.assert_array_equal(ssd.cpu().numpy().view(np.uint32), lsd.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(sse.cpu().numpy(), lse.cpu().numpy())

    o, d, tmax = (cu(x) for x in rays)
    m = len(rays[0])
    rh, rt = torch.empty(m, dtype=torch.uint8, device="cuda"), torch.empty(m, device="cuda")
    ruv, ri = torch.empty((m, 2), device="cuda"), torch.empty(m, dtype=torch.int32, device="cuda")
    ra = torch.empty(m, dtype=torch.uint8, device="cuda")
    assert L.shim_ray(vp, _p(o), _p(d), _p(tmax), m, _p(rh), _p(rt), _p(ruv), _p(ri), _p(ra)) == 0
    lh, lt, luv, lri = s.query_ray(o, d, tmax)
    np.testing.assert_array_equal(rh.cpu().numpy(), lh.cpu().numpy())
    np.testing.assert_array_equal(rt.cpu().numpy().view(np.uint32), lt.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(ruv.cpu().numpy().view(np.uint32), luv.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(ri.cpu().numpy(), lri.cpu().numpy())
    np.testing.assert_array_equal(ra.cpu().numpy(), s.query_ray_test(o, d, tmax).cpu().numpy())

    c, r, u, u2, v2 = (cu(x) for x in spheres)
    k = len(spheres[0])
    xi, xp = torch.empty(k, dtype=torch.int32, device="cuda"), torch.empty(k, device="cuda")
    xpt = torch.empty((k, 3), device="cuda")
    assert L.shim_sample(vp, _p(c), _p(r), _p(u), _p(u2), _p(v2), k, _p(xi), _p(xp), _p(xpt)) == 0
    li2, lp2 = s.sample_in_sphere(c, r, u)
    np.testing.assert_array_equal(xi.cpu().numpy(), li2.cpu().numpy())
    np.testing.assert_array_equal(xp.cpu().numpy().view(np.uint32), lp2.cpu().numpy().view(np.uint32))
    ok = li2 >= 0  # the library's sample_on_object rejects the -1 of a draw that found nothing
    lpt = s.sample_on_object(li2[ok], u2[ok], v2[ok])
    got = xpt.cpu().numpy()
    np.testing.assert_array_equal(got[ok.cpu().numpy()].view(np.uint32), lpt.cpu().numpy().view(np.uint32))
    assert np.isnan(got[~ok.cpu().numpy()]).all()  # the shim's answer for an index out of range
    assert s.device_status() == 0
    s.set_option(snch.OPT_PACKET, 2)


def workload(v, f, n, seed, scale=1.2):
    """Points in the mesh box (with vertex / edge-midpoint / centroid tie probes),
    rays through it and sphere draws, half with flip = true."""
    rng = np.random.default_rng(seed)
    lo, hi = v.min(0), v.max(0)
    ctr, half = (lo + hi) / 2, (hi - lo) / 2 * scale + 1e-3
    box = lambda k: (ctr + half * (2 * rng.random((k, 3)) - 1)).astype(np.float32)
    pts = np.concatenate([box(n), tie_probes(v, f)]).astype(np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = np.exp(rng.uniform(np.log(1e-3), np.log(4 * half.max()), n)).astype(np.float32)
    rays = (box(n), d.astype(np.float32), tmax)
    rad = np.exp(rng.uniform(np.log(1e-3), np.log(half.max()), n)).astype(np.float32)
    spheres = (box(n), rad, rng.random(n, dtype=np.float32), rng.random(n, dtype=np.float32),
               rng.random(n, dtype=np.float32))
    return pts, flip, rays, spheres


@pytest.mark.parametrize("name", golden_names())
def test_device_shim_equals_library_golden(shim, name):
    import snch_lbvh_gb300 as snch
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    compare(snch, shim, s, *workload(g["verts"], g["tris"], 20_000, seed=3))


def test_device_shim_equals_library_config1(shim):
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    compare(snch, shim, built_scene(snch, v, f), *workload(v, f, 500_000, seed=4))


def test_device_shim_equals_library_wost_scene(shim):
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    s = built_scene(snch, sc.verts, sc.faces)
    rng = np.random.default_rng(9)
    pts = rng.random((500_000, 3), dtype=np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    q = meshes.wost_queries(1, 1, 500_000, 200_000, seed=8)
    spheres = (q["smp_c"], q["smp_r"], q["smp_u"], rng.random(200_000, dtype=np.float32),
               rng.random(200_000, dtype=np.float32))
    compare(snch, shim, s, pts, flip, (q["ray_o"], q["ray_d"], q["ray_tmax"]), spheres)


def test_traversal_view_rejects_batched_and_unbuilt(shim):
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(2, 1.0, 0.01, seed=1)
    s = snch.Scene(v, f)
    with pytest.raises(snch.SnchError):
        s.get_traversal_view()
    b = snch.BatchedScene([(v, f), (v, f)])
    b.compute_silhouettes()
    b.build_bvh()
    with pytest.raises(snch.SnchError):
        b.get_traversal_view()
