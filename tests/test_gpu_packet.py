"""Warp-packet searches (SNCH_OPT_PACKET): a warp's 32 queries walk one shared
traversal, each lane with its own tests and answer. Results equal the per-lane
near-first searches bit for bit -- indices, distances, silhouette edge ids,
exact-tie probes included -- on the golden meshes, the config-1 icosphere, the
2M-triangle scene (ordered and unordered batches), batched scenes with warps
that straddle meshes, and seeded searches."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import bits, built_scene, check_edge_ids, check_tri_ids
from test_gpu_wide import answers, tie_probes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def check_packet(snch, s, pts, flip, verts, tris):
    s.set_option(snch.OPT_PACKET, 0)
    base = answers(s, pts, flip)
    s.set_option(snch.OPT_PACKET, 1)
    got = answers(s, pts, flip)
    s.set_option(snch.OPT_PACKET, 2)
    for name, x, y in zip(("nearest dist", "silhouette dist"), base[1:3], got[1:3]):
        np.testing.assert_array_equal(y, x, err_msg=name)
    check_tri_ids(got[0], base[0], base[1].view(np.float32), pts, verts, tris)
    check_edge_ids(got[3], base[3], base[2].view(np.float32), pts, verts, s.export_topology()[2])
    assert s.device_status() == 0


@pytest.mark.parametrize("name", golden_names())
def test_packet_equals_per_lane_golden(snch, name):
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    pts = np.concatenate([g["near_pts"], g["sil_pts"], tie_probes(g["verts"], g["tris"])]).astype(np.float32)
    check_packet(snch, s, pts, (np.arange(len(pts)) % 2).astype(np.uint8), g["verts"], g["tris"])


def test_packet_equals_per_lane_config1(snch):
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = np.concatenate([meshes.box_queries(v, 1_000_000, 1.2, seed=1), tie_probes(v, f)])
    flip = (np.random.default_rng(2).random(len(pts)) < 0.5).astype(np.uint8)
    check_packet(snch, built_scene(snch, v, f), pts, flip, v, f)


@pytest.mark.parametrize("ordered", [1, 0])
def test_packet_equals_per_lane_wost_scene(snch, ordered):
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    s = built_scene(snch, sc.verts, sc.faces)
    s.set_option(snch.OPT_QUERY_ORDER, ordered)  # unordered: incoherent packets, same answers
    rng = np.random.default_rng(6)
    pts = rng.random((1_000_000 if ordered else 200_000, 3), dtype=np.float32)
    check_packet(snch, s, pts, (rng.random(len(pts)) < 0.5).astype(np.uint8), sc.verts, sc.faces)


def test_packet_batched_and_seeded(snch):
    from test_gpu_batched import mixed_meshes
    from test_gpu_seeded import radii_mix
    rng = np.random.default_rng(13)
    ms = mixed_meshes(rng, 40)
    ms.insert(3, (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32)))
    b = snch.BatchedScene(ms)
    b.compute_silhouettes()
    b.build_bvh()
    mesh, pts = [], []
    for m, (v, f) in enumerate(ms):
        k = int(rng.integers(5, 3000))  # uneven counts: warps straddle meshes
        lo, hi = v.min(0), v.max(0)
        pts.append((lo + (hi - lo + 1e-3) * (1.4 * rng.random((k, 3)) - 0.2)).astype(np.float32))
        mesh.append(np.full(k, m, np.int32))
    mesh, pts = np.concatenate(mesh), np.concatenate(pts)
    perm = rng.permutation(len(pts))
    mesh, pts = mesh[perm], pts[perm]
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)

    def run():
        i, d = b.query_nearest_batch(mesh, pts)
        sd, se = b.query_silhouette_batch(mesh, pts, flip)
        return [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]

    b.set_option(snch.OPT_PACKET, 0)
    base = run()
    b.set_option(snch.OPT_PACKET, 1)
    got = run()
    for x, y in zip(base[1:3], got[1:3]):
        np.testing.assert_array_equal(y, x)
    # indices per mesh: equal, or an exact tie (the duplicated-triangle golden mesh has them)
    for m, (v, f) in enumerate(ms):
        sel = np.nonzero(mesh == m)[0]
        if len(f) and len(sel):
            s1 = built_scene(snch, v, f)
            check_tri_ids(got[0][sel], base[0][sel], base[1][sel].view(np.float32), pts[sel], v, f, max_frac=1e-2)
            check_edge_ids(got[3][sel], base[3][sel], base[2][sel].view(np.float32), pts[sel], v,
                           s1.export_topology()[2], max_frac=1e-2)
    assert b.device_status() == 0

    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=2, n_meshes=8, torus_nu=60, torus_nv=30, ico_level=4)
    s = built_scene(snch, sc.verts, sc.faces)
    q = rng.random((300_000, 3), dtype=np.float32)
    fl = (rng.random(len(q)) < 0.5).astype(np.uint8)
    i0, d0 = s.query_nearest(q)
    sd0, se0 = s.query_silhouette(q, fl)
    s.set_option(snch.OPT_PACKET, 1)
    r, _ = radii_mix(d0.cpu().numpy(), rng)
    i1, d1 = s.query_nearest_seeded(q, r)
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d0.cpu().numpy()))
    check_tri_ids(i1.cpu().numpy(), i0.cpu().numpy(), d0.cpu().numpy(), q, sc.verts, sc.faces)
    rs, _ = radii_mix(sd0.cpu().numpy(), rng)
    sd1, se1 = s.query_silhouette_seeded(q, rs, fl)
    np.testing.assert_array_equal(bits(sd1.cpu().numpy()), bits(sd0.cpu().numpy()))
    check_edge_ids(se1.cpu().numpy(), se0.cpu().numpy(), sd0.cpu().numpy(), q, sc.verts, s.export_topology()[2])
    assert s.device_status() == 0


@pytest.mark.parametrize("n", [1, 31, 32, 33, 1025, 2 * 32 * 32 + 7, 70_001])
def test_pooled_persistent_kernels_at_small_sizes(snch, n):
    """The persistent packet searches and the pooled rays forced on at any size
    (SNCH_OPT_PACKET_PERSISTENT_MIN = 1): batches smaller than one pool chunk, a
    partly filled last packet and last chunk give the per-lane searches'
    answers (nearest, silhouette, closest hit, occlusion) on the config-1 sphere,
    and every warp stops (no work-timeout status)."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    s = built_scene(snch, v, f)
    rng = np.random.default_rng(n)
    pts = meshes.box_queries(v, n, 1.2, seed=n)
    flip = (rng.random(n) < 0.5).astype(np.uint8)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = np.full(n, 3.0, np.float32)

    def run():
        i, nd = s.query_nearest(pts)
        sd, se = s.query_silhouette(pts, flip)
        h, t, uv, ri = s.query_ray(pts, d, tmax)
        occ = s.query_ray_test(pts, d, tmax)
        return [x.cpu().numpy() for x in (i, nd, sd, se, h, t, uv, ri, occ)]

    s.set_option(snch.OPT_PACKET, 0)
    base = run()
    s.set_option(snch.OPT_PACKET, 1)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1)
    got = run()
    assert s.device_status() == 0
    for k in (1, 2, 4, 5, 6, 7, 8):  # distances, ray hit / t / uv / triangle, occlusion
        np.testing.assert_array_equal(got[k].view(np.uint8), base[k].view(np.uint8))
    check_tri_ids(got[0], base[0], base[1].view(np.float32), pts, v, f)
    check_edge_ids(got[3], base[3], base[2].view(np.float32), pts, v, s.export_topology()[2])
