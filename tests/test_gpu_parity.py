"""CUDA path (through the C ABI) against the reference's own outputs and the oracle.

Bars:
  * topology, Morton codes, sorted order, nodes, AABBs: bit-exact;
  * nearest / ray / sphere-sample / sample-on-object: bit-exact indices and floats
    (same IEEE operation sequence, no contraction, correctly rounded / and sqrt);
  * normal cones: CUDA's acosf/sinf/cosf vs libm: |diff| <= CONE_TOL (radians /
    unit-axis components) on every node whose cone is defined in the reference;
  * silhouette distances: bit-exact except where a cone test on the cull
    boundary flips; such queries must still agree within SIL_RTOL relative and
    be rarer than SIL_MAX_FLIP_FRACTION.
"""
import ctypes as C
import numpy as np
import pytest

from conftest import d1_tainted, golden_names, load_golden

pytestmark = pytest.mark.gpu

CONE_TOL = 2e-5
FP64_ABS_TOL = 2.5e-7  # two float32 ulps at unit coordinates
SIL_RTOL = 1e-6
SIL_MAX_FLIP_FRACTION = 1e-3


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def seg_dist64(p, a, b):
    """FP64 distance from points p (n, 3) to segments a-b (n, 3)."""
    p, a, b = (np.asarray(x, np.float64) for x in (p, a, b))
    u, v = b - a, p - a
    t = np.clip(np.einsum("ij,ij->i", u, v) / np.maximum(np.einsum("ij,ij->i", u, u), 1e-300), 0.0, 1.0)
    return np.linalg.norm(p - (a + u * t[:, None]), axis=1)


def check_edge_ids(got, exp, dist, pts, verts, edge_verts, max_frac=1e-4):
    """Silhouette edge ids of two searches with bit-identical distances: equal, or
    both edges at the returned distance (an exact tie that falls on a rounding
    boundary of a box test, where the reference's own choice depends on its visit
    order), in at most max_frac of the queries (and at most 3 below 30,000)."""
    got, exp = np.asarray(got), np.asarray(exp)
    bad = np.nonzero(got != exp)[0]
    assert len(bad) <= max(3, max_frac * len(got)), f"{len(bad)} edge ids differ"
    if len(bad) == 0:
        return 0
    assert np.all(got[bad] >= 0) and np.all(exp[bad] >= 0), "only one search found a silhouette edge"
    d = np.asarray(dist, np.float64)[bad]
    for e in (got[bad], exp[bad]):
        ev = np.asarray(edge_verts)[e]
        de = seg_dist64(np.asarray(pts)[bad], verts[ev[:, 1]], verts[ev[:, 2]])
        assert np.all(np.abs(de - d) <= 1e-6 * np.maximum(d, 1e-3)), "differing edge ids are not a distance tie"
    return len(bad)


def tri_dist64(p, a, b, c):
    """FP64 distance from points p (n, 3) to triangles a, b, c (n, 3 each):
    the closest point by its Voronoi region (Ericson, Real-Time Collision
    Detection 5.1.5), vectorised."""
    p, a, b, c = (np.asarray(x, np.float64) for x in (p, a, b, c))
    dot = lambda x, y: np.einsum("ij,ij->i", x, y)
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = dot(ab, ap), dot(ac, ap)
    bp = p - b
    d3, d4 = dot(ab, bp), dot(ac, bp)
    cp = p - c
    d5, d6 = dot(ab, cp), dot(ac, cp)
    va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
    den = np.where(va + vb + vc == 0, 1.0, va + vb + vc)
    q = a + ab * (vb / den)[:, None] + ac * (vc / den)[:, None]  # face
    w = np.clip(d2 / np.where(d2 - d6 == 0, 1, d2 - d6), 0, 1)
    q = np.where(((vb <= 0) & (d2 >= 0) & (d6 <= 0))[:, None], a + ac * w[:, None], q)  # edge ac
    w = np.clip((d4 - d3) / np.where((d4 - d3) + (d5 - d6) == 0, 1, (d4 - d3) + (d5 - d6)), 0, 1)
    q = np.where(((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0))[:, None], b + (c - b) * w[:, None], q)  # edge bc
    w = np.clip(d1 / np.where(d1 - d3 == 0, 1, d1 - d3), 0, 1)
    q = np.where(((vc <= 0) & (d1 >= 0) & (d3 <= 0))[:, None], a + ab * w[:, None], q)  # edge ab
    q = np.where(((d6 >= 0) & (d5 <= d6))[:, None], c, q)
    q = np.where(((d3 >= 0) & (d4 <= d3))[:, None], b, q)
    q = np.where(((d1 <= 0) & (d2 <= 0))[:, None], a, q)
    return np.linalg.norm(p - q, axis=1)


def check_tri_ids(got, exp, dist, pts, verts, tris, max_frac=1e-4):
    """Nearest-triangle indices of two searches with bit-identical distances:
    equal, or both triangles at the returned distance (the tie case of
    check_edge_ids), in at most max_frac of the queries."""
    got, exp = np.asarray(got).view(np.int32), np.asarray(exp).view(np.int32)
    bad = np.nonzero(got != exp)[0]
    assert len(bad) <= max(3, max_frac * len(got)), f"{len(bad)} triangle indices differ"
    if len(bad) == 0:
        return 0
    d = np.asarray(dist, np.float64)[bad]
    for t in (got[bad], exp[bad]):
        tv = np.asarray(tris)[t]
        dt = tri_dist64(np.asarray(pts)[bad], verts[tv[:, 0]], verts[tv[:, 1]], verts[tv[:, 2]])
        assert np.all(np.abs(dt - d) <= 1e-6 * np.maximum(d, 1e-3)), "differing triangles are not a distance tie"
    return len(bad)


def built_scene(snch, verts, tris):
    s = snch.Scene(verts, tris)
    s.compute_silhouettes()
    s.build_bvh()
    return s


def check_cones(gpu_cones, ref_cones, nodes, d1):
    taint = d1_tainted(nodes, d1)
    valid = ref_cones[:, 3] >= 0
    np.testing.assert_array_equal((gpu_cones[:, 3] >= 0)[~taint], valid[~taint])
    ok = valid & ~taint
    g64, r64 = gpu_cones[ok].astype(np.float64), ref_cones[ok].astype(np.float64)
    both_nan = np.isnan(g64) & np.isnan(r64)  # degenerate triangles: 0/0 axes in both
    diff = np.where(both_nan, 0.0, np.abs(g64 - r64))
    diff[np.isnan(diff)] = np.inf
    rad = np.abs(ref_cones[ok, 4]).astype(np.float64)
    assert diff[:, :4].max(initial=0) <= CONE_TOL, diff[:, :4].max()
    assert np.all(diff[:, 4] <= CONE_TOL * np.maximum(rad, 1.0))
    assert np.all(gpu_cones[taint, 3] >= 0)


def check_silhouette(gpu, ref):
    same = bits(gpu) == bits(ref)
    both_inf = np.isinf(gpu) & np.isinf(ref)
    flips = ~(same | both_inf)
    assert flips.mean() <= SIL_MAX_FLIP_FRACTION, (flips.sum(), len(gpu))
    fin = flips & np.isfinite(gpu) & np.isfinite(ref)
    if fin.any():
        rel = np.abs(gpu[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-30)
        assert rel.max() <= SIL_RTOL or flips.sum() <= max(1, int(SIL_MAX_FLIP_FRACTION * len(gpu)))


@pytest.mark.parametrize("name", golden_names())
def test_build_matches_reference(snch, oracle_mod, name):
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    te, to, ev = s.export_topology()
    np.testing.assert_array_equal(te, g["ref_tri_edges"])
    np.testing.assert_array_equal(to, g["ref_tri_owned"])
    np.testing.assert_array_equal(ev, g["ref_edge_verts"])
    tr = s.export_tree()
    n = len(g["tris"])
    ref_sorted = g["ref_nodes"][n - 1:, 3]
    np.testing.assert_array_equal(tr["sorted_idx"], ref_sorted)
    np.testing.assert_array_equal(tr["morton"], g["ref_morton"][ref_sorted])
    np.testing.assert_array_equal(tr["nodes"], g["ref_nodes"])
    np.testing.assert_array_equal(bits(tr["aabbs"]), bits(g["ref_aabbs"]))
    orc = oracle_mod.Tree(g["verts"], g["tris"])
    check_cones(tr["cones"], g["ref_cones"], orc.nodes, orc.d1)
    assert s.device_status() == 0


@pytest.mark.parametrize("name", golden_names())
def test_queries_match_reference(snch, name):
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    if len(g["ref_near_idx"]):
        idx, dist = s.query_nearest(g["near_pts"])
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), g["ref_near_idx"])
        np.testing.assert_array_equal(bits(dist.cpu().numpy()), bits(g["ref_near_dist"]))
        sd, _ = s.query_silhouette(g["sil_pts"], g["sil_flip"])
        check_silhouette(sd.cpu().numpy(), g["ref_sil_dist"])
    hit, t, uv, ri = s.query_ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
    np.testing.assert_array_equal(hit.cpu().numpy(), g["ref_ray_hit"])
    # ray_intersect<TestOnly = true>: the same hit flags, from the first accepted hit
    np.testing.assert_array_equal(s.query_ray_test(g["ray_o"], g["ray_d"], g["ray_tmax"]).cpu().numpy(),
                                  g["ref_ray_hit"])
    np.testing.assert_array_equal(bits(t.cpu().numpy()), bits(g["ref_ray_t"]))
    np.testing.assert_array_equal(bits(uv.cpu().numpy()), bits(g["ref_ray_uv"]))
    np.testing.assert_array_equal(ri.cpu().numpy().view(np.uint32), g["ref_ray_idx"])
    si, sp = s.sample_in_sphere(g["smp_c"], g["smp_r"], g["smp_u"])
    np.testing.assert_array_equal(si.cpu().numpy(), g["ref_smp_idx"])
    np.testing.assert_array_equal(bits(sp.cpu().numpy()), bits(g["ref_smp_pdf"]))
    pts = s.sample_on_object(g["obj_idx"], g["obj_u"], g["obj_v"])
    np.testing.assert_array_equal(bits(pts.cpu().numpy()), bits(g["ref_obj_pts"]))
    assert s.device_status() == 0


def test_config1_workload_against_oracle(snch, oracle_mod):
    """Config 1: level-5 noisy icosphere, 1M nearest queries uniform in the AABB x 1.2."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = meshes.box_queries(v, 1_000_000, 1.2, seed=1)
    s = built_scene(snch, v, f)
    idx, dist = s.query_nearest(pts)
    idx, dist = idx.cpu().numpy().view(np.uint32), dist.cpu().numpy()
    orc = oracle_mod.Tree(v, f)
    oi, od = orc.nearest(pts)
    np.testing.assert_array_equal(bits(dist), bits(od))
    check_tri_ids(idx, oi, od, pts, v, f)
    # FP64 brute force on a subset: the reference algorithm's FP32 error. The
    # chosen triangle is compared through its FP64 distance, because exact ties
    # (a shared vertex or edge is the nearest feature) are common and brute
    # force keeps a different tied triangle than the reference's visit order.
    sub = np.arange(0, len(pts), 122)[:8192]
    bi, bd = oracle_mod.brute_nearest_f64(v, f, pts[sub])
    err = np.abs(dist[sub].astype(np.float64) - bd)
    assert err.max() <= FP64_ABS_TOL, err.max()
    for k in np.nonzero(idx[sub] != bi)[0][:256]:
        _, dk = oracle_mod.brute_nearest_f64(v, f[idx[sub][k]][None], pts[sub][k][None])
        assert abs(dk[0] - bd[k]) <= FP64_ABS_TOL
    assert s.device_status() == 0


def test_host_forms_equal_device_forms(snch):
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(4, 1.0, 0.01, seed=2)
    q = meshes.wost_queries(300_000, 300_000, 300_000, 100_000, seed=4)
    s = built_scene(snch, v * 0.4 + 0.5, f)
    i1, d1 = s.query_nearest(q["near_pts"])
    i2, d2 = s.query_nearest_host(q["near_pts"])
    np.testing.assert_array_equal(i1.cpu().numpy().view(np.uint32), i2)
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d2))
    s1, e1 = s.query_silhouette(q["sil_pts"], q["sil_flip"])
    s2, e2 = s.query_silhouette_host(q["sil_pts"], q["sil_flip"])
    np.testing.assert_array_equal(bits(s1.cpu().numpy()), bits(s2))
    np.testing.assert_array_equal(e1.cpu().numpy(), e2)
    r1 = s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])
    r2 = s.query_ray_host(q["ray_o"], q["ray_d"], q["ray_tmax"])
    np.testing.assert_array_equal(r1[0].cpu().numpy(), r2[0])
    np.testing.assert_array_equal(bits(r1[1].cpu().numpy()), bits(r2[1]))
    np.testing.assert_array_equal(bits(r1[2].cpu().numpy()), bits(r2[2]))
    np.testing.assert_array_equal(r1[3].cpu().numpy().view(np.uint32), r2[3])
    p1 = s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"])
    p2 = s.sample_in_sphere_host(q["smp_c"], q["smp_r"], q["smp_u"])
    np.testing.assert_array_equal(p1[0].cpu().numpy(), p2[0])
    np.testing.assert_array_equal(bits(p1[1].cpu().numpy()), bits(p2[1]))


@pytest.mark.parametrize("name", golden_names())
def test_persistent_rays_match_reference(snch, name):
    """Lane-refill ray kernels (closest hit and occlusion) give the reference's answers."""
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    s.set_option(snch.OPT_PERSISTENT_RAY, 1)
    hit, t, uv, ri = s.query_ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
    np.testing.assert_array_equal(hit.cpu().numpy(), g["ref_ray_hit"])
    np.testing.assert_array_equal(bits(t.cpu().numpy()), bits(g["ref_ray_t"]))
    np.testing.assert_array_equal(bits(uv.cpu().numpy()), bits(g["ref_ray_uv"]))
    np.testing.assert_array_equal(ri.cpu().numpy().view(np.uint32), g["ref_ray_idx"])
    np.testing.assert_array_equal(s.query_ray_test(g["ray_o"], g["ray_d"], g["ray_tmax"]).cpu().numpy(),
                                  g["ref_ray_hit"])
    assert s.device_status() == 0


def test_persistent_rays_full_scene(snch):
    """Lane-refill rays equal one-thread-per-ray rays bit for bit on 2M rays of the
    two-million-triangle scene (tmax log-uniform over three decades)."""
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    q = meshes.wost_queries(1, 1, 2_000_000, 1, seed=21)
    s = built_scene(snch, sc.verts, sc.faces)
    a = [x.cpu().numpy() for x in s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])]
    at = s.query_ray_test(q["ray_o"], q["ray_d"], q["ray_tmax"]).cpu().numpy()
    s.set_option(snch.OPT_PERSISTENT_RAY, 1)
    b = [x.cpu().numpy() for x in s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])]
    bt = s.query_ray_test(q["ray_o"], q["ray_d"], q["ray_tmax"]).cpu().numpy()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    np.testing.assert_array_equal(at, bt)
    np.testing.assert_array_equal(bt, a[0])
    assert s.device_status() == 0


def test_query_before_build_raises(snch):
    import torch
    s = snch.Scene(np.eye(3, dtype=np.float32), np.array([[0, 1, 2]], np.int32))
    with pytest.raises(snch.SnchError, match="BVH is not built yet."):
        s.query_nearest(torch.zeros((4, 3), device="cuda"))
    with pytest.raises(snch.SnchError, match="BVH is not built yet."):
        s.get_bvh_device_ptr()


def test_empty_and_single_triangle(snch):
    empty = snch.Scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    empty.build_bvh()
    idx, dist = empty.query_nearest(np.zeros((5, 3), np.float32))
    assert np.all(idx.cpu().numpy() == -1) and np.all(np.isinf(dist.cpu().numpy()))
    hit, t, _, ri = empty.query_ray(np.zeros((2, 3), np.float32), np.ones((2, 3), np.float32), np.ones(2, np.float32))
    assert not hit.cpu().numpy().any()
    assert not empty.query_ray_test(np.zeros((2, 3), np.float32), np.ones((2, 3), np.float32),
                                    np.ones(2, np.float32)).cpu().numpy().any()
    one = built_scene(snch, np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32))
    idx, dist = one.query_nearest(np.array([[0.2, 0.2, 1.0], [2.0, 0.0, 0.0]], np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), [0, 0])
    np.testing.assert_allclose(dist.cpu().numpy(), [1.0, 1.0], rtol=1e-6)
    view = one.get_bvh_device_ptr()
    assert view.num_nodes == 1 and view.num_objects == 1


def test_device_create_validates_indices(snch):
    import torch
    v = torch.zeros((3, 3), device="cuda")
    bad = torch.tensor([[0, 1, 7]], dtype=torch.int32, device="cuda")
    with pytest.raises(snch.SnchError, match="out of range"):
        snch.Scene(v, bad)
    ok = snch.Scene(v + torch.eye(3, device="cuda"), torch.tensor([[0, 1, 2]], dtype=torch.int32, device="cuda"))
    ok.build_bvh()
    assert ok.info() == (3, 1, 3)


def run_all(s, q, mode):
    s.set_traversal(mode)
    i, d = s.query_nearest(q["near_pts"])
    sd, se = s.query_silhouette(q["sil_pts"], q["sil_flip"])
    return [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]


@pytest.mark.parametrize("name", golden_names())
def test_near_first_equals_reference_order_golden(snch, oracle_mod, name):
    """The near-first traversals return the reference-order results bit for bit,
    tie winners included (golden inputs hold vertex / edge / face-centre probes)."""
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    orc = oracle_mod.Tree(g["verts"], g["tris"])
    np.testing.assert_array_equal(s.leaf_ranks(), orc.leaf_ranks())
    q = {"near_pts": g["near_pts"], "sil_pts": g["sil_pts"], "sil_flip": g["sil_flip"]}
    a = run_all(s, q, snch.TRAVERSAL_REFERENCE_ORDER)
    b = run_all(s, q, snch.TRAVERSAL_NEAR_FIRST)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    if len(g["ref_near_idx"]):
        np.testing.assert_array_equal(b[0].view(np.uint32), g["ref_near_idx"])
        np.testing.assert_array_equal(b[1], bits(g["ref_near_dist"]))


def test_near_first_equals_reference_order_config1(snch):
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = meshes.box_queries(v, 1_000_000, 1.2, seed=1)
    # add exact-tie probes: every vertex and every edge midpoint
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    mids = (0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])).astype(np.float32)
    pts = np.concatenate([pts, v, mids]).astype(np.float32)
    q = {"near_pts": pts, "sil_pts": pts, "sil_flip": (np.arange(len(pts)) % 2).astype(np.uint8)}
    s = built_scene(snch, v, f)
    a = run_all(s, q, snch.TRAVERSAL_REFERENCE_ORDER)
    b = run_all(s, q, snch.TRAVERSAL_NEAR_FIRST)
    for x, y in zip(a[1:3], b[1:3]):
        np.testing.assert_array_equal(x, y)
    check_tri_ids(b[0], a[0], a[1].view(np.float32), pts, v, f)
    check_edge_ids(b[3], a[3], a[2].view(np.float32), pts, v, s.export_topology()[2])
    assert s.device_status() == 0


def test_query_order_does_not_change_results(snch):
    """Morton-sorted batches (default for >= 65536 queries) equal input-order batches."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    q = meshes.wost_queries(400_000, 200_000, 400_000, 200_000, seed=9)
    for k in ("near_pts", "sil_pts", "ray_o", "smp_c"):
        q[k] = (q[k] * 2.4 - 1.2).astype(np.float32)
    s = built_scene(snch, v, f)

    def everything():
        i, d = s.query_nearest(q["near_pts"])
        sd, se = s.query_silhouette(q["sil_pts"], q["sil_flip"])
        h, t, uv, ri = s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])
        si, sp = s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"])
        return [x.cpu().numpy() for x in (i, d, sd, se, h, t, uv, ri, si, sp)]

    s.set_option(snch.OPT_QUERY_ORDER, 0)
    a = everything()
    s.set_option(snch.OPT_QUERY_ORDER, 1)
    b = everything()
    for k, (x, y) in enumerate(zip(a, b)):
        if k not in (0, 3):  # nearest index / silhouette edge id: ordered batches run as warp packets
            np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    check_tri_ids(b[0], a[0], a[1], q["near_pts"], v, f)
    check_edge_ids(b[3], a[3], a[2], q["sil_pts"], v, s.export_topology()[2])
    assert s.device_status() == 0


@pytest.mark.parametrize("n", [1, 31, 33, 1000, 300_000])
def test_persistent_equals_one_thread_per_query(snch, n):
    """Lane-refill persistent kernels (default) equal one-thread-per-query kernels,
    plain and seeded, at batch sizes below, at and above one warp and one chunk."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    rng = np.random.default_rng(n)
    pts = meshes.box_queries(v, n, 1.2, seed=n + 3)
    if n >= 1000:  # exact-tie probes: vertices and edge midpoints
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]]])[: n // 4]
        mids = (0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])).astype(np.float32)
        pts[: len(mids)] = mids
        pts[len(mids): len(mids) + min(len(v), n // 4)] = v[: n // 4]
    flip = (rng.random(n) < 0.5).astype(np.uint8)
    s = built_scene(snch, v, f)

    def run():
        i, d = s.query_nearest(pts)
        sd, se = s.query_silhouette(pts, flip)
        r = np.where(rng.random(n) < 0.5, 0.01, 1.0).astype(np.float32)
        i2, d2 = s.query_nearest_seeded(pts, r)
        sd2, se2 = s.query_silhouette_seeded(pts, r, flip)
        return [x.cpu().numpy() for x in (i, d, sd, se, i2, d2, sd2, se2)]

    state = rng.bit_generator.state
    s.set_option(snch.OPT_PERSISTENT, 0)
    a = run()
    rng.bit_generator.state = state
    s.set_option(snch.OPT_PERSISTENT, 1)
    b = run()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0


def test_fast_cone_test_agrees_with_exact(snch):
    """The silhouette traversal's fast normal-cone test decides only where its
    error bound allows and then agrees with the reference-arithmetic test: 4M
    random cases, half of them within 1e-3 rad of the decision boundary."""
    import torch
    counts = torch.zeros(3, dtype=torch.int64, device="cuda")
    for seed in (1, 2):
        snch.check(snch.lib().snch_selfcheck_cone_filter(2_000_000, seed, C.c_void_p(counts.data_ptr()),
                                                         C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    agree, disagree, undecided = (int(x) for x in counts.cpu())
    assert agree + disagree + undecided == 4_000_000
    assert disagree == 0
    assert agree >= 0.5 * 4_000_000, (agree, undecided)


@pytest.mark.parametrize("cap", [1, 7, 128])
def test_tail_cap_does_not_change_results(snch, cap):
    """Capped first pass + seeded second pass (SNCH_OPT_TAIL_CAP) equals the
    uncapped searches, plain and seeded, on random points and exact-tie probes."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    rng = np.random.default_rng(cap)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]]])
    mids = (0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])).astype(np.float32)
    pts = np.concatenate([meshes.box_queries(v, 200_000, 1.2, seed=cap), v, mids]).astype(np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    radius = np.where(rng.random(len(pts)) < 0.5, 0.02, 0.5).astype(np.float32)
    s = built_scene(snch, v, f)

    def run():
        i, d = s.query_nearest(pts)
        sd, se = s.query_silhouette(pts, flip)
        i2, d2 = s.query_nearest_seeded(pts, radius)
        sd2, se2 = s.query_silhouette_seeded(pts, radius, flip)
        return [x.cpu().numpy() for x in (i, d, sd, se, i2, d2, sd2, se2)]

    s.set_option(snch.OPT_TAIL_CAP, 0)
    a = run()
    s.set_option(snch.OPT_TAIL_CAP, cap)
    b = run()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0
