"""Full-size checks on the two-million-triangle walk-on-stars scene (64 placed
tori and icospheres): the whole build bit-exact against the oracle, queries
against the oracle on a seeded subset, determinism and size-independent
properties of the tree."""
import numpy as np
import pytest

from test_gpu_parity import bits, built_scene, check_cones, check_edge_ids, check_silhouette, check_tri_ids

PERSISTENT_MIN_DEFAULT = 1 << 19  # SNCH_OPT_PACKET_PERSISTENT_MIN's default (include/snch_gb300.h)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(oracle_mod):
    import torch
    assert torch.cuda.is_available()
    import snch_lbvh_gb300
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    s = built_scene(snch_lbvh_gb300, sc.verts, sc.faces)
    orc = oracle_mod.Tree(sc.verts, sc.faces)
    return sc, s, orc


def test_full_build_bit_exact(big):
    sc, s, orc = big
    assert len(sc.faces) == 1_993_600
    te, to, ev = s.export_topology()
    np.testing.assert_array_equal(te, orc.tri_edges)
    np.testing.assert_array_equal(to, orc.tri_owned)
    np.testing.assert_array_equal(ev, orc.edge_verts)
    tr = s.export_tree()
    np.testing.assert_array_equal(tr["sorted_idx"], orc.sorted_idx)
    np.testing.assert_array_equal(tr["morton"], orc.morton[orc.sorted_idx])
    np.testing.assert_array_equal(tr["nodes"], orc.nodes)
    np.testing.assert_array_equal(bits(tr["aabbs"]), bits(orc.aabbs))
    check_cones(tr["cones"], orc.cones, orc.nodes, orc.d1)
    assert s.device_status() == 0


def test_tree_properties(big):
    sc, s, _ = big
    tr = s.export_tree()
    n = len(sc.faces)
    m = tr["morton"]
    assert np.all(m[1:] >= m[:-1]), "Morton codes must come out sorted"
    same = m[1:] == m[:-1]
    assert np.all(tr["sorted_idx"][1:][same] > tr["sorted_idx"][:-1][same]), "sort must be stable"
    assert np.array_equal(np.sort(tr["sorted_idx"]), np.arange(n, dtype=np.uint32))
    nodes = tr["nodes"]
    ni = n - 1
    L, R = nodes[:ni, 1], nodes[:ni, 2]
    assert np.all(nodes[L, 0] == np.arange(ni)) and np.all(nodes[R, 0] == np.arange(ni))
    child_count = np.bincount(np.concatenate([L, R]), minlength=2 * n - 1)
    assert child_count[0] == 0 and np.all(child_count[1:] == 1)
    a = tr["aabbs"]
    for c in (L, R):
        assert np.all(a[:ni, :3] >= a[c, :3]) and np.all(a[:ni, 3:] <= a[c, 3:])


def test_build_is_deterministic(big):
    import snch_lbvh_gb300
    sc, s, _ = big
    s2 = built_scene(snch_lbvh_gb300, sc.verts, sc.faces)
    t1, t2 = s.export_tree(), s2.export_tree()
    for k in t1:
        np.testing.assert_array_equal(bits(t1[k]), bits(t2[k]))


def test_queries_against_oracle_subset(big):
    from snch_lbvh_gb300 import meshes
    sc, s, orc = big
    q = meshes.wost_queries(200_000, 100_000, 200_000, 200_000, seed=11)
    idx, dist = s.query_nearest(q["near_pts"])
    oi, od = orc.nearest(q["near_pts"])
    np.testing.assert_array_equal(bits(dist.cpu().numpy()), bits(od))
    check_tri_ids(idx.cpu().numpy(), oi, od, q["near_pts"], sc.verts, sc.faces)
    sd, _ = s.query_silhouette(q["sil_pts"], q["sil_flip"])
    osd, _ = orc.silhouette(q["sil_pts"], q["sil_flip"])
    check_silhouette(sd.cpu().numpy(), osd)
    hit, t, uv, ri = s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])
    oh, ot, ouv, oi = orc.ray(q["ray_o"], q["ray_d"], q["ray_tmax"])
    np.testing.assert_array_equal(hit.cpu().numpy(), oh)
    np.testing.assert_array_equal(s.query_ray_test(q["ray_o"], q["ray_d"], q["ray_tmax"]).cpu().numpy(), oh)
    np.testing.assert_array_equal(bits(t.cpu().numpy()), bits(ot))
    np.testing.assert_array_equal(ri.cpu().numpy().view(np.uint32), oi)
    si, sp = s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"])
    osi, osp = orc.sample(q["smp_c"], q["smp_r"], q["smp_u"])
    np.testing.assert_array_equal(si.cpu().numpy(), osi)
    np.testing.assert_array_equal(bits(sp.cpu().numpy()), bits(osp))
    assert s.device_status() == 0


def test_near_first_equals_reference_order_full_scene(big):
    """On the 2M-triangle scene: 1M nearest + 250k silhouette queries, both orders."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    from test_gpu_parity import run_all
    sc, s, _ = big
    q = meshes.wost_queries(1_000_000, 250_000, 1, 1, seed=21)
    a = run_all(s, q, snch.TRAVERSAL_REFERENCE_ORDER)
    b = run_all(s, q, snch.TRAVERSAL_NEAR_FIRST)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert s.device_status() == 0


def test_persistent_equals_one_thread_per_query_full_scene(big):
    """On the 2M-triangle scene: 2M nearest + 1M silhouette queries, lane-refill
    persistent kernels vs one thread per query."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(2_000_000, 1_000_000, 1, 1, seed=23)

    def run():
        i, d = s.query_nearest(q["near_pts"])
        sd, se = s.query_silhouette(q["sil_pts"], q["sil_flip"])
        return [x.cpu().numpy() for x in (i, d, sd, se)]

    s.set_option(snch.OPT_PERSISTENT, 0)
    a = run()
    s.set_option(snch.OPT_PERSISTENT, 1)
    b = run()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0


def test_tail_cap_full_scene(big):
    """On the 2M-triangle scene: 2M nearest + 1M silhouette queries, uncapped vs
    a cap of 32 expansions (most queries deferred) vs the default."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(2_000_000, 1_000_000, 1, 1, seed=29)

    def run():
        i, d = s.query_nearest(q["near_pts"])
        sd, se = s.query_silhouette(q["sil_pts"], q["sil_flip"])
        return [x.cpu().numpy() for x in (i, d, sd, se)]

    s.set_option(snch.OPT_TAIL_CAP, 0)
    a = run()
    for cap in (32, 128):
        s.set_option(snch.OPT_TAIL_CAP, cap)
        b = run()
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0


def _packet_answers(s, q, flip):
    i, d = s.query_nearest(q)
    sd, se = s.query_silhouette(q, flip)
    return [x.cpu().numpy() for x in (i, d, sd, se)]


def _check_persistent_packets(snch, sc, s, orc, pts, flip, n_oracle):
    """Persistent warp packets (nearest_packet_persistent_kernel,
    silhouette_packet_persistent_kernel) against the grid-launched packets
    (bit for bit: the same packets walk the same traversals), the per-lane
    searches (distances bit for bit, ids equal or an FP64 distance tie) and, on
    a seeded subset of the same batch, the oracle (query.cuh:239-318, 326-423)."""
    s.set_option(snch.OPT_PACKET, 0)
    lane = _packet_answers(s, pts, flip)
    s.set_option(snch.OPT_PACKET, 2)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1 << 40)  # grid launch
    grid = _packet_answers(s, pts, flip)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1)  # persistent at any size
    pers = _packet_answers(s, pts, flip)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, PERSISTENT_MIN_DEFAULT)
    assert s.get_option(snch.OPT_PACKET_PERSISTENT_MIN) == PERSISTENT_MIN_DEFAULT
    assert s.device_status() == 0
    for name, x, y in zip(("nearest idx", "nearest dist", "silhouette dist", "silhouette edge"), grid, pers):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32), err_msg=name)
    np.testing.assert_array_equal(bits(pers[1]), bits(lane[1]))
    np.testing.assert_array_equal(bits(pers[2]), bits(lane[2]))
    check_tri_ids(pers[0], lane[0], lane[1], pts, sc.verts, sc.faces)
    check_edge_ids(pers[3], lane[3], lane[2], pts, sc.verts, s.export_topology()[2])
    sub = np.random.default_rng(len(pts)).choice(len(pts), n_oracle, replace=False)
    oi, od = orc.nearest(pts[sub])
    np.testing.assert_array_equal(bits(pers[1][sub]), bits(od))
    check_tri_ids(pers[0][sub], oi, od, pts[sub], sc.verts, sc.faces)
    osd, ose = orc.silhouette(pts[sub], flip[sub])
    check_silhouette(pers[2][sub], osd)
    same = bits(pers[2][sub]) == bits(osd)
    check_edge_ids(pers[3][sub][same], ose[same], osd[same], pts[sub][same], sc.verts, s.export_topology()[2])


def test_persistent_packets_full_scene(big, oracle_mod):
    """2M nearest + 2M silhouette queries on the 2M-triangle scene with the
    persistent packet kernels forced below their default batch size."""
    import snch_lbvh_gb300 as snch
    sc, s, orc = big
    rng = np.random.default_rng(31)
    pts = rng.random((2_000_000, 3), dtype=np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    _check_persistent_packets(snch, sc, s, orc, pts, flip, 100_000)


def test_persistent_packets_bench_size(big, oracle_mod):
    """A batch above 2^23 queries, run with the default settings as the
    16M-query walk-on-stars step runs (persistent packets from per-SM pools)."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, orc = big
    n = (1 << 23) + 12_345
    q = meshes.wost_queries(n, 1, 1, 1, seed=37)
    pts = q["near_pts"]
    flip = np.zeros(n, np.uint8)  # the step's silhouette queries carry flip = false
    _check_persistent_packets(snch, sc, s, orc, pts, flip, 65_536)


def test_output_scatter_equals_direct_stores(big):
    """SNCH_OPT_OUTPUT_SCATTER: results written in batch (Morton) order and then
    scattered to input order equal the results stored at input positions by the
    search kernels, for all four query types (Morton-ordered 1M-query batches)."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(1_000_000, 1_000_000, 1_000_000, 1_000_000, seed=43)

    def run():
        r = list(s.query_nearest(q["near_pts"])) + list(s.query_silhouette(q["sil_pts"], q["sil_flip"]))
        r += list(s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"]))
        r += list(s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"]))
        return [x.cpu().numpy() for x in r]

    assert s.get_option(snch.OPT_OUTPUT_SCATTER) == 0
    a = run()
    s.set_option(snch.OPT_OUTPUT_SCATTER, 1)
    b = run()
    s.set_option(snch.OPT_OUTPUT_SCATTER, 0)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0


@pytest.mark.parametrize("levels", [1, 5, 7])
def test_top_levels_in_shared_memory_equal(big, levels):
    """SNCH_OPT_TOP_LEVELS: the persistent packet searches reading the top tree
    levels from a shared-memory copy (bulk-copied per block) give the answers of
    the searches reading them from global memory, bit for bit (2M queries each,
    persistent packets forced at this size)."""
    import snch_lbvh_gb300 as snch
    sc, s, _ = big
    rng = np.random.default_rng(47 + levels)
    pts = rng.random((2_000_000, 3), dtype=np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1)
    a = _packet_answers(s, pts, flip)
    s.set_option(snch.OPT_TOP_LEVELS, levels)
    b = _packet_answers(s, pts, flip)
    s.set_option(snch.OPT_TOP_LEVELS, 0)
    s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, PERSISTENT_MIN_DEFAULT)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
    assert s.device_status() == 0


def test_ray_length_order_equal(big):
    """SNCH_OPT_RAY_ORDER = 1 (rays ordered by length bucket, then origin) gives
    the same closest hits and occlusion flags as the origin-ordered batch
    (1M rays with tmax log-uniform over three decades)."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(1, 1, 1_000_000, 1, seed=53)

    def run():
        r = [x.cpu().numpy() for x in s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])]
        return r + [s.query_ray_test(q["ray_o"], q["ray_d"], q["ray_tmax"]).cpu().numpy()]

    a = run()
    s.set_option(snch.OPT_RAY_ORDER, 1)
    b = run()
    s.set_option(snch.OPT_RAY_ORDER, 0)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s.device_status() == 0


@pytest.mark.parametrize("bits", [30, 16])
def test_order_bits_same_answers(big, bits):
    """SNCH_OPT_ORDER_BITS: ordering batches by fewer Morton bits changes which
    queries share a warp packet, not the answers: distances, ray hits and sphere
    samples bit for bit, triangle indices / silhouette edge ids equal or an FP64
    distance tie (1M queries per type)."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(1_000_000, 1_000_000, 1_000_000, 1_000_000, seed=59)

    def run():
        r = list(s.query_nearest(q["near_pts"])) + list(s.query_silhouette(q["sil_pts"], q["sil_flip"]))
        r += list(s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"]))
        r += list(s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"]))
        return [x.cpu().numpy() for x in r]

    assert s.get_option(snch.OPT_ORDER_BITS) == 24
    a = run()
    s.set_option(snch.OPT_ORDER_BITS, bits)
    b = run()
    s.set_option(snch.OPT_ORDER_BITS, 24)
    for k in (1, 2, 4, 5, 6, 7, 8, 9):  # distances, ray hit/t/uv/triangle, sample index/pdf
        np.testing.assert_array_equal(a[k].view(np.uint8), b[k].view(np.uint8))
    check_tri_ids(b[0], a[0], a[1], q["near_pts"], sc.verts, sc.faces)
    check_edge_ids(b[3], a[3], a[2], q["sil_pts"], sc.verts, s.export_topology()[2])
    assert s.device_status() == 0


def test_ray_pools_equal_grid_launch(big):
    """Ray batches of at least SNCH_OPT_PACKET_PERSISTENT_MIN rays run as warps
    that take 32 rays at a time from per-SM pools (ray_pool_kernel): the same
    per-ray traversal as the one-thread-per-ray grid launch, so hit flags, t, uv,
    triangle indices and occlusion flags are identical (2M rays, 2M-triangle
    scene, ordered and unordered batches)."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc, s, _ = big
    q = meshes.wost_queries(1, 1, 2_000_003, 1, seed=73)
    args = (q["ray_o"], q["ray_d"], q["ray_tmax"])
    try:
        for ordered in (1, 0):
            s.set_option(snch.OPT_QUERY_ORDER, ordered)
            s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1 << 40)  # grid launch
            grid = [x.cpu().numpy() for x in s.query_ray(*args)] + [s.query_ray_test(*args).cpu().numpy()]
            s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, 1)  # pools at any size
            pool = [x.cpu().numpy() for x in s.query_ray(*args)] + [s.query_ray_test(*args).cpu().numpy()]
            for name, x, y in zip(("hit", "t", "uv", "triangle", "occluded"), grid, pool):
                np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8), err_msg=name)
    finally:
        s.set_option(snch.OPT_QUERY_ORDER, 1)
        s.set_option(snch.OPT_PACKET_PERSISTENT_MIN, PERSISTENT_MIN_DEFAULT)
    assert s.device_status() == 0
