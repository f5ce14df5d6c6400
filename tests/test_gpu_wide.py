"""4- and 8-way nodes: the near-first nearest and silhouette searches over the
wide records return exactly what the binary near-first searches (and so the
reference's traversal order) return -- indices, distances and silhouette edge
ids bit for bit, exact-tie probes included -- on the golden meshes, the
config-1 icosphere, the 2M-triangle scene, batched scenes and seeded searches."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import bits, built_scene

pytestmark = pytest.mark.gpu

WIDTHS = (4, 8)


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def answers(s, pts, flip):
    i, d = s.query_nearest(pts)
    sd, se = s.query_silhouette(pts, flip)
    return [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]


def check_widths(snch, s, pts, flip):
    s.set_option(snch.OPT_PACKET, 0)  # wide searches run per lane: compare with per-lane binary
    s.set_option(snch.OPT_NODE_WIDTH, 2)
    base = answers(s, pts, flip)
    for w in WIDTHS:
        s.set_option(snch.OPT_NODE_WIDTH, w)
        got = answers(s, pts, flip)
        for name, x, y in zip(("nearest idx", "nearest dist", "silhouette dist", "silhouette edge"), base, got):
            np.testing.assert_array_equal(y, x, err_msg=f"width {w}: {name}")
        assert s.device_status() == 0
    s.set_option(snch.OPT_NODE_WIDTH, 2)
    return base


def tie_probes(v, f):
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    mids = (0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])).astype(np.float32)
    cent = (v[f].astype(np.float64).mean(1)).astype(np.float32)
    return np.concatenate([v, mids, cent]).astype(np.float32)


@pytest.mark.parametrize("name", golden_names())
def test_wide_equals_binary_golden(snch, name):
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    pts = np.concatenate([g["near_pts"], g["sil_pts"], tie_probes(g["verts"], g["tris"])]).astype(np.float32)
    flip = (np.arange(len(pts)) % 2).astype(np.uint8)
    base = check_widths(snch, s, pts, flip)
    if len(g["ref_near_idx"]):
        k = len(g["ref_near_idx"])
        np.testing.assert_array_equal(base[0][:k].view(np.uint32), g["ref_near_idx"])


def test_wide_equals_binary_config1(snch):
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = np.concatenate([meshes.box_queries(v, 1_000_000, 1.2, seed=1), tie_probes(v, f)])
    flip = (np.random.default_rng(2).random(len(pts)) < 0.5).astype(np.uint8)
    s = built_scene(snch, v, f)
    check_widths(snch, s, pts, flip)


def test_wide_equals_binary_wost_scene(snch):
    """The 1,993,600-triangle scene, 1M uniform points (Morton-ordered batches)."""
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    s = built_scene(snch, sc.verts, sc.faces)
    rng = np.random.default_rng(5)
    pts = rng.random((1_000_000, 3), dtype=np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    check_widths(snch, s, pts, flip)


def test_wide_set_before_build_and_per_type(snch):
    """Widths chosen before the build, per query type, and rebuilds."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(4, 1.0, 0.01, seed=3)
    pts = np.concatenate([meshes.box_queries(v, 200_000, 1.2, seed=2), tie_probes(v, f)])
    flip = (np.arange(len(pts)) % 3 == 0).astype(np.uint8)
    s0 = built_scene(snch, v, f)
    s0.set_option(snch.OPT_PACKET, 0)
    ref = answers(s0, pts, flip)
    for wn, ws in ((4, 8), (8, 4), (2, 8), (4, 2)):
        s = snch.Scene(v, f)
        s.set_option(snch.OPT_PACKET, 0)
        s.set_option(snch.OPT_NODE_WIDTH_NEAREST, wn)
        s.set_option(snch.OPT_NODE_WIDTH_SILHOUETTE, ws)
        s.compute_silhouettes()
        s.build_bvh()
        for _ in range(2):  # a rebuild replaces the wide records
            got = answers(s, pts, flip)
            for x, y in zip(ref, got):
                np.testing.assert_array_equal(y, x)
            s.build_bvh()
        assert s.device_status() == 0
    with pytest.raises(snch.SnchError):
        s.set_option(snch.OPT_NODE_WIDTH, 3)


def test_wide_small_trees(snch):
    """One, two and three triangles: every node is a root or a leaf child."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5], [2, 0, 0.2]], np.float32)
    for f in ([[0, 1, 2]], [[0, 1, 2], [1, 3, 2]], [[0, 1, 2], [1, 3, 2], [1, 4, 3]]):
        f = np.array(f, np.int32)
        s = built_scene(snch, v, f)
        pts = np.concatenate([v, np.random.default_rng(0).random((500, 3), dtype=np.float32) * 3 - 1])
        check_widths(snch, s, pts, (np.arange(len(pts)) % 2).astype(np.uint8))


@pytest.mark.parametrize("w", WIDTHS)
def test_wide_seeded_equals_unseeded(snch, w):
    from snch_lbvh_gb300 import meshes
    from test_gpu_seeded import radii_mix
    rng = np.random.default_rng(7)
    sc = meshes.wost_scene(seed=2, n_meshes=8, torus_nu=60, torus_nv=30, ico_level=4)
    s = built_scene(snch, sc.verts, sc.faces)
    s.set_option(snch.OPT_PACKET, 0)
    pts = rng.random((300_000, 3), dtype=np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    i0, d0 = s.query_nearest(pts)
    sd0, se0 = s.query_silhouette(pts, flip)
    s.set_option(snch.OPT_NODE_WIDTH, w)
    r, _ = radii_mix(d0.cpu().numpy(), rng)
    i1, d1 = s.query_nearest_seeded(pts, r)
    np.testing.assert_array_equal(i1.cpu().numpy(), i0.cpu().numpy())
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d0.cpu().numpy()))
    rs, _ = radii_mix(sd0.cpu().numpy(), rng)
    sd1, se1 = s.query_silhouette_seeded(pts, rs, flip)
    np.testing.assert_array_equal(bits(sd1.cpu().numpy()), bits(sd0.cpu().numpy()))
    np.testing.assert_array_equal(se1.cpu().numpy(), se0.cpu().numpy())
    assert s.device_status() == 0


@pytest.mark.parametrize("w", WIDTHS)
def test_wide_batched_equals_binary(snch, w):
    """Batched scenes: every mesh's subtree gets its own wide root."""
    from test_gpu_batched import mixed_meshes
    rng = np.random.default_rng(11)
    ms = mixed_meshes(rng, 30)
    ms.insert(4, (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32)))
    b = snch.BatchedScene(ms)
    b.set_option(snch.OPT_PACKET, 0)
    b.compute_silhouettes()
    b.build_bvh()
    mesh, pts = [], []
    for m, (v, f) in enumerate(ms):
        lo, hi = v.min(0), v.max(0)
        p = (lo + (hi - lo + 1e-3) * (1.4 * rng.random((2000, 3)) - 0.2)).astype(np.float32)
        p[: min(len(v), 500)] = v[:500]
        pts.append(p)
        mesh.append(np.full(len(p), m, np.int32))
    mesh, pts = np.concatenate(mesh), np.concatenate(pts)
    perm = rng.permutation(len(pts))
    mesh, pts = mesh[perm], pts[perm]
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)

    def run():
        i, d = b.query_nearest_batch(mesh, pts)
        sd, se = b.query_silhouette_batch(mesh, pts, flip)
        return [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]

    base = run()
    b.set_option(snch.OPT_NODE_WIDTH, w)
    for x, y in zip(base, run()):
        np.testing.assert_array_equal(y, x)
    assert b.device_status() == 0


def test_wide_visits_fewer_nodes(snch):
    """A wide search expands fewer (wider) nodes than the binary one."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = meshes.box_queries(v, 100_000, 1.2, seed=8)
    flip = np.zeros(len(pts), np.uint8)
    s = built_scene(snch, v, f)
    counts = {}
    for w in (2, 4, 8):
        s.set_option(snch.OPT_NODE_WIDTH, w)
        counts[w] = (s.query_visits("nearest", pts)[:, 0].mean(),
                     s.query_visits("silhouette", pts, flip=flip)[:, 0].mean())
    assert counts[4][0] < 0.75 * counts[2][0] and counts[8][0] < counts[4][0]
    assert counts[4][1] < 0.75 * counts[2][1] and counts[8][1] < counts[4][1]


@pytest.mark.parametrize("block", [64, 256])
def test_block_size_same_results(snch, block):
    """64- and 256-thread blocks of the binary searches return the 128-thread results."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = np.concatenate([meshes.box_queries(v, 300_000, 1.2, seed=12), tie_probes(v, f)])
    flip = (np.arange(len(pts)) % 2).astype(np.uint8)
    s = built_scene(snch, v, f)
    base = answers(s, pts, flip)
    s.set_option(snch.OPT_BLOCK, block)
    assert s.search_config("nearest")[:2] == (2, block) and s.search_config("silhouette")[:2] == (2, block)
    for x, y in zip(base, answers(s, pts, flip)):
        np.testing.assert_array_equal(y, x)
    with pytest.raises(snch.SnchError):
        s.set_option(snch.OPT_BLOCK, 96)
