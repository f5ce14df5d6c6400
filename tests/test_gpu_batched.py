"""Batched scenes: many meshes built and queried together give, mesh by mesh,
exactly what a Scene of that mesh alone gives (per-mesh triangle indices and
silhouette edge ids, distances bit for bit), in any mix and order of queries."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import bits, built_scene, check_edge_ids, check_tri_ids

pytestmark = pytest.mark.gpu


def mixed_meshes(rng, count):
    from snch_lbvh_gb300 import meshes
    out = []
    for k in range(count):
        kind = k % 3
        if kind == 0:
            v, f = meshes.noisy_icosphere(int(rng.integers(0, 4)), float(rng.uniform(0.2, 1.0)), 0.01,
                                          seed=int(rng.integers(1 << 30)))
        elif kind == 1:
            nu = int(rng.integers(6, 40))
            v, f = meshes.noisy_torus(float(rng.uniform(0.2, 0.5)), 0.1, nu, max(3, nu // 2), 0.002,
                                      seed=int(rng.integers(1 << 30)))
        else:
            g = load_golden(golden_names()[k // 3 % len(golden_names())])
            v, f = g["verts"], g["tris"]
        v = (v + rng.uniform(-2, 2, 3)).astype(np.float32)  # meshes overlap in space and in Morton boxes
        out.append((v.astype(np.float32), f.astype(np.int32)))
    return out


def check_batch(snch, ms, rng, per_mesh=3000, options=None):
    b = snch.BatchedScene(ms)
    b.compute_silhouettes()
    b.build_bvh()
    for k, val in (options or {}).items():
        b.set_option(k, val)
    assert b.num_meshes == len(ms)
    mesh_ids, pts, flips, expect, tops = [], [], [], [], []
    for m, (v, f) in enumerate(ms):
        if len(v) == 0:
            p = rng.random((50, 3), dtype=np.float32)
        else:
            p = snch_box_queries(v, per_mesh, rng)
        fl = (rng.random(len(p)) < 0.5).astype(np.uint8)
        if len(f):
            s = built_scene(snch, v, f)
            i, d = s.query_nearest(p)
            sd, se = s.query_silhouette(p, fl)
            expect.append([x.cpu().numpy() for x in (i, d, sd, se)])
            tops.append(s.export_topology()[2])
        else:
            tops.append(None)
            n = len(p)
            expect.append([np.full(n, -1, np.int32), np.full(n, np.inf, np.float32), np.full(n, np.inf, np.float32),
                           np.full(n, -1, np.int32)])
        mesh_ids.append(np.full(len(p), m, np.int32))
        pts.append(p)
        flips.append(fl)
    mesh_ids, pts, flips = np.concatenate(mesh_ids), np.concatenate(pts), np.concatenate(flips)
    exp = [np.concatenate([e[k] for e in expect]) for k in range(4)]
    perm = rng.permutation(len(pts))  # queries of all meshes interleaved
    i, d = b.query_nearest_batch(mesh_ids[perm], pts[perm])
    sd, se = b.query_silhouette_batch(mesh_ids[perm], pts[perm], flips[perm])
    got = [x.cpu().numpy() for x in (i, d, sd, se)]
    for g, e in zip(got[1:3], exp[1:3]):
        np.testing.assert_array_equal(bits(g), bits(e[perm]))
    # silhouette edge ids, mesh by mesh: equal or an exact tie (warp packets)
    back = np.empty_like(perm)
    back[perm] = np.arange(len(perm))
    se_in, ni_in = got[3][back], got[0][back]
    start = 0
    for m, (v, f) in enumerate(ms):
        k = int((mesh_ids == m).sum())  # mesh_ids are mesh-major before the permutation
        sl = slice(start, start + k)
        if tops[m] is not None:
            check_tri_ids(ni_in[sl], exp[0][sl], exp[1][sl], pts[sl], v, f, max_frac=1e-2)
            check_edge_ids(se_in[sl], exp[3][sl], exp[2][sl], pts[sl], v, tops[m], max_frac=1e-2)
        else:
            np.testing.assert_array_equal(se_in[sl], exp[3][sl])
            np.testing.assert_array_equal(ni_in[sl], exp[0][sl])
        start += k
    assert b.device_status() == 0
    return b


def snch_box_queries(v, n, rng):
    lo, hi = v.min(0), v.max(0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.2 + 1e-3
    p = (c + h * (2 * rng.random((n, 3)) - 1)).astype(np.float32)
    # exact-tie probes: vertices
    k = min(len(v), n // 4)
    p[:k] = v[:k]
    return p


def test_batched_equals_single_scenes_golden_and_mixed(snch_mod):
    rng = np.random.default_rng(1)
    ms = mixed_meshes(rng, 24)
    ms.insert(5, (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)))  # an empty mesh
    ms.insert(9, (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32)))
    check_batch(snch_mod, ms, rng)


def test_batched_many_meshes_ordered_batch(snch_mod):
    """300 meshes (mesh ids need 9 bits), > 65536 queries (Morton-ordered by mesh)."""
    rng = np.random.default_rng(2)
    from snch_lbvh_gb300 import meshes
    ms = []
    for k in range(300):
        v, f, _ = meshes.icosphere(int(rng.integers(0, 3)), float(rng.uniform(0.1, 1)))
        ms.append(((v + rng.uniform(-1, 1, 3)).astype(np.float32), f.astype(np.int32)))
    check_batch(snch_mod, ms, rng, per_mesh=400)


def test_batched_persistent_work_stealing(snch_mod):
    """Persistent work-stealing searches (SNCH_OPT_PERSISTENT) on a batched scene:
    per-mesh roots, empty and one-triangle meshes, results as single scenes give,
    and bit for bit the one-thread-per-query searches' results."""
    snch = snch_mod
    rng = np.random.default_rng(3)
    ms = mixed_meshes(rng, 18)
    ms.insert(4, (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)))
    ms.insert(7, (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32)))
    # one query per lane (warp packets run persistent anyway and are covered by
    # check_batch in the other tests)
    b = check_batch(snch, ms, rng, per_mesh=2000, options={snch.OPT_PERSISTENT: 1, snch.OPT_PACKET: 0})
    n = 100_000
    mesh = rng.integers(0, len(ms), n).astype(np.int32)
    pts = rng.uniform(-3, 3, (n, 3)).astype(np.float32)
    flip = (rng.random(n) < 0.5).astype(np.uint8)

    def run():
        out = list(b.query_nearest_batch(mesh, pts)) + list(b.query_silhouette_batch(mesh, pts, flip))
        return [x.cpu().numpy() for x in out]

    got = run()
    b.set_option(snch.OPT_PERSISTENT, 0)
    want = run()
    for x, y in zip(got, want):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    assert b.device_status() == 0
    b.close()


def test_batched_seeded_equals_plain(snch_mod):
    """Seeded batched searches (per-query radii: exact, too small, large, zero)
    return the plain batched results bit for bit and count the fallbacks."""
    import torch
    snch = snch_mod
    rng = np.random.default_rng(4)
    ms = mixed_meshes(rng, 12)
    b = snch.BatchedScene(ms)
    b.compute_silhouettes()
    b.build_bvh()
    n = 200_000
    mesh = torch.from_numpy(rng.integers(0, len(ms), n).astype(np.int32)).cuda()
    pts = torch.from_numpy(rng.uniform(-3, 3, (n, 3)).astype(np.float32)).cuda()
    flip = torch.from_numpy((rng.random(n) < 0.5).astype(np.uint8)).cuda()
    i0, d0 = b.query_nearest_batch(mesh, pts)
    s0, e0 = b.query_silhouette_batch(mesh, pts, flip)
    for scale in (1.0, 0.5, 4.0, 0.0):
        rn = torch.where(torch.isfinite(d0), d0 * scale, torch.full_like(d0, 1.0))
        rs = torch.where(torch.isfinite(s0), s0 * scale, torch.full_like(s0, 1.0))
        nf = torch.zeros(2, dtype=torch.int32, device="cuda")
        i1, d1 = b.query_nearest_batch_seeded(mesh, pts, rn, num_fallback=nf[0:1])
        s1, e1 = b.query_silhouette_batch_seeded(mesh, pts, rs, flip, num_fallback=nf[1:2])
        assert torch.equal(d1.view(torch.int32), d0.view(torch.int32)), scale
        assert torch.equal(s1.view(torch.int32), s0.view(torch.int32)), scale
        same_i = (i1 == i0) | torch.isinf(d0)
        same_e = (e1 == e0) | torch.isinf(s0)
        # indices: equal up to exact ties whose distance falls on a rounding boundary
        # of a box test (a radius equal to the answer prunes at that boundary; the
        # distances above are identical). Silhouette points nearest to a vertex tie
        # between the edges sharing it: 63 of 200,000 differed at scale 1.
        assert same_i.float().mean().item() > 0.999 and same_e.float().mean().item() > 0.999, scale
        fb = nf.cpu().numpy()
        if scale < 1.0:
            assert fb[0] > 0  # radii below the answer: those queries fall back
        if scale > 1.0:
            assert fb[0] < n // 100 and fb[1] < n // 100
    assert b.device_status() == 0
    b.close()


def test_batched_rejects_bad_input(snch_mod):
    snch = snch_mod
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    with pytest.raises(snch.SnchError):
        snch.BatchedScene([(v, np.array([[0, 1, 3]], np.int32))])  # index 3 outside its mesh
    with pytest.raises(snch.SnchError):
        snch.BatchedScene([])
    s = snch.Scene(v, np.array([[0, 1, 2]], np.int32))
    s.compute_silhouettes()
    s.build_bvh()
    with pytest.raises(snch.SnchError):
        s_b = snch.BatchedScene.__new__(snch.BatchedScene)
        s_b._h = s._h
        try:
            s_b.query_nearest_batch(np.zeros(1, np.int32), np.zeros((1, 3), np.float32))
        finally:
            s_b._h = None


@pytest.fixture(scope="module")
def snch_mod():
    import torch
    assert torch.cuda.is_available()
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300
