"""CUDA-graph capture of a solver step (snch_graph_create): a captured rebuild +
nearest + silhouette batch, replayed on refilled buffers (moved vertices, new
query points), gives exactly what the same calls give outside a graph -- for a
plain scene, a batched scene and wide nodes; and the autotuner keeps a width
whose results are the plain ones."""
import numpy as np
import pytest

from test_gpu_parity import bits, check_edge_ids, check_tri_ids

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def direct(snch, v, f, pts, flip, width=2):
    s = snch.Scene(v, f)
    s.set_option(snch.OPT_NODE_WIDTH, width)
    s.compute_silhouettes()
    s.build_bvh()
    i, d = s.query_nearest(pts)
    sd, se = s.query_silhouette(pts, flip)
    return [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]


@pytest.mark.parametrize("width", [2, 4])
def test_graph_rebuild_and_queries(snch, width):
    import torch
    from snch_lbvh_gb300 import meshes
    v0, f = meshes.noisy_icosphere(4, 1.0, 0.01, seed=1)
    rng = np.random.default_rng(3)
    n = 150_000  # above the Morton-ordering threshold: the ordering sort is captured too
    s = snch.Scene(v0, f)
    s.set_option(snch.OPT_NODE_WIDTH, width)
    s.compute_silhouettes()
    s.build_bvh()
    pts = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    flip = torch.empty(n, dtype=torch.uint8, device="cuda")
    out_n = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"))
    out_s = (torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))
    st = torch.cuda.Stream()
    torch.cuda.synchronize()  # the first build (current stream) is done before the graph's
    g = s.capture(True, pts, out_n, pts, flip, out_s, stream=st)
    for k in range(3):
        v = (v0 * np.float32(1.0 + 0.05 * k) + np.float32(0.01 * k)).astype(np.float32)  # moved vertices
        q = meshes.box_queries(v, n, 1.2, seed=10 + k)
        fl = (rng.random(n) < 0.5).astype(np.uint8)
        with torch.cuda.stream(st):
            s.vertices().copy_(torch.from_numpy(v))
            pts.copy_(torch.from_numpy(q))
            flip.copy_(torch.from_numpy(fl))
            g.launch(st)
        st.synchronize()
        got = [out_n[0].cpu().numpy(), bits(out_n[1].cpu().numpy()), bits(out_s[0].cpu().numpy()),
               out_s[1].cpu().numpy()]
        exp = direct(snch, v, f, q, fl, width)
        for x, y in zip(exp, got):
            np.testing.assert_array_equal(y, x)
    assert s.device_status() == 0
    g.close()


def test_graph_batched_queries(snch):
    import torch
    from test_gpu_batched import mixed_meshes
    rng = np.random.default_rng(4)
    ms = mixed_meshes(rng, 20)
    b = snch.BatchedScene(ms)
    b.compute_silhouettes()
    b.build_bvh()
    mesh, pts = [], []
    for m, (v, f) in enumerate(ms):
        lo, hi = v.min(0), v.max(0)
        pts.append((lo + (hi - lo + 1e-3) * rng.random((3000, 3))).astype(np.float32))
        mesh.append(np.full(3000, m, np.int32))
    perm = rng.permutation(3000 * len(ms))
    mesh = torch.from_numpy(np.concatenate(mesh)[perm]).cuda()
    pts = torch.from_numpy(np.concatenate(pts)[perm]).cuda()
    flip = torch.from_numpy((rng.random(len(pts)) < 0.5).astype(np.uint8)).cuda()
    i0, d0 = b.query_nearest_batch(mesh, pts)
    sd0, se0 = b.query_silhouette_batch(mesh, pts, flip)
    n = len(pts)
    out_n = (torch.full((n,), 7, dtype=torch.int32, device="cuda"), torch.zeros(n, dtype=torch.float32, device="cuda"))
    out_s = (torch.zeros(n, dtype=torch.float32, device="cuda"), torch.zeros(n, dtype=torch.int32, device="cuda"))
    st = torch.cuda.Stream()
    # the graph rebuilds the scene on another stream: the direct queries above
    # (current stream) must be done before it runs
    torch.cuda.synchronize()
    g = b.capture(True, pts, out_n, pts, flip, out_s, near_mesh=mesh, sil_mesh=mesh, stream=st)
    for _ in range(2):
        g.launch(st)
        st.synchronize()
        np.testing.assert_array_equal(out_n[0].cpu().numpy(), i0.cpu().numpy())
        np.testing.assert_array_equal(bits(out_n[1].cpu().numpy()), bits(d0.cpu().numpy()))
        np.testing.assert_array_equal(bits(out_s[0].cpu().numpy()), bits(sd0.cpu().numpy()))
        np.testing.assert_array_equal(out_s[1].cpu().numpy(), se0.cpu().numpy())
    assert b.device_status() == 0
    g.close()


def test_graph_needs_a_built_scene_and_a_stream(snch):
    import torch
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    s = snch.Scene(v, np.array([[0, 1, 2]], np.int32))
    p = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    o = (torch.empty(4, dtype=torch.int32, device="cuda"), torch.empty(4, dtype=torch.float32, device="cuda"))
    with pytest.raises(snch.SnchError):
        s.capture(True, p, o, stream=torch.cuda.Stream())
    s.compute_silhouettes()
    s.build_bvh()
    with pytest.raises(snch.SnchError):
        s.capture(True, p, o, stream=torch.cuda.default_stream())


def test_autotune_keeps_results(snch):
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    pts = meshes.box_queries(v, 200_000, 1.2, seed=6)
    flip = (np.arange(len(pts)) % 2).astype(np.uint8)
    exp = direct(snch, v, f, pts, flip)
    s = snch.Scene(v, f)
    s.compute_silhouettes()
    s.build_bvh()
    ms = s.autotune(pts, pts, flip)
    for kind in ("nearest", "silhouette"):
        assert set(ms[kind]) == set(s.AUTOTUNE_CONFIGS) and all(t > 0 for t in ms[kind].values())
        assert s.search_config(kind) == min(ms[kind], key=ms[kind].get)
    i, d = s.query_nearest(pts)
    sd, se = s.query_silhouette(pts, flip)
    got = [i.cpu().numpy(), bits(d.cpu().numpy()), bits(sd.cpu().numpy()), se.cpu().numpy()]
    for x, y in zip(exp[1:3], got[1:3]):
        np.testing.assert_array_equal(y, x)
    check_tri_ids(got[0], exp[0], d.cpu().numpy(), pts, v, f)
    check_edge_ids(got[3], exp[3], sd.cpu().numpy(), pts, v, s.export_topology()[2])
    s.build_bvh()  # a rebuild keeps the chosen widths
    assert s.device_status() == 0
