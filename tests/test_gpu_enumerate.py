"""AABB-overlap and line enumeration (query.cuh:177-231, 15-77) on the GPU:
triangle indices in the reference's order, line parameters and counts bit for
bit against the reference's own outputs (golden) and the oracle (config-1
icosphere, 2M-triangle scene), truncation to max_per_query, count-only calls,
one-triangle trees."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import bits, built_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def as_u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("name", golden_names())
def test_enumeration_matches_reference_golden(snch, oracle_mod, name):
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    k = 64
    idx, cnt = s.query_overlap(g["box_q"], k)
    li, lt, lc = s.query_line(g["line_o"], g["line_d"], k)
    if len(g["ref_box_count"]):
        np.testing.assert_array_equal(as_u32(cnt), g["ref_box_count"])
        np.testing.assert_array_equal(as_u32(idx), g["ref_box_idx"])
        np.testing.assert_array_equal(as_u32(lc), g["ref_line_count"])
        np.testing.assert_array_equal(as_u32(li), g["ref_line_idx"])
        np.testing.assert_array_equal(bits(lt.cpu().numpy()), bits(g["ref_line_t"]))
    else:  # one triangle: the reference reads past its node array; the oracle tests the leaf
        t = oracle_mod.Tree(g["verts"], g["tris"])
        oi, oc = t.overlap(g["box_q"], k)
        np.testing.assert_array_equal(as_u32(cnt), oc)
        np.testing.assert_array_equal(as_u32(idx), oi)
        oli, olt, olc = t.line(g["line_o"], g["line_d"], k)
        np.testing.assert_array_equal(as_u32(lc), olc)
        np.testing.assert_array_equal(as_u32(li), oli)
        np.testing.assert_array_equal(bits(lt.cpu().numpy()), bits(olt))
    assert s.device_status() == 0


@pytest.mark.parametrize("mesh", ["config1", "wost"])
def test_enumeration_matches_oracle(snch, oracle_mod, mesh):
    from snch_lbvh_gb300 import meshes
    rng = np.random.default_rng(21)
    if mesh == "config1":
        v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    else:
        sc = meshes.wost_scene(seed=0)
        v, f = sc.verts, sc.faces
    lo, hi = v.min(0), v.max(0)
    n = 20_000
    c = lo + (hi - lo) * rng.random((n, 3))
    h = np.exp(rng.uniform(np.log(1e-4), np.log(0.05), (n, 3))) * (hi - lo).max()
    boxes = np.concatenate([c - h, c + h], 1).astype(np.float32)
    d = rng.standard_normal((n, 3))
    d[: n // 8, :2] = 0.0  # axis-aligned lines: 0 * inf in the slab test
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o, d = c.astype(np.float32), d.astype(np.float32)
    s = built_scene(snch, v, f)
    t = oracle_mod.Tree(v, f)
    for k in (0, 5, 48):
        idx, cnt = s.query_overlap(boxes, k)
        oi, oc = t.overlap(boxes, k)
        np.testing.assert_array_equal(as_u32(cnt), oc)
        np.testing.assert_array_equal(as_u32(idx), oi)
        li, lt, lc = s.query_line(o, d, k)
        oli, olt, olc = t.line(o, d, k)
        np.testing.assert_array_equal(as_u32(lc), olc)
        np.testing.assert_array_equal(as_u32(li), oli)
        np.testing.assert_array_equal(bits(lt.cpu().numpy()), bits(olt))
    assert int(cnt.max()) > 48  # truncation was exercised
    assert s.device_status() == 0


def test_enumeration_rejects_batched(snch):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b = snch.BatchedScene([(v, np.array([[0, 1, 2]], np.int32))] * 2)
    b.compute_silhouettes()
    b.build_bvh()
    with pytest.raises(snch.SnchError):
        b.query_overlap(np.zeros((1, 6), np.float32))


def test_scene_save_load_roundtrip(snch, tmp_path):
    """A saved and reloaded scene has the same tree and answers every query the
    same, bit for bit, without a rebuild; damaged files are refused."""
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(4, 1.0, 0.01, seed=4)
    q = meshes.wost_queries(20_000, 20_000, 20_000, 20_000, seed=3)
    for k in ("near_pts", "sil_pts", "ray_o", "smp_c"):
        q[k] = (q[k] * 2.4 - 1.2).astype(np.float32)
    a = built_scene(snch, v, f)
    path = str(tmp_path / "scene.snch")
    a.save(path)
    b = snch.Scene.load(path)

    def everything(s):
        tr = s.export_tree()
        i, d = s.query_nearest(q["near_pts"])
        sd, se = s.query_silhouette(q["sil_pts"], q["sil_flip"])
        h, t, uv, ri = s.query_ray(q["ray_o"], q["ray_d"], q["ray_tmax"])
        si, sp = s.sample_in_sphere(q["smp_c"], q["smp_r"], q["smp_u"])
        oi, oc = s.query_overlap(np.concatenate([q["smp_c"] - 0.05, q["smp_c"] + 0.05], 1)[:2000], 16)
        return [tr[k] for k in sorted(tr)] + [x.cpu().numpy() for x in (i, d, sd, se, h, t, uv, ri, si, sp, oi, oc)]

    for x, y in zip(everything(a), everything(b)):
        np.testing.assert_array_equal(bits(np.ascontiguousarray(x)) if x.dtype == np.float32 else x,
                                      bits(np.ascontiguousarray(y)) if y.dtype == np.float32 else y)
    assert b.info() == a.info() and b.get_bvh_device_ptr().num_objects == len(f)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:-100])
    with pytest.raises(snch.SnchError, match="truncated"):
        snch.Scene.load(path)
    open(path, "wb").write(b"NOTASCENE" + raw[9:])
    with pytest.raises(snch.SnchError):
        snch.Scene.load(path)
    b.build_bvh()  # a loaded scene can be rebuilt like any other
    assert b.device_status() == 0
