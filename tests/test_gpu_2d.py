"""2D scenes on the GPU (snch_scene2_*) against the reference's own outputs
(tests/golden/2d/) and the 2D oracle: silhouette vertices, owned vertices,
Morton codes, sorted order, tree and boxes bit for bit; cones within CONE_TOL
(CUDA's acosf / sinf / cosf against libm's) except where the reference leaves
them undefined; nearest and ray bit for bit; silhouette distances bit for bit
in all but a cone-test boundary fraction; circle samples (CUDA's logf in the
weights) bit for bit in all but a boundary fraction."""
import glob
import os

import numpy as np
import pytest

from conftest import d1_tainted
from test_gpu_parity import CONE_TOL, bits

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(ROOT, "tests", "golden", "2d", "*.npz")))


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def load2(name):
    with np.load(os.path.join(ROOT, "tests", "golden", "2d", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def check_cones2(gpu, ref, nodes, d1):
    """Cones where the queries read them: a half-angle >= pi/2 makes the overlap
    test pass on its first line (cone.cuh:84), and every ancestor of such a cone
    has one too, so there only that property is compared. (Near pi the merge is
    ill-conditioned: rotate(float2) takes its direction from the sign of a cross
    product of nearly opposite axes, cone.cuh:268-269, which one ulp of acosf
    can flip.)"""
    taint = d1_tainted(nodes, d1)
    valid = ref[:, 2] >= 0
    np.testing.assert_array_equal((gpu[:, 2] >= 0)[~taint], valid[~taint])
    half_pi = np.float32(np.pi / 2)
    wide = valid & ~taint & (ref[:, 2] >= half_pi - CONE_TOL)
    assert np.all(gpu[wide, 2] >= half_pi - 2 * CONE_TOL)
    ok = valid & ~taint & ~wide
    diff = np.abs(gpu[ok].astype(np.float64) - ref[ok])
    both_nan = np.isnan(gpu[ok]) & np.isnan(ref[ok])
    diff = np.where(both_nan, 0.0, diff)
    assert np.nan_to_num(diff[:, :3], nan=np.inf).max(initial=0) <= CONE_TOL
    assert np.all(np.nan_to_num(diff[:, 3], nan=np.inf) <= CONE_TOL * np.maximum(np.abs(ref[ok, 3]), 1.0))
    assert np.all(gpu[taint, 2] >= 0)


def close_frac(a, b, rtol=1e-6):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    same = (a == b) | (np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b)))
    with np.errstate(invalid="ignore"):
        same |= np.abs(a - b) <= rtol * np.abs(b)
    return same.mean()


@pytest.mark.parametrize("name", NAMES)
def test_2d_matches_reference(snch, oracle_mod, name):
    g = load2(name)
    s = snch.Scene2(g["verts"], g["segs"])
    s.build()
    e = s.export()
    np.testing.assert_array_equal(e["sv"], g["ref_sv"])
    np.testing.assert_array_equal(e["seg_owned"], g["ref_seg_owned"])
    np.testing.assert_array_equal(e["morton"], g["ref_morton"][e["sorted_idx"]])
    np.testing.assert_array_equal(e["nodes"], g["ref_nodes"])
    np.testing.assert_array_equal(bits(e["aabbs"]), bits(g["ref_aabbs"]))
    orc = oracle_mod.Tree2(g["verts"], g["segs"])
    check_cones2(e["cones"], g["ref_cones"], orc.nodes, orc.d1)

    i, d = s.query_nearest(g["near_pts"])
    sd, _ = s.query_silhouette(g["sil_pts"], g["sil_flip"])
    h, t, sp, ri = s.query_ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
    si, spdf = s.sample_in_circle(g["smp_c"], g["smp_r"], g["smp_u"])
    if len(g["ref_near_idx"]):
        ref = {k: g[k] for k in ("ref_near_idx", "ref_near_dist", "ref_sil_dist", "ref_ray_hit", "ref_ray_t",
                                 "ref_ray_s", "ref_ray_idx", "ref_smp_idx", "ref_smp_pdf")}
    else:  # one segment: the reference reads past its node array; the oracle evaluates the segment
        oi, od = orc.nearest(g["near_pts"])
        osd, _ = orc.silhouette(g["sil_pts"], g["sil_flip"])
        oh, ot, osp, ori = orc.ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
        osi, opdf = orc.sample(g["smp_c"], g["smp_r"], g["smp_u"])
        ref = dict(zip(("ref_near_idx", "ref_near_dist", "ref_sil_dist", "ref_ray_hit", "ref_ray_t", "ref_ray_s",
                        "ref_ray_idx", "ref_smp_idx", "ref_smp_pdf"), (oi, od, osd, oh, ot, osp, ori, osi, opdf)))
    np.testing.assert_array_equal(i.cpu().numpy().view(np.uint32), ref["ref_near_idx"])
    np.testing.assert_array_equal(bits(d.cpu().numpy()), bits(ref["ref_near_dist"]))
    assert close_frac(sd.cpu().numpy(), ref["ref_sil_dist"]) >= 0.999
    np.testing.assert_array_equal(h.cpu().numpy(), ref["ref_ray_hit"])
    np.testing.assert_array_equal(bits(t.cpu().numpy()), bits(ref["ref_ray_t"]))
    np.testing.assert_array_equal(bits(sp.cpu().numpy()), bits(ref["ref_ray_s"]))
    np.testing.assert_array_equal(ri.cpu().numpy().view(np.uint32), ref["ref_ray_idx"])
    same_i = si.cpu().numpy() == ref["ref_smp_idx"]
    assert same_i.mean() >= 0.99
    assert close_frac(spdf.cpu().numpy()[same_i], ref["ref_smp_pdf"][same_i], rtol=1e-5) >= 0.99
    assert s.device_status() == 0


def test_2d_large_scene_against_oracle(snch, oracle_mod):
    """A 200,000-segment scene of noisy loops and open polylines, 200k queries
    per type, against the 2D oracle."""
    rng = np.random.default_rng(3)
    verts, segs = [], []
    off = 0
    for k in range(400):
        m = int(rng.integers(8, 900))
        c = rng.random(2) * 20
        a = np.sort(rng.random(m)) * 2 * np.pi
        r = rng.uniform(0.05, 0.6) * (1 + 0.02 * rng.standard_normal(m))
        verts.append(np.stack([c[0] + r * np.cos(a), c[1] + r * np.sin(a)], 1))
        idx = np.arange(m)
        closed = k % 3 != 0
        segs.append(np.stack([idx, (idx + 1) % m], 1)[: m if closed else m - 1] + off)
        off += m
    v = np.concatenate(verts).astype(np.float32)
    sg = np.concatenate(segs).astype(np.int32)
    s = snch.Scene2(v, sg)
    s.build()
    orc = oracle_mod.Tree2(v, sg)
    e = s.export()
    np.testing.assert_array_equal(e["nodes"], orc.nodes)
    np.testing.assert_array_equal(bits(e["aabbs"]), bits(orc.aabbs))
    n = 200_000
    p = (rng.random((n, 2)) * 21 - 0.5).astype(np.float32)
    fl = (rng.random(n) < 0.5).astype(np.uint8)
    i, d = s.query_nearest(p)
    oi, od = orc.nearest(p)
    np.testing.assert_array_equal(i.cpu().numpy().view(np.uint32), oi)
    np.testing.assert_array_equal(bits(d.cpu().numpy()), bits(od))
    sd, _ = s.query_silhouette(p, fl)
    osd, _ = orc.silhouette(p, fl)
    assert close_frac(sd.cpu().numpy(), osd) >= 0.999
    dirs = rng.standard_normal((n, 2)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    tm = np.exp(rng.uniform(np.log(1e-2), np.log(30), n)).astype(np.float32)
    h, t, sp, ri = s.query_ray(p, dirs, tm)
    oh, ot, osp, ori = orc.ray(p, dirs, tm)
    np.testing.assert_array_equal(h.cpu().numpy(), oh)
    np.testing.assert_array_equal(s.query_ray_test(p, dirs, tm).cpu().numpy(), oh)  # TestOnly = true
    np.testing.assert_array_equal(bits(t.cpu().numpy()), bits(ot))
    np.testing.assert_array_equal(ri.cpu().numpy().view(np.uint32), ori)
    rr = np.exp(rng.uniform(np.log(1e-2), np.log(3), n)).astype(np.float32)
    u = rng.random(n).astype(np.float32)
    si, spdf = s.sample_in_circle(p, rr, u)
    osi, opdf = orc.sample(p, rr, u)
    assert (si.cpu().numpy() == osi).mean() >= 0.99
    pts = s.sample_on_object(si.clamp(min=0), u)
    assert np.isfinite(pts.cpu().numpy()).all()
    assert s.device_status() == 0


def test_2d_errors(snch):
    with pytest.raises(snch.SnchError):
        snch.Scene2(np.zeros((2, 2), np.float32), np.array([[0, 2]], np.int32))
    s = snch.Scene2(np.zeros((2, 2), np.float32), np.array([[0, 1]], np.int32))
    with pytest.raises(snch.SnchError, match="BVH is not built yet."):
        s.query_nearest(np.zeros((1, 2), np.float32))
