"""The reference's own CUDA queries (its headers compiled for sm_103a with its own
flags) run over a tree built by this library through the byte-compatible
snch_bvh_view, and agree with this library's kernels.

The reference compiles with nvcc's default FMA contraction, this library
without it (and bit-exactly equal to the reference's uncontracted arithmetic,
tests/test_gpu_parity.py), so floats agree to within RTOL relative or ATOL
absolute (two float32 ulps at unit coordinates; near-surface distances of
~0.01 differ by 1-3e-8 between the two builds), and indices agree except
where two candidates' distances are that close.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import built_scene

pytestmark = pytest.mark.gpu

RTOL = 1e-6
ATOL = 2.5e-7


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_gpu
    ok, why = ref_gpu.available()
    if not ok:
        pytest.skip(why)
    ref_gpu.lib()
    return ref_gpu


def close(a, b, rtol=RTOL, atol=ATOL):
    a, b = a.astype(np.float64), b.astype(np.float64)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    with np.errstate(invalid="ignore"):  # inf - inf where both are infinite
        return both_inf | (np.abs(a - b) <= np.maximum(rtol * np.abs(b), atol))


def compare_all(snch, ref, s, q, min_agree=0.999):
    """Ours vs the reference's CUDA build over the same tree; returns agreement rates."""
    import torch
    R = ref.RefQueries(s)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in q.items() if not k.startswith("_")}
    ri, rd = R.nearest(d["near_pts"])
    mi, md = s.query_nearest(d["near_pts"])
    rd, md = rd.cpu().numpy(), md.cpu().numpy()
    rates = {"near_dist": close(rd, md).mean()}
    # indices: equal, or an exact tie that the two builds' rounding breaks differently
    ri, mi = ri.cpu().numpy().view(np.uint32), mi.cpu().numpy().view(np.uint32)
    diff = np.nonzero(ri != mi)[0]
    rates["near_idx"] = 1.0 - len(diff) / len(ri)
    if len(diff):
        from oracle import oracle
        v, f = q["_verts"], q["_tris"]
        pts = q["near_pts"][diff]
        explained = 0
        for k in range(min(len(diff), 256)):
            _, da = oracle.brute_nearest_f64(v, f[ri[diff[k]]][None], pts[k][None])
            _, db = oracle.brute_nearest_f64(v, f[mi[diff[k]]][None], pts[k][None])
            explained += abs(da[0] - db[0]) <= max(RTOL * db[0], ATOL)
        rates["near_idx_ties_explained"] = explained / min(len(diff), 256)
    rs = R.silhouette(d["sil_pts"], d["sil_flip"]).cpu().numpy()
    ms = s.query_silhouette(d["sil_pts"], d["sil_flip"])[0].cpu().numpy()
    rates["sil_dist"] = close(rs, ms).mean()
    rh, rt, rr = R.ray(d["ray_o"], d["ray_d"], d["ray_tmax"])
    mh, mt, _, mr = s.query_ray(d["ray_o"], d["ray_d"], d["ray_tmax"])
    hit_same = rh.cpu().numpy() == mh.cpu().numpy()
    rates["ray_hit"] = hit_same.mean()
    both = (rh.cpu().numpy() == 1) & hit_same
    rates["ray_t"] = close(rt.cpu().numpy()[both], mt.cpu().numpy()[both]).mean() if both.any() else 1.0
    rsi, rsp = R.sample(d["smp_c"], d["smp_r"], d["smp_u"])
    msi, msp = s.sample_in_sphere(d["smp_c"], d["smp_r"], d["smp_u"])
    rates["sample_idx"] = (rsi.cpu().numpy() == msi.cpu().numpy()).mean()
    torch.cuda.synchronize()
    return rates


@pytest.mark.parametrize("name", [n for n in golden_names() if n not in ("single_tri",)])
def test_reference_cuda_runs_on_our_tree_golden(ref, name):
    """On the golden inputs (built to sit on ties: vertices, edge midpoints,
    face centres) the reference's CUDA build disagrees with the reference's own
    uncontracted results exactly as much as it disagrees with ours, because ours
    ARE those results (tests/test_gpu_parity.py)."""
    import torch
    import snch_lbvh_gb300 as snch
    g = load_golden(name)
    s = built_scene(snch, g["verts"], g["tris"])
    R = ref.RefQueries(s)
    pts = torch.from_numpy(g["near_pts"]).cuda()
    ri, rd = R.nearest(pts)
    mi, md = s.query_nearest(pts)
    ours = md.cpu().numpy()
    np.testing.assert_array_equal(ours.view(np.uint32), g["ref_near_dist"].view(np.uint32))
    agree_ref_cpu = close(rd.cpu().numpy(), g["ref_near_dist"]).mean()
    agree_ours = close(rd.cpu().numpy(), ours).mean()
    assert agree_ours == agree_ref_cpu
    if name != "degenerate":  # zero-area triangles are ill-conditioned under FMA contraction
        assert agree_ours >= 0.99, agree_ours
    sil_ref_cuda = R.silhouette(torch.from_numpy(g["sil_pts"]).cuda(), torch.from_numpy(g["sil_flip"]).cuda())
    assert close(sil_ref_cuda.cpu().numpy(), g["ref_sil_dist"]).mean() >= 0.95


def test_reference_cuda_runs_on_our_tree_config1(ref):
    """Random queries (no engineered ties) on the config-1 mesh."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    q = meshes.wost_queries(200_000, 100_000, 200_000, 100_000, seed=12)
    for k in ("near_pts", "sil_pts", "ray_o", "smp_c"):
        q[k] = (q[k] * 2.4 - 1.2).astype(np.float32)
    s = built_scene(snch, v, f)
    q["_verts"], q["_tris"] = v, f
    r = compare_all(snch, ref, s, q)
    assert r["near_dist"] >= 0.999, r
    assert r["near_idx"] >= 0.98 and r.get("near_idx_ties_explained", 1.0) == 1.0, r
    assert r["sil_dist"] >= 0.995, r
    assert r["ray_hit"] >= 0.999 and r["ray_t"] >= 0.999, r
    assert r["sample_idx"] >= 0.999, r
