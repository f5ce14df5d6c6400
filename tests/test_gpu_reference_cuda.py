"""The reference's own CUDA queries (its headers compiled for sm_103a with its own
flags) against this library's kernels, query by query, over the same tree.

The reference's CUDA build contracts a*b+c into FMAs (nvcc's default); this
library does not, and equals the reference's uncontracted arithmetic bit for bit
(tests/test_gpu_parity.py). So the two differ only by rounding, and every query
must satisfy, with the float64 ground truth computed here:

* distances (nearest, silhouette): within RTOL relative or ATOL absolute;
* a differing triangle index / silhouette edge id: a tie -- the float64 distances
  of the two candidates differ by at most TIE, the resolution of float32 inputs
  of magnitude ~1 (checked for every differing query);
* rays: the same hit flag, or a float64 hit that lies within its float32 error
  bound of tmax or of the triangle's edges; the same triangle, or a float64 tie
  in t; t and (u, v) within twice the float32 forward-error bound of
  Moller-Trumbore for that ray (which grows as 1 / |det| for grazing rays) --
  with hit points within RTOL relative wherever the ray is well conditioned;
* sphere samples: the same triangle, or a float64 descent that passes within
  one unit of accumulated rounding of a branch probability (u against the left
  child's probability, rescaled at each level); pdfs within PDF_RTOL where the
  triangle is the same.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from test_gpu_parity import built_scene, seg_dist64, tri_dist64

pytestmark = pytest.mark.gpu

RTOL = 1e-6
ATOL = 2.5e-7          # two float32 ulps at unit coordinates
TIE = 1.1920928955078125e-07  # one float32 ulp at 1.0
PDF_RTOL = 1e-5
U32 = 2.0 ** -24       # float32 unit roundoff


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


def ray_f64(o, d, a, b, c):
    """float64 Moller-Trumbore (t, u, v) of rays against triangles, with the
    first-order float32 forward-error bounds of the reference's expression
    (scene.cuh:1005-1052): numerator and determinant are triple products whose
    float32 evaluation (rounded input differences, cross and dot products) errs
    by at most ~8u times the product of their operands' norms."""
    o, d, a, b, c = (np.asarray(x, np.float64) for x in (o, d, a, b, c))
    n = lambda x: np.linalg.norm(x, axis=1)
    e1, e2, s = b - a, c - a, o - a
    h, qv = np.cross(d, e2), np.cross(s, e1)
    det = np.einsum("ij,ij->i", e1, h)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.einsum("ij,ij->i", e2, qv) / det
        u = np.einsum("ij,ij->i", s, h) / det
        v = np.einsum("ij,ij->i", d, qv) / det
        den = n(e1) * n(d) * n(e2)
        bt = 8 * U32 * (n(e2) * n(s) * n(e1) + np.abs(t) * den) / np.abs(det) + 2 * U32 * np.abs(t)
        bu = 8 * U32 * (n(s) * n(d) * n(e2) + np.abs(u) * den) / np.abs(det) + 2 * U32 * np.abs(u)
        bv = 8 * U32 * (n(s) * n(e1) * n(d) + np.abs(v) * den) / np.abs(det) + 2 * U32 * np.abs(v)
    return t, u, v, bt, bu, bv


def sample_margins_f64(nodes, boxes, tris_n, c, r, u):
    """The descent of sample.cuh:26-91 in float64: for each draw the smallest
    distance between u and the left child's probability over the levels where
    both children can be taken, in units of the rounding u has accumulated
    (2^-24 per level times the product of the 1 / p rescalings so far)."""
    boxes = boxes.astype(np.float64)
    c, r, u = c.astype(np.float64), r.astype(np.float64), u.astype(np.float64).copy()
    n, ni = len(c), tris_n - 1
    node, live = np.zeros(n, np.int64), np.ones(n, bool)
    scale, margin = np.ones(n), np.full(n, np.inf)

    def box_hit(b, c, r):
        cl = np.maximum(b[:, 3:], np.minimum(c, b[:, :3]))
        return ((cl - c) ** 2).sum(1) <= r * r

    def green(b, c):
        return 1 / (4 * np.pi * np.maximum(np.linalg.norm(c - (b[:, :3] + b[:, 3:]) * 0.5, axis=1), 1e-4))

    for lvl in range(128):
        live &= node < ni
        k = np.nonzero(live)[0]
        if not len(k):
            break
        L, R = nodes[node[k], 1], nodes[node[k], 2]
        Lw = np.where(box_hit(boxes[L], c[k], r[k]), green(boxes[L], c[k]), 0.0)
        Rw = np.where(box_hit(boxes[R], c[k], r[k]), green(boxes[R], c[k]), 0.0)
        tw = Lw + Rw
        dead = ~(tw > 0)
        live[k[dead]] = False
        k, L, R, Lw, tw = k[~dead], L[~dead], R[~dead], Lw[~dead], tw[~dead]
        Lp = Lw / tw
        choice = (Lw > 0) & (Lp < 1)
        m = np.abs(u[k] - Lp) / (scale[k] * U32 * (lvl + 1))
        margin[k[choice]] = np.minimum(margin[k[choice]], m[choice])
        go_l = u[k] < Lp
        with np.errstate(divide="ignore", invalid="ignore"):
            u[k] = np.where(go_l, u[k] / Lp, (u[k] - Lp) / (1 - Lp))
            scale[k] *= np.where(go_l, 1 / Lp, 1 / (1 - Lp))
        node[k] = np.where(go_l, L, R)
    return margin


def check_per_query(ref, s, v, f, q, label):
    """Every query of every type against the reference's CUDA build (see the
    module docstring); returns the counts of explained differences."""
    import torch
    R = ref.RefQueries(s)
    d = {k: torch.from_numpy(np.ascontiguousarray(x)).cuda() for k, x in q.items()}
    stats = {}
    # nearest
    ri, rd = (x.cpu().numpy() for x in R.nearest(d["near_pts"]))
    mi, md = (x.cpu().numpy() for x in s.query_nearest(d["near_pts"]))
    assert close(rd, md).all(), (label, "nearest distance", np.abs(rd - md.astype(np.float64)).max())
    ri, mi = ri.view(np.uint32), mi.view(np.uint32)
    bad = np.nonzero(ri != mi)[0]
    if len(bad):
        p = q["near_pts"][bad]
        da = tri_dist64(p, v[f[ri[bad], 0]], v[f[ri[bad], 1]], v[f[ri[bad], 2]])
        db = tri_dist64(p, v[f[mi[bad], 0]], v[f[mi[bad], 1]], v[f[mi[bad], 2]])
        assert np.all(np.abs(da - db) <= TIE), (label, "nearest index not a tie", np.abs(da - db).max())
    stats["nearest_index_ties"] = len(bad)
    # silhouette, with the edge the reference's traversal ended on
    ev = s.export_topology()[2]
    rsd, rse = (x.cpu().numpy() for x in R.silhouette_edge(d["sil_pts"], d["sil_flip"]))
    msd, mse = (x.cpu().numpy() for x in s.query_silhouette(d["sil_pts"], d["sil_flip"]))
    assert close(rsd, msd).all(), (label, "silhouette distance")
    bad = np.nonzero(rse != mse)[0]
    if len(bad):
        assert np.all(rse[bad] >= 0) and np.all(mse[bad] >= 0), (label, "silhouette found by one build only")
        p = q["sil_pts"][bad]
        da = seg_dist64(p, v[ev[rse[bad], 1]], v[ev[rse[bad], 2]])
        db = seg_dist64(p, v[ev[mse[bad], 1]], v[ev[mse[bad], 2]])
        assert np.all(np.abs(da - db) <= TIE), (label, "silhouette edge not a tie", np.abs(da - db).max())
    stats["silhouette_edge_ties"] = len(bad)
    # rays
    rh, rt, ruv, rix = (x.cpu().numpy() for x in R.ray_uv(d["ray_o"], d["ray_d"], d["ray_tmax"]))
    mh, mt, muv, mix = (x.cpu().numpy() for x in s.query_ray(d["ray_o"], d["ray_d"], d["ray_tmax"]))
    rix, mix = rix.view(np.uint32), mix.view(np.uint32)
    o, dr, tm = q["ray_o"], q["ray_d"], q["ray_tmax"].astype(np.float64)
    one = np.nonzero(rh != mh)[0]
    for k in one:  # a hit in one build only: on the edge of a triangle or at tmax, within rounding
        ti = (rix if rh[k] else mix)[k]
        tri = f[ti]
        t, u, vv, bt, bu, bv = ray_f64(o[k:k + 1], dr[k:k + 1], v[tri[0]][None], v[tri[1]][None], v[tri[2]][None])
        near = (abs(t[0] - tm[k]) <= 2 * bt[0] or abs(u[0]) <= 2 * bu[0] or abs(vv[0]) <= 2 * bv[0]
                or abs(u[0] + vv[0] - 1) <= 2 * (bu[0] + bv[0]) or abs(t[0]) <= 2 * bt[0])
        assert near, (label, "ray hit flag differs away from any boundary", k)
    stats["ray_hit_flips"] = len(one)
    both = np.nonzero((rh == 1) & (mh == 1))[0]
    other = both[rix[both] != mix[both]]
    for k in other:
        ta = ray_f64(o[k:k + 1], dr[k:k + 1], *(v[f[rix[k], i]][None] for i in range(3)))
        tb = ray_f64(o[k:k + 1], dr[k:k + 1], *(v[f[mix[k], i]][None] for i in range(3)))
        assert abs(ta[0][0] - tb[0][0]) <= 2 * (ta[3][0] + tb[3][0]), (label, "ray triangle not a tie in t", k)
    stats["ray_triangle_ties"] = len(other)
    same = both[rix[both] == mix[both]]
    tri = f[mix[same]]
    t64, u64, v64, bt, bu, bv = ray_f64(o[same], dr[same], v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]])
    dt = np.abs(rt[same].astype(np.float64) - mt[same])
    assert np.all(dt <= 2 * bt), (label, "ray t beyond the float32 bound", (dt / (2 * bt)).max())
    assert np.all(np.abs(ruv[same, 0].astype(np.float64) - muv[same, 0]) <= 2 * bu), (label, "ray u")
    assert np.all(np.abs(ruv[same, 1].astype(np.float64) - muv[same, 1]) <= 2 * bv), (label, "ray v")
    hp = o[same].astype(np.float64) + mt[same, None].astype(np.float64) * dr[same]
    rel = dt * np.linalg.norm(dr[same], axis=1) / np.maximum(np.linalg.norm(hp, axis=1), 1e-30)
    stats["ray_hit_point_beyond_rtol"] = int((rel > RTOL).sum())  # all ill-conditioned (inside the bound)
    # sphere samples
    rsi, rsp = (x.cpu().numpy() for x in R.sample(d["smp_c"], d["smp_r"], d["smp_u"]))
    msi, msp = (x.cpu().numpy() for x in s.sample_in_sphere(d["smp_c"], d["smp_r"], d["smp_u"]))
    flips = np.nonzero(rsi != msi)[0]
    if len(flips):
        tr = s.export_tree()
        m = sample_margins_f64(tr["nodes"], tr["aabbs"], len(f), q["smp_c"][flips], q["smp_r"][flips],
                               q["smp_u"][flips])
        assert np.all(m <= 1.0), (label, "sample index differs away from a branch boundary", m.max())
    stats["sample_branch_flips"] = len(flips)
    ok = (rsi == msi) & (msi >= 0)
    assert np.all(np.abs(rsp[ok].astype(np.float64) - msp[ok]) <= PDF_RTOL * msp[ok]), (label, "sample pdf")
    print(label, stats)
    return stats


def test_reference_cuda_per_query_config1(ref):
    """Config 1 (20,480-triangle noisy icosphere), queries in its box x 1.2."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    q = meshes.wost_queries(200_000, 100_000, 200_000, 100_000, seed=12)
    for k in ("near_pts", "sil_pts", "ray_o", "smp_c"):
        q[k] = (q[k] * 2.4 - 1.2).astype(np.float32)
    q["sil_flip"] = (np.arange(len(q["sil_pts"])) % 2).astype(np.uint8)
    check_per_query(ref, built_scene(snch, v, f), v, f, q, "config1")


def test_reference_cuda_per_query_wost_scene(ref):
    """The 1,993,600-triangle scene: 500k nearest, 300k silhouette, 500k ray and
    500k sphere-sample queries of the walk-on-stars distributions."""
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    q = meshes.wost_queries(500_000, 300_000, 500_000, 500_000, seed=41)
    check_per_query(ref, built_scene(snch, sc.verts, sc.faces), sc.verts, sc.faces, q, "wost_2m")


@pytest.mark.parametrize("name", [n for n in golden_names() if n not in ("single_tri", "degenerate")])
def test_reference_cuda_per_query_golden(ref, name):
    """The golden inputs, built to sit on ties (vertices, edge midpoints, face
    centres): every query of every type meets the per-query criteria. (The
    degenerate golden mesh's zero-area triangles make the closest-point
    arithmetic ill-conditioned under FMA contraction; there the reference's CUDA
    build is compared with the reference's own CPU results in
    test_reference_cuda_degenerate_mesh.)"""
    import snch_lbvh_gb300 as snch
    g = load_golden(name)
    v, f = g["verts"], g["tris"]
    rng = np.random.default_rng(len(f))
    lo, hi = v.min(0), v.max(0)
    box = lambda n: (lo - 0.1 + (hi - lo + 0.2) * rng.random((n, 3))).astype(np.float32)
    d = rng.standard_normal((4096, 3)).astype(np.float32)
    q = {"near_pts": g["near_pts"], "sil_pts": g["sil_pts"], "sil_flip": g["sil_flip"],
         "ray_o": box(4096), "ray_d": (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32),
         "ray_tmax": np.full(4096, 4 * float((hi - lo).max()) + 1, np.float32),
         "smp_c": box(4096), "smp_r": rng.uniform(0.01, float((hi - lo).max()) + 0.1, 4096).astype(np.float32),
         "smp_u": rng.random(4096, dtype=np.float32)}
    check_per_query(ref, built_scene(snch, v, f), v, f, q, name)


def test_reference_cuda_degenerate_mesh(ref):
    """On the golden mesh with zero-area triangles, the reference's CUDA build
    disagrees with the reference's own uncontracted CPU results exactly where it
    disagrees with ours: ours ARE those results."""
    import torch
    import snch_lbvh_gb300 as snch
    g = load_golden("degenerate")
    s = built_scene(snch, g["verts"], g["tris"])
    R = ref.RefQueries(s)
    pts = torch.from_numpy(g["near_pts"]).cuda()
    _, rd = R.nearest(pts)
    _, md = s.query_nearest(pts)
    ours = md.cpu().numpy()
    np.testing.assert_array_equal(ours.view(np.uint32), g["ref_near_dist"].view(np.uint32))
    np.testing.assert_array_equal(close(rd.cpu().numpy(), g["ref_near_dist"]), close(rd.cpu().numpy(), ours))


def test_reference_cuda_on_oracle_built_tree(ref, oracle_mod):
    """The reference arm's tree (oracle/ref_gpu.py RefTree: built by the CPU
    restatement, uploaded in the reference's device layout, no code of this
    library) gives the reference's CUDA queries the answers they give over this
    library's byte-compatible view: the two trees are equal bit for bit except
    where CUDA's transcendental functions enter the cones."""
    import torch
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    q = meshes.wost_queries(100_000, 100_000, 100_000, 100_000, seed=13)
    for k in ("near_pts", "sil_pts", "ray_o", "smp_c"):
        q[k] = (q[k] * 2.4 - 1.2).astype(np.float32)
    d = {k: torch.from_numpy(np.ascontiguousarray(x)).cuda() for k, x in q.items()}
    a = ref.RefQueries(ref.RefTree(oracle_mod.Tree(v, f)))
    b = ref.RefQueries(built_scene(snch, v, f))
    for x, y in zip(a.nearest(d["near_pts"]), b.nearest(d["near_pts"])):
        np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32), y.cpu().numpy().view(np.uint32))
    ra = [x.cpu().numpy() for x in a.ray_uv(d["ray_o"], d["ray_d"], d["ray_tmax"])]
    rb = [x.cpu().numpy() for x in b.ray_uv(d["ray_o"], d["ray_d"], d["ray_tmax"])]
    for k in (0, 1, 3):  # hit, t, triangle
        np.testing.assert_array_equal(ra[k].view(np.uint8), rb[k].view(np.uint8))
    hit = ra[0] == 1  # the reference leaves (u, v) unset on a miss
    np.testing.assert_array_equal(ra[2][hit].view(np.uint32), rb[2][hit].view(np.uint32))
    for x, y in zip(a.sample(d["smp_c"], d["smp_r"], d["smp_u"]), b.sample(d["smp_c"], d["smp_r"], d["smp_u"])):
        np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32), y.cpu().numpy().view(np.uint32))
    sa = a.silhouette(d["sil_pts"], d["sil_flip"]).cpu().numpy()
    sb = b.silhouette(d["sil_pts"], d["sil_flip"]).cpu().numpy()
    assert np.mean(sa.view(np.uint32) == sb.view(np.uint32)) >= 0.999
