"""The CPU oracle against the reference's own outputs (tests/golden/, written by
tests/golden/make_golden.py from the unmodified reference headers).

Bit-exact everywhere except cone fields the reference leaves uninitialised:
the axis/radius of a merge of two invalid cones (cone.cuh:474-477) and the
half-angle where o_theta >= pi (cone.cuh:454-458, plus every ancestor of such
a node, whose cone depends on that undefined value).
"""
import numpy as np
import pytest

from conftest import d1_tainted, golden_names, load_golden


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module", params=golden_names())
def case(request, oracle_mod):
    g = load_golden(request.param)
    return request.param, g, oracle_mod.Tree(g["verts"], g["tris"])


def test_topology(case):
    _, g, t = case
    np.testing.assert_array_equal(t.tri_edges, g["ref_tri_edges"])
    np.testing.assert_array_equal(t.tri_owned, g["ref_tri_owned"])
    np.testing.assert_array_equal(t.edge_verts, g["ref_edge_verts"])


def test_morton_and_tree(case):
    _, g, t = case
    np.testing.assert_array_equal(t.morton, g["ref_morton"])
    np.testing.assert_array_equal(t.nodes, g["ref_nodes"])
    np.testing.assert_array_equal(bits(t.aabbs), bits(g["ref_aabbs"]))
    n = len(t.tris)
    np.testing.assert_array_equal(t.sorted_idx, g["ref_nodes"][n - 1:, 3])


def test_cones(case):
    name, g, t = case
    ref = g["ref_cones"]
    taint = d1_tainted(t.nodes, t.d1)
    valid = ref[:, 3] >= 0
    np.testing.assert_array_equal((t.cones[:, 3] >= 0)[~taint], valid[~taint])
    assert np.all(t.cones[taint, 3] >= 0)
    exact = valid & ~taint
    np.testing.assert_array_equal(bits(t.cones[exact]), bits(ref[exact]))
    # invalid cones: only the half-angle (-pi) is defined in the reference
    inv = ~valid & ~taint
    np.testing.assert_array_equal(bits(t.cones[inv, 3]), bits(ref[inv, 3]))
    # where the reference is undefined the oracle stores the conservative pi
    assert np.all(t.cones[t.d1.astype(bool), 3] == np.float32(np.pi))


def test_nearest(case):
    _, g, t = case
    if len(g["ref_near_idx"]) == 0:
        pytest.skip("the reference's nearest query reads past a one-node tree")
    idx, dist = t.nearest(g["near_pts"])
    np.testing.assert_array_equal(idx, g["ref_near_idx"])
    np.testing.assert_array_equal(bits(dist), bits(g["ref_near_dist"]))


def test_silhouette(case):
    _, g, t = case
    if len(g["ref_sil_dist"]) == 0:
        pytest.skip("the reference's silhouette query reads past a one-node tree")
    dist, _ = t.silhouette(g["sil_pts"], g["sil_flip"])
    np.testing.assert_array_equal(bits(dist), bits(g["ref_sil_dist"]))


def test_ray(case):
    _, g, t = case
    hit, tt, uv, idx = t.ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
    np.testing.assert_array_equal(hit, g["ref_ray_hit"])
    np.testing.assert_array_equal(bits(tt), bits(g["ref_ray_t"]))
    np.testing.assert_array_equal(bits(uv), bits(g["ref_ray_uv"]))
    np.testing.assert_array_equal(idx, g["ref_ray_idx"])


def test_sample(case):
    _, g, t = case
    idx, pdf = t.sample(g["smp_c"], g["smp_r"], g["smp_u"])
    np.testing.assert_array_equal(idx, g["ref_smp_idx"])
    np.testing.assert_array_equal(bits(pdf), bits(g["ref_smp_pdf"]))
    pts = t.sample_on_object(g["obj_idx"], g["obj_u"], g["obj_v"])
    np.testing.assert_array_equal(bits(pts), bits(g["ref_obj_pts"]))


def test_golden_cases_cover_edge_cases():
    """The fixture set holds the cases the reference's code paths branch on."""
    names = set(golden_names())
    assert {"tetra", "single_tri", "two_tri", "open_grid", "duplicated", "degenerate",
            "cfg1_icosphere_l5"} <= names
    dup = load_golden("duplicated")
    codes = dup["ref_morton"]
    assert len(np.unique(codes)) < len(codes), "duplicated case must force the 64-bit key path"
    grid = load_golden("open_grid")
    assert np.any(grid["ref_edge_verts"][:, 0] == -1) or np.any(grid["ref_edge_verts"][:, 3] == -1)


def test_overlap_enumeration(case):
    """query_device(overlaps(box)) query.cuh:177-231: the same triangles in the
    same order, and the same total count, as the reference."""
    name, g, t = case
    if len(g["ref_box_count"]) == 0:
        pytest.skip("one-triangle tree: the reference reads past its node array")
    k = g["ref_box_idx"].shape[1]
    idx, cnt = t.overlap(g["box_q"], k)
    np.testing.assert_array_equal(cnt, g["ref_box_count"])
    np.testing.assert_array_equal(idx, g["ref_box_idx"])


def test_line_enumeration(case):
    """query_device(line_intersect(line), element_test) query.cuh:15-77 with the
    triangle test of intersect_test for a line: triangles, line parameters and
    counts bit for bit, in the reference's order."""
    name, g, t = case
    if len(g["ref_line_count"]) == 0:
        pytest.skip("one-triangle tree: the reference reads past its node array")
    k = g["ref_line_idx"].shape[1]
    idx, tt, cnt = t.line(g["line_o"], g["line_d"], k)
    np.testing.assert_array_equal(cnt, g["ref_line_count"])
    np.testing.assert_array_equal(idx, g["ref_line_idx"])
    np.testing.assert_array_equal(bits(tt), bits(g["ref_line_t"]))
