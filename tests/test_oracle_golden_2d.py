"""The 2D oracle (scene<2>: line segments, silhouette vertices) against the
reference's own outputs (tests/golden/2d/, written by tests/golden/make_golden.py
from the unmodified reference headers): topology, Morton codes, tree, boxes bit
for bit; cones bit for bit except where the reference leaves a merged cone
undefined (cone.cuh:347-351) and their ancestors; the four queries bit for bit."""
import glob
import os

import numpy as np
import pytest

from conftest import d1_tainted

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(ROOT, "tests", "golden", "2d", "*.npz")))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def load2(name):
    with np.load(os.path.join(ROOT, "tests", "golden", "2d", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module", params=NAMES)
def case2(request, oracle_mod):
    g = load2(request.param)
    return request.param, g, oracle_mod.Tree2(g["verts"], g["segs"])


def test_2d_topology_and_tree(case2):
    _, g, t = case2
    np.testing.assert_array_equal(t.sv, g["ref_sv"])
    np.testing.assert_array_equal(t.seg_owned, g["ref_seg_owned"])
    np.testing.assert_array_equal(t.morton, g["ref_morton"])
    np.testing.assert_array_equal(t.nodes, g["ref_nodes"])
    np.testing.assert_array_equal(bits(t.aabbs), bits(g["ref_aabbs"]))
    ref = g["ref_cones"]
    taint = d1_tainted(t.nodes, t.d1)
    valid = ref[:, 2] >= 0
    np.testing.assert_array_equal((t.cones[:, 2] >= 0)[~taint], valid[~taint])
    exact = valid & ~taint
    np.testing.assert_array_equal(bits(t.cones[exact]), bits(ref[exact]))
    # invalid cones: only the half-angle (-pi) is defined in the reference (a
    # merge of two invalid cones leaves axis and radius unset, cone.cuh:364-367)
    inv = ~valid & ~taint
    np.testing.assert_array_equal(bits(t.cones[inv, 2]), bits(ref[inv, 2]))
    assert np.all(t.cones[t.d1.astype(bool), 2] == np.float32(np.pi))


def test_2d_queries(case2):
    name, g, t = case2
    if len(g["ref_near_idx"]) == 0:
        pytest.skip("one segment: the reference reads past its node array")
    i, d = t.nearest(g["near_pts"])
    np.testing.assert_array_equal(i, g["ref_near_idx"])
    np.testing.assert_array_equal(bits(d), bits(g["ref_near_dist"]))
    sd, _ = t.silhouette(g["sil_pts"], g["sil_flip"])
    np.testing.assert_array_equal(bits(sd), bits(g["ref_sil_dist"]))
    h, tt, sp, ri = t.ray(g["ray_o"], g["ray_d"], g["ray_tmax"])
    np.testing.assert_array_equal(h, g["ref_ray_hit"])
    np.testing.assert_array_equal(bits(tt), bits(g["ref_ray_t"]))
    np.testing.assert_array_equal(bits(sp), bits(g["ref_ray_s"]))
    np.testing.assert_array_equal(ri, g["ref_ray_idx"])
    si, spdf = t.sample(g["smp_c"], g["smp_r"], g["smp_u"])
    np.testing.assert_array_equal(si, g["ref_smp_idx"])
    np.testing.assert_array_equal(bits(spdf), bits(g["ref_smp_pdf"]))
