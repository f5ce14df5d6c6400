"""snch_obj_read against the reference's own OBJ reader (scene_loader<3>,
scene_loader.cuh:86-152, run on tests/golden/obj/torus.obj by
tests/golden/make_golden.py): the same vertices bit for bit and the same
triangles; plus the forms the reference cannot read (v/vt/vn face tokens),
missing files and empty files. Host code only: no GPU needed."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OBJ_DIR = os.path.join(ROOT, "tests", "golden", "obj")


def test_obj_matches_reference_reader():
    import snch_lbvh_gb300 as snch
    v, t = snch.read_obj(os.path.join(OBJ_DIR, "torus.obj"))
    with np.load(os.path.join(OBJ_DIR, "torus_ref.npz")) as r:
        np.testing.assert_array_equal(v.view(np.uint32), r["ref_verts"].view(np.uint32))
        np.testing.assert_array_equal(t, r["ref_tris"])


def test_obj_slash_tokens_and_edge_cases(tmp_path):
    import snch_lbvh_gb300 as snch
    p = tmp_path / "m.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvt 0 0\nvn 0 0 1\n"
                 "f 1/1/1 2/1/1 3/1/1\nf 1//1 3//1 4//1\nf 2 3 4 1\n\n# end")
    v, t = snch.read_obj(str(p))
    assert v.shape == (4, 3) and np.array_equal(v[3], [0, 0, 1])
    np.testing.assert_array_equal(t, [[0, 1, 2], [0, 2, 3], [1, 2, 3]])
    p.write_text("")
    v, t = snch.read_obj(str(p))
    assert v.shape == (0, 3) and t.shape == (0, 3)
    with pytest.raises(snch.SnchError, match="Could not open .obj file."):
        snch.read_obj(str(tmp_path / "missing.obj"))
