"""Seeded workload generators: sizes, orientation, determinism, ranges."""
import numpy as np

from snch_lbvh_gb300 import meshes


def test_icosphere_counts_and_orientation():
    for level in range(4):
        v, f, _ = meshes.icosphere(level)
        assert len(f) == 20 * 4 ** level and len(v) == 10 * 4 ** level + 2
        a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
        n = np.cross(b - a, c - a)
        assert np.all((n * (a + b + c)).sum(1) > 0), "faces must be counter-clockwise seen from outside"


def test_config1_mesh():
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    assert v.dtype == np.float32 and f.dtype == np.int32
    assert f.shape == (20480, 3) and v.shape == (10242, 3)
    r = np.linalg.norm(v.astype(np.float64), axis=1)
    assert 0.95 < r.min() and r.max() < 1.05 and 0.005 < r.std() < 0.015
    v2, _ = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    np.testing.assert_array_equal(v, v2)


def test_torus_closed_and_outward():
    v, f, nrm = meshes.torus(0.4, 0.1, 24, 12)
    assert f.shape == (2 * 24 * 12, 3)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2), "torus must be a closed 2-manifold"
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    assert np.all((np.cross(b - a, c - a) * nrm[f[:, 0]]).sum(1) > 0)


def test_wost_scene_size_and_placement():
    s = meshes.wost_scene(seed=0, n_meshes=4, torus_nu=20, torus_nv=10, ico_level=2)
    assert len(s.mesh_offsets) == 5 and s.mesh_offsets[-1] == len(s.faces)
    assert len(s.faces) == 2 * 320 + 2 * 400
    assert s.face_flags.dtype == np.uint8 and set(np.unique(s.face_flags)) <= {0, 1}
    assert s.faces.max() < len(s.verts)
    full = meshes.WOST_MESHES // 2 * (20 * 4 ** meshes.WOST_ICO_LEVEL) + \
        meshes.WOST_MESHES // 2 * (2 * meshes.WOST_TORUS_NU * meshes.WOST_TORUS_NV)
    assert abs(full - 2_000_000) <= 20_000


def test_wost_queries_ranges():
    q = meshes.wost_queries(1000, 1000, 1000, 500, seed=3)
    assert q["near_pts"].shape == (1000, 3) and q["near_pts"].min() >= 0 and q["near_pts"].max() < 1
    np.testing.assert_allclose(np.linalg.norm(q["ray_d"], axis=1), 1, rtol=1e-6)
    assert q["ray_tmax"].min() >= 1e-3 * 0.999 and q["ray_tmax"].max() <= 1.0
    assert q["smp_r"].min() >= 1e-3 * 0.999 and q["smp_r"].max() <= 0.5 * 1.0001
    assert q["smp_u"].min() >= 0 and q["smp_u"].max() < 1
