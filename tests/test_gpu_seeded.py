"""Seeded searches (a per-query starting radius, then an unbounded pass for the
queries with nothing inside it) return exactly the unseeded results: radii
below, at and above the answer, tiny and huge, on the config-1 mesh and the
2M-triangle scene."""
import numpy as np
import pytest

from test_gpu_parity import bits, built_scene

pytestmark = pytest.mark.gpu


def radii_mix(true_d, rng):
    """below (fallback), exactly at, slightly above, far above, and tiny."""
    kind = rng.integers(0, 5, len(true_d))
    r = np.where(kind == 0, true_d * 0.5, true_d)
    r = np.where(kind == 2, true_d * np.float32(1.1) + np.float32(1e-4), r)
    r = np.where(kind == 3, np.float32(10.0), r)
    r = np.where(kind == 4, np.float32(1e-7), r)
    r = np.where(np.isfinite(r), r, np.float32(1.0))
    return r.astype(np.float32), kind


@pytest.mark.parametrize("mesh", ["config1", "wost_small"])
def test_seeded_equals_unseeded(mesh):
    import torch
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    rng = np.random.default_rng(3)
    if mesh == "config1":
        v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
        pts = meshes.box_queries(v, 300_000, 1.2, seed=4)
    else:
        sc = meshes.wost_scene(seed=2, n_meshes=8, torus_nu=60, torus_nv=30, ico_level=4)
        v, f = sc.verts, sc.faces
        pts = rng.random((300_000, 3), dtype=np.float32)
    s = built_scene(snch, v, f)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    i0, d0 = s.query_nearest(pts)
    sd0, se0 = s.query_silhouette(pts, flip)
    d0n, sd0n = d0.cpu().numpy(), sd0.cpu().numpy()

    r, kind = radii_mix(d0n, rng)
    nf = torch.zeros(1, dtype=torch.int32, device="cuda")
    i1, d1 = s.query_nearest_seeded(pts, r, num_fallback=nf)
    np.testing.assert_array_equal(i1.cpu().numpy(), i0.cpu().numpy())
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d0n))
    expect = int(((r * r) < (d0n * d0n)).sum())  # nothing inside the radius: fallback
    assert int(nf.item()) == expect

    rs, _ = radii_mix(sd0n, rng)
    sd1, se1 = s.query_silhouette_seeded(pts, rs, flip, num_fallback=nf)
    np.testing.assert_array_equal(bits(sd1.cpu().numpy()), bits(sd0n))
    np.testing.assert_array_equal(se1.cpu().numpy(), se0.cpu().numpy())
    assert s.device_status() == 0
