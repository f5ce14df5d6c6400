"""Seeded searches (a per-query starting radius, then an unbounded pass for the
queries with nothing inside it) return exactly the unseeded results: radii
below, at and above the answer, tiny and huge, on the config-1 mesh and the
2M-triangle scene."""
import numpy as np
import pytest

from test_gpu_parity import bits, built_scene, check_edge_ids, check_tri_ids

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
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d0n))
    check_tri_ids(i1.cpu().numpy(), i0.cpu().numpy(), d0n, pts, v, f)
    expect = int(((r * r) < (d0n * d0n)).sum())  # nothing inside the radius: fallback
    assert int(nf.item()) == expect

    rs, _ = radii_mix(sd0n, rng)
    sd1, se1 = s.query_silhouette_seeded(pts, rs, flip, num_fallback=nf)
    np.testing.assert_array_equal(bits(sd1.cpu().numpy()), bits(sd0n))
    check_edge_ids(se1.cpu().numpy(), se0.cpu().numpy(), sd0n, pts, v, s.export_topology()[2])
    assert s.device_status() == 0


def test_seeded_reference_order_equals_unseeded():
    """The reference's own traversal order with a starting bound (the learned
    radius applied to the reference's algorithm) returns the unseeded
    reference-order results, including exact ties (vertex and edge-midpoint probes)."""
    import torch
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    rng = np.random.default_rng(8)
    v, f = meshes.noisy_icosphere(4, 1.0, 0.01, seed=0)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]]])
    mids = (0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])).astype(np.float32)
    pts = np.concatenate([meshes.box_queries(v, 60_000, 1.2, seed=5), v, mids]).astype(np.float32)
    flip = (rng.random(len(pts)) < 0.5).astype(np.uint8)
    s = built_scene(snch, v, f)
    s.set_traversal(snch.TRAVERSAL_REFERENCE_ORDER)
    i0, d0 = s.query_nearest(pts)
    sd0, se0 = s.query_silhouette(pts, flip)
    d0n, sd0n = d0.cpu().numpy(), sd0.cpu().numpy()
    nf = torch.zeros(1, dtype=torch.int32, device="cuda")
    r, _ = radii_mix(d0n, rng)
    i1, d1 = s.query_nearest_seeded(pts, r, num_fallback=nf)
    np.testing.assert_array_equal(i1.cpu().numpy(), i0.cpu().numpy())
    np.testing.assert_array_equal(bits(d1.cpu().numpy()), bits(d0n))
    assert int(nf.item()) == int(((r * r) < (d0n * d0n)).sum())
    rs, _ = radii_mix(sd0n, rng)
    sd1, se1 = s.query_silhouette_seeded(pts, rs, flip, num_fallback=nf)
    np.testing.assert_array_equal(bits(sd1.cpu().numpy()), bits(sd0n))
    np.testing.assert_array_equal(se1.cpu().numpy(), se0.cpu().numpy())
    s.set_traversal(snch.TRAVERSAL_NEAR_FIRST)
    i2, d2 = s.query_nearest(pts)
    np.testing.assert_array_equal(bits(d2.cpu().numpy()), bits(d0n))
    check_tri_ids(i2.cpu().numpy(), i0.cpu().numpy(), d0n, pts, v, f)
    assert s.device_status() == 0
