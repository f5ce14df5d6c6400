"""Walk-on-stars driver: the walks estimate the harmonic u(x) = x_0 without
bias beyond the epsilon shell, and seeding the distance queries with a
learned radius leaves every walk (so every estimate) bit for bit unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere_scenes():
    import snch_lbvh_gb300 as snch  # noqa: F401
    from snch_lbvh_gb300 import meshes, wost
    v, f = meshes.noisy_icosphere(4, 1.0, 0.002, seed=3)
    flags = (np.random.default_rng(4).random(len(f)) < 0.5).astype(np.uint8)
    return v, f, flags, wost.split_boundary(v, f, flags)


def check_unbiased(est, start, stats, n, eps):
    e, x0 = est.cpu().numpy().astype(np.float64), start.cpu().numpy()[:, 0].astype(np.float64)
    err = e - x0
    assert np.all(np.isfinite(e))
    se = err.std() / np.sqrt(n)
    assert abs(err.mean()) < 5 * se + 3 * eps, (err.mean(), se)
    assert stats["terminated"] >= 0.97 * n, stats["terminated"]
    live = stats["live"]
    assert live[0] == n and all(a >= b for a, b in zip(live, live[1:]))


def test_wost_dirichlet_only_is_walk_on_spheres(sphere_scenes):
    """All faces Dirichlet: the estimate is x_0 of the exit point."""
    from snch_lbvh_gb300 import wost
    v, f, _, _ = sphere_scenes
    d, nsc = wost.split_boundary(v, f, np.zeros(len(f), np.uint8))
    n, eps = 100_000, 1e-3
    est, start, stats = wost.trace(d, nsc, n, epsilon=eps, seed=1)
    check_unbiased(est, start, stats, n, eps)


def test_wost_mixed_boundary_unbiased(sphere_scenes):
    from snch_lbvh_gb300 import wost
    _, _, _, (d, nsc) = sphere_scenes
    n, eps = 200_000, 1e-3
    est, start, stats = wost.trace(d, nsc, n, epsilon=eps, seed=2)
    check_unbiased(est, start, stats, n, eps)
    assert d.device_status() == 0 and nsc.device_status() == 0


def test_wost_learned_radius_same_walks(sphere_scenes):
    import torch
    from snch_lbvh_gb300 import wost
    from snch_lbvh_gb300.learned import LearnedRadius, training_points
    v, f, flags, (d, nsc) = sphere_scenes
    pts = torch.from_numpy(training_points(v, f, 200_000, 200_000, 0.05, lo=(-1, -1, -1), hi=(1, 1, 1),
                                           seed=5)).cuda()
    _, dd = d.query_nearest(pts)
    ds, _ = nsc.query_silhouette(pts)
    t = torch.stack([dd, ds], 1)
    t = torch.log(torch.where(torch.isfinite(t) & (t > 0), t, torch.full_like(t, float("nan"))))
    m = LearnedRadius(np.full(3, -1.05), np.full(3, 1.05), seed=2)
    m.train(pts, t, epochs=4, batch=32768, lr=2e-3, tau=0.9)
    n = 100_000
    e0, s0, st0 = wost.trace(d, nsc, n, seed=7)
    e1, s1, st1 = wost.trace(d, nsc, n, seed=7, model=m, margin=1.5)
    np.testing.assert_array_equal(e0.cpu().numpy().view(np.uint32), e1.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(s0.cpu().numpy(), s1.cpu().numpy())
    assert st0["live"] == st1["live"] and st0["terminated"] == st1["terminated"]
    assert sum(st1["fallback"]) < 0.5 * sum(st1["live"]) * 2
