"""Device-memory reuse and the chunked host forms: a destroyed scene's arrays
are held for the next scene and give it the same answers; the *_host forms
split a batch into SNCH_OPT_HOST_CHUNK-sized chunks on two streams and their
outputs equal the device forms' for every chunk size (per-lane searches, whose
answers do not depend on the batch order); releasing the cache empties it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def snch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import snch_lbvh_gb300
    snch_lbvh_gb300.lib()
    return snch_lbvh_gb300


def mesh():
    from snch_lbvh_gb300 import meshes
    return meshes.noisy_torus(1.0, 0.35, 96, 48, 0.01, seed=3)


def queries(n, seed):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-1.6, 1.6, (n, 3)).astype(np.float32)
    flip = (rng.random(n) < 0.5).astype(np.uint8)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = np.full(n, np.inf, np.float32)
    r = rng.uniform(0.05, 0.6, n).astype(np.float32)
    u = rng.random(n).astype(np.float32)
    return pts, flip, d, tmax, r, u


def host_answers(s, q):
    pts, flip, d, tmax, r, u = q
    out = list(s.query_nearest_host(pts))
    out += list(s.query_silhouette_host(pts, flip))
    out += list(s.query_ray_host(pts, d, tmax))
    out += list(s.sample_in_sphere_host(pts, r, u))
    return [np.array(a) for a in out]


def device_answers(s, q):
    import torch
    pts, flip, d, tmax, r, u = (torch.from_numpy(a).cuda() for a in q)
    out = list(s.query_nearest(pts))
    out += list(s.query_silhouette(pts, flip))
    out += list(s.query_ray(pts, d, tmax))
    out += list(s.sample_in_sphere(pts, r, u))
    torch.cuda.synchronize()
    return [a.cpu().numpy() for a in out]


def same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(np.ascontiguousarray(x).view(np.uint8), np.ascontiguousarray(y).view(np.uint8))


def test_host_chunks_equal_device_forms(snch):
    v, t = mesh()
    s = snch.Scene(v, t)
    s.compute_silhouettes()
    s.build_bvh()
    s.set_option(snch.OPT_PACKET, 0)
    q = queries(70_001, seed=11)
    want = device_answers(s, q)
    for chunk in (1024, 4097, 65536, 1 << 24):
        s.set_option(snch.OPT_HOST_CHUNK, chunk)
        same(host_answers(s, q), want)
    with pytest.raises(snch.SnchError):
        s.set_option(snch.OPT_HOST_CHUNK, 100)
    assert s.device_status() == 0
    s.close()


def test_reused_blocks_give_the_same_answers(snch):
    v, t = mesh()
    q = queries(20_000, seed=12)
    snch.release_cached_memory()
    assert snch.cached_memory_bytes() == 0
    s = snch.Scene(v, t)
    s.compute_silhouettes()
    s.build_bvh()
    first = host_answers(s, q)
    s.close()
    held = snch.cached_memory_bytes()
    assert held > 0
    for _ in range(2):
        s = snch.Scene(v, t)
        assert snch.cached_memory_bytes() < held  # the new scene took the released blocks
        s.compute_silhouettes()
        s.build_bvh()
        same(host_answers(s, q), first)
        s.close()
    # a smaller scene next to a held larger one, then the larger one again
    from snch_lbvh_gb300 import meshes
    vs, ts, _ = meshes.icosphere(3)
    small = snch.Scene(vs, ts)
    small.compute_silhouettes()
    small.build_bvh()
    s = snch.Scene(v, t)
    s.build_bvh()
    same(host_answers(s, q), first)
    s.close()
    small.close()
    snch.release_cached_memory()
    assert snch.cached_memory_bytes() == 0


def test_options_read_back(snch):
    """snch_get_option returns what snch_set_option set, per query type."""
    v, t = mesh()
    s = snch.Scene(v, t)
    s.build_bvh()
    assert s.get_option(snch.OPT_HOST_CHUNK) == 0  # automatic per query type
    s.set_option(snch.OPT_HOST_CHUNK, 1 << 20)
    assert s.get_option(snch.OPT_HOST_CHUNK) == 1 << 20
    s.set_option(snch.OPT_PACKET_SILHOUETTE, 0)
    assert s.get_option(snch.OPT_PACKET_NEAREST) == 2 and s.get_option(snch.OPT_PACKET_SILHOUETTE) == 0
    s.set_option(snch.OPT_PERSISTENT_NEAREST, 1)
    assert s.search_config("nearest")[3] == 1 and s.search_config("silhouette")[3] == 0
    s.set_option(snch.OPT_NODE_WIDTH_SILHOUETTE, 4)
    assert s.search_config("silhouette")[0] == 4 and s.search_config("nearest")[0] == 2
    with pytest.raises(snch.SnchError):
        s.get_option(99)
    s.close()
