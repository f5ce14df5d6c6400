"""The FP64 restatement of the learned-radius MLP (oracle/mlp_oracle.py):
its analytic gradient against central finite differences, and its feature
frequencies against the package's."""
import numpy as np

from oracle import mlp_oracle as mo


def random_params(rng):
    p = []
    for s in mo.SIZES:
        fan_in = s[1] if len(s) == 2 else 64
        p.append(rng.uniform(-1, 1, s) * np.sqrt(6.0 / fan_in))
    return np.concatenate([x.reshape(-1) for x in p])


def test_num_params_and_scales():
    from snch_lbvh_gb300.learned import NUM_FREQ, feature_scales
    assert sum(int(np.prod(s)) for s in mo.SIZES) == 24962
    assert NUM_FREQ == mo.FREQ
    s = feature_scales()
    assert s.dtype == np.float32 and s[0] == 1.0 and s[4] == 2.0 and s[31] == np.float32(2 ** 7.75)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    lo, hi = np.zeros(3, np.float32), np.ones(3, np.float32)
    pts = rng.random((64, 3)).astype(np.float32)
    params = random_params(rng)
    o, _ = mo.forward(params, pts, lo, hi, emulate_bf16=False)
    targets = o + rng.normal(0, 0.5, o.shape)  # residuals well away from the pinball kink
    targets[::7, 1] = np.nan
    tau = 0.2
    loss, g = mo.loss_and_grad(params, pts, targets, lo, hi, tau, emulate_bf16=False)
    assert np.isfinite(loss) and g.shape == params.shape
    eps = 1e-6
    idx = np.concatenate([rng.choice(len(params), 200, replace=False), np.arange(len(params) - 130, len(params))])
    fd = []
    for i in idx:
        pp, pm = params.copy(), params.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = mo.loss_and_grad(pp, pts, targets, lo, hi, tau, emulate_bf16=False)
        lm, _ = mo.loss_and_grad(pm, pts, targets, lo, hi, tau, emulate_bf16=False)
        fd.append((lp - lm) / (2 * eps))
    fd = np.array(fd)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-4, atol=1e-7)


def test_bf16_rounding():
    ulp = 2.0 ** -7  # bf16 spacing at 1.0
    x = np.array([1.0, 1 + ulp / 2, 1 + ulp / 4, 1 + 0.75 * ulp, 1 + 1.5 * ulp, -3.3, 0.0])
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie -> even
    assert r[2] == 1.0
    assert r[3] == 1.0 + ulp
    assert r[4] == 1.0 + 2 * ulp  # tie -> even (up)
    assert abs(r[5] + 3.3) < 3.3 * 2 ** -8 and r[6] == 0.0
