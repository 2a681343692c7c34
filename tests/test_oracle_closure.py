"""The closure oracle's gradient (oracle/closure_oracle.py) against central
finite differences of its own float64 loss: pins the backward pass the GPU
gradient is compared with in tests/test_gpu_closure.py."""
import numpy as np

from oracle import closure_oracle as CO


def _waves(rng, B, H, W):
    c = (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W))) * 0.3 + 1.0
    f = c + 0.05 * (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W)))
    return c, f


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = CO.init_params(5, scale_last=1.0).astype(np.float64)
    c, f = _waves(rng, 1, 5, 6)
    loss, g = CO.gradient(p, c, f, bf=False)
    assert np.isfinite(loss) and loss > 0
    # a sample of parameters from every layer, weights and biases
    offs = np.cumsum([0] + [9 * co * ci * 2 + co * 2 for ci, co in CO.LAYERS])
    idx = []
    for l in range(6):
        idx += list(rng.integers(offs[l], offs[l + 1], 6))
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (CO.forward(pp, c, f, bf=False)[1] - CO.forward(pm, c, f, bf=False)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(g).max()), (i, fd, g[i])


def test_param_layout_and_expansion():
    assert CO.param_count() == 9 * 32 * 2 + 64 + 4 * (9 * 32 * 32 * 2 + 64) + 9 * 32 * 2 + 2
    w = np.random.default_rng(1).standard_normal((9, 3, 2, 2))
    R = CO.expand(w)
    assert R.shape == (9, 6, 4)
    # the expanded real map acts on [re; im] as the complex weights on complex inputs
    x = np.random.default_rng(2).standard_normal(2) + 1j * np.random.default_rng(4).standard_normal(2)
    y = (w[0, ..., 0] + 1j * w[0, ..., 1]) @ x
    yr = R[0] @ np.concatenate([x.real, x.imag])
    np.testing.assert_allclose(yr, np.concatenate([y.real, y.imag]), atol=1e-12)
    np.testing.assert_allclose(CO.contract(R, 3, 2)[..., 0], 2 * w[..., 0], atol=1e-12)
