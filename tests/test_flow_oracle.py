"""The flow oracle is checked on its own before the device flow is compared
with it: inverse(forward(z)) = z, the log-determinant equals log|det| of the
numerical Jacobian, the gradients in z and in theta equal central finite
differences (CmdStan diagnose defaults: epsilon 1e-6, error 1e-6,
arg_test_grad_eps.hpp:15 / arg_test_grad_err.hpp:15), and one Adam step equals
its closed form."""
import numpy as np
import pytest

import oracle
from cmdstan_gb300 import workloads


def _theta(fl, rng, scale=0.3):
    return rng.normal(0, scale, fl.n_params)


@pytest.mark.parametrize("d", [1, 2, 7, 33])
def test_masks_split_every_layer(d):
    fl = oracle.OracleFlow(d, layers=8, hidden=16)
    seen_a = np.zeros(d, bool)
    for l in range(fl.L):
        m = fl.mask(l)
        if d > 1:
            assert 0 < m.sum() < d
        seen_a |= m == 0
    assert seen_a.all() or d == 1


@pytest.mark.parametrize("d", [2, 9, 20])
def test_inverse_and_logdet(d):
    rng = np.random.default_rng(d)
    fl = oracle.OracleFlow(d, layers=5, hidden=12, clamp=3.0)
    th = _theta(fl, rng)
    z = rng.normal(size=d)
    x, ld = fl.forward(th, z)
    z2, ld2 = fl.inverse(th, x)
    assert np.allclose(z2, z, atol=1e-12)
    assert abs(ld - ld2) < 1e-12
    J = np.zeros((d, d))
    h = 1e-6
    for i in range(d):
        e = np.zeros(d)
        e[i] = h
        J[:, i] = (fl.forward(th, z + e)[0] - fl.forward(th, z - e)[0]) / (2 * h)
    assert abs(np.linalg.slogdet(J)[1] - ld) < 1e-6


@pytest.mark.parametrize("model_id", ["funnel", "hier"])
def test_gradients_match_finite_differences(model_id):
    rng = np.random.default_rng(7)
    data = {"K": 6} if model_id == "funnel" else workloads.eight_schools()
    om = oracle.OracleModel(model_id, data)
    d = om.dim
    fl = oracle.OracleFlow(d, layers=4, hidden=10, clamp=3.0)
    th = _theta(fl, rng, 0.2)
    z = rng.normal(0, 0.5, d)
    lp, gz, gth, x, lpx = fl.log_prob_grad(om, th, z, param_grad=True)
    assert abs(lp - (lpx + fl.forward(th, z)[1])) < 1e-10
    h = 1e-6
    for i in range(d):
        e = np.zeros(d)
        e[i] = h
        fd = (fl.log_prob_grad(om, th, z + e)[0] - fl.log_prob_grad(om, th, z - e)[0]) / (2 * h)
        assert abs(fd - gz[i]) < 1e-6 * max(1.0, abs(gz[i])), (i, fd, gz[i])
    for i in rng.choice(fl.n_params, 60, replace=False):
        e = np.zeros(fl.n_params)
        e[i] = h
        fd = (fl.log_prob_grad(om, th + e, z)[0] - fl.log_prob_grad(om, th - e, z)[0]) / (2 * h)
        assert abs(fd - gth[i]) < 1e-6 * max(1.0, abs(gth[i])), (i, fd, gth[i])


def test_adam_closed_form():
    rng = np.random.default_rng(3)
    n = 50
    th, m, v = rng.normal(size=n), np.zeros(n), np.zeros(n)
    th0 = th.copy()
    g = rng.normal(size=n)
    oracle.adam(th, m, v, g, 1, lr=0.01)
    # first step: m_hat = g, v_hat = g^2 -> step = lr * g / (|g| + eps)
    assert np.allclose(th, th0 - 0.01 * g / (np.abs(g) + 1e-8), rtol=1e-12, atol=1e-14)
    g2 = rng.normal(size=n)
    m_ref = 0.9 * (0.1 * g) + 0.1 * g2
    v_ref = 0.999 * (0.001 * g * g) + 0.001 * g2 * g2
    th1 = th.copy()
    oracle.adam(th, m, v, g2, 2, lr=0.01)
    step = 0.01 * (m_ref / (1 - 0.9 ** 2)) / (np.sqrt(v_ref / (1 - 0.999 ** 2)) + 1e-8)
    assert np.allclose(th, th1 - step, rtol=1e-12, atol=1e-14)


def test_device_flow_layout_matches_oracle_without_gpu():
    """Creating a flow is host-only: its parameter count equals the oracle's."""
    import cmdstan_gb300 as gn
    for d, L, H in [(2, 8, 32), (66, 8, 128), (101, 8, 128), (128, 16, 64)]:
        assert gn.Flow(d, layers=L, hidden=H).n_params == oracle.OracleFlow(d, L, H).n_params
    with pytest.raises(gn.GnutsError):
        gn.Flow(1)
    with pytest.raises(gn.GnutsError):
        gn.Flow(129)
    with pytest.raises(gn.GnutsError):
        gn.Flow(10, hidden=100)
