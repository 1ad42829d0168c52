"""Batched uneven posteriors: P varying-intercept regressions of different
sizes sampled in one launch (one chain group per posterior).

Each member's log density and gradient are compared with the FP64 oracle's
varint model on the same rows (the set orders parameters [beta, log sigma_y,
log tau, alpha]; the oracle [alpha, beta, log sigma_y, log tau]): exact to
1e-10 with FP64 rows, and within 1e-5 relative (lp) / 1e-4 of the largest
component (gradient) with the FP32 rows of the batched workload.  Sampling:
every member's posterior means agree with a separate FP64 run of that
posterior within 4.5 combined MCSE."""
import numpy as np
import pytest

import oracle
import cmdstan_gb300 as gn
from cmdstan_gb300 import workloads

pytestmark = pytest.mark.gpu


def _perm(J, K):
    """set position -> oracle position"""
    return np.r_[J + np.arange(K), J + K, J + K + 1, np.arange(J)]


@pytest.mark.parametrize("fp32", [0, 1])
def test_members_log_prob_grad_match_oracle(fp32):
    data = workloads.varint_set(seed=2, P=6, Jmax=60)
    data["fp32"] = fp32
    m = gn.Model("varint_set", data)
    rng = np.random.default_rng(1)
    per = 2
    q = np.zeros((6 * per, m.dim))
    for p in range(6):
        Dp = int(data["J"][p]) + 12
        q[p * per:(p + 1) * per, :Dp] = rng.uniform(-1, 1, (per, Dp))
    lp, g = m.log_prob_grad(q)
    for p in range(6):
        md = workloads.varint_set_member(data, p)
        om = oracle.OracleModel("varint", md)
        J, K = md["J"], md["K"]
        pm = _perm(J, K)
        for i in range(p * per, (p + 1) * per):
            qo = np.zeros(om.dim)
            qo[pm] = q[i, :J + K + 2]
            olp, og = om.log_prob_grad(qo)
            gs = g[i, :J + K + 2]
            if fp32:
                assert abs(lp[i] - olp) <= 1e-5 * abs(olp) + 1e-6, (p, lp[i], olp)
                assert np.abs(gs - og[pm]).max() <= 1e-4 * np.abs(og).max(), p
            else:
                assert abs(lp[i] - olp) <= 1e-10 * abs(olp), (p, lp[i], olp)
                assert np.allclose(gs, og[pm], rtol=1e-10, atol=1e-10), p
            assert np.all(g[i, J + K + 2:] == 0)


def test_set_sampling_matches_separate_runs():
    P, cpp = 4, 16
    data = workloads.varint_set(seed=5, P=P, Jmax=24)
    ms = gn.Model("varint_set", data)
    fit = ms.sample(num_chains=P * cpp, num_warmup=500, num_samples=500, seed=9)
    assert np.all(fit.status == 0)
    for p in range(P):
        md = workloads.varint_set_member(data, p)
        J, K = md["J"], md["K"]
        sub = fit.draws[p * cpp:(p + 1) * cpp]
        # columns past this posterior's parameters are NaN
        assert np.all(np.isnan(sub[:, :, 7 + J + K + 2:]))
        ref = gn.Model("varint", md).sample(num_chains=cpp, num_warmup=500, num_samples=500, seed=100 + p)
        pm = _perm(J, K)
        for k in range(J + K + 2):
            a = gn.summary(sub[:, :, 7 + k])
            b = gn.summary(ref.draws[:, :, 7 + pm[k]])
            z = abs(a["mean"] - b["mean"]) / np.hypot(a["mcse"], b["mcse"])
            assert z < 4.5, (p, k, a["mean"], b["mean"], z)
            assert a["rhat"] < 1.05, (p, k, a["rhat"])


def test_set_rejects_chain_counts_that_do_not_divide():
    data = workloads.varint_set(seed=1, P=3, Jmax=12)
    m = gn.Model("varint_set", data)
    with pytest.raises(gn.GnutsError):
        m.sample(num_chains=4, num_warmup=10, num_samples=10)
