"""Parity at the shapes the benchmark times.

The other gradient tests run at small N; these run the mixed-precision
gradients at the benchmarked sizes against the FP64 oracle
(src/cmdstan/command_helper.hpp:589-593 is the log_prob_grad contract):

* logistic regression, X 100,000 x 100, 1024 points: the tcgen05 kernel runs
  8 chain tiles x 19 row splits, the last split ends in a partial row tile;
  a second call with 1000 points ends in a partial chain tile.
* regularised-horseshoe logistic regression, X 200,000 x 1000, 256 points
  (the wide-design path).
* a 1024-chain mixed-precision run of the logistic workload against an FP64
  GPU run of the same data: every posterior mean and sd within 3 combined
  MCSE (the sd's standard error from the ESS of the squared deviations).
  With 101 parameters a handful of 3-sigma excursions is expected by
  chance alone (0.27 % each), so the test bounds their count (at most 2) and
  the largest |z| (below 4, a 0.6 % family-wise level).

Tolerances of the mixed path: lp relative 1e-4 and gradient 2e-3 of its
largest component at random points; at draws of the posterior lp 1e-6 and
gradient 3e-3.
"""
import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import workloads
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def logistic_bench():
    data = workloads.logistic(seed=0, N=100_000, D=100)
    return data, gn.Model("logistic", data), oracle.OracleModel("logistic", data)


def _check_points(gm, om, q, idx, lp_rtol, g_rtol):
    lp, g = gm.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    assert np.all(np.isfinite(lp)) and np.all(np.isfinite(g))
    worst_lp, worst_g = 0.0, 0.0
    for i in idx:
        olp, og = om.log_prob_grad(q[i])
        worst_lp = max(worst_lp, abs(lp[i] - olp) / abs(olp))
        worst_g = max(worst_g, np.max(np.abs(g[i] - og)) / np.max(np.abs(og)))
    assert worst_lp <= lp_rtol, worst_lp
    assert worst_g <= g_rtol, worst_g
    return worst_lp, worst_g


def _se_sd(x, s):
    """Monte Carlo standard error of a sample sd: sd / sqrt(2 ESS) with the
    ESS of the squared deviations (NUTS draws are often antithetic for the
    mean, so the mean's ESS would understate the sd's error)."""
    return s["sd"] / np.sqrt(2.0 * oracle.ess_bulk((x - s["mean"]) ** 2))


@pytest.mark.parametrize("n", [1024, 1000])
def test_tensor_core_gradient_at_bench_shape(logistic_bench, n):
    data, gm, om = logistic_bench
    rng = np.random.default_rng(n)
    q = rng.normal(0, 0.3, (n, gm.dim))
    # one or two points of every 128-chain tile, including the last (partial) one
    idx = sorted({0, 1, n - 1, n - 2} | {t * 128 + 127 for t in range(n // 128)} | set(range(128, n, 128)))
    idx = [i for i in idx if i < n]
    _check_points(gm, om, q, idx, 1e-4, 2e-3)


def test_tensor_core_gradient_at_posterior_draws(logistic_bench):
    """At posterior draws (where the sampler spends its time) lp is far more
    accurate than at random points: the linear likelihood part is FP64 and the
    even part's FP32 terms are small."""
    data, gm, om = logistic_bench
    fit = gm.sample(num_chains=128, num_warmup=150, num_samples=8, seed=3, precision=gn.PRECISION_MIXED)
    q = np.array([gm.unconstrain(c) for c in fit.draws[:, -1, 7:]])
    _check_points(gm, om, q, list(range(0, q.shape[0], 9)), 1e-6, 3e-3)


def test_wide_gradient_at_bench_shape():
    data = workloads.horseshoe(seed=0)
    gm, om = gn.Model("horseshoe", data), oracle.OracleModel("horseshoe", data)
    rng = np.random.default_rng(5)
    n = 256
    q = rng.normal(0, 0.3, (n, gm.dim))
    _check_points(gm, om, q, [0, 1, 127, 128, 254, 255], 1e-4, 2e-3)


def test_mixed_moments_match_fp64_at_bench_shape(logistic_bench):
    data, gm, om = logistic_bench
    mixed = gm.sample(num_chains=1024, num_warmup=1000, num_samples=1000, seed=1, precision=gn.PRECISION_MIXED)
    fp64 = gm.sample(num_chains=64, num_warmup=300, num_samples=300, seed=1)
    zm, zs = [], []
    for j in range(gm.num_constrained):
        x, y = mixed.draws[:, :, 7 + j], fp64.draws[:, :, 7 + j]
        sx, sy = oracle.summary(x), oracle.summary(y)
        assert sx["rhat"] < 1.01 and sy["rhat"] < 1.01, (gm.param_names[j], sx["rhat"], sy["rhat"])
        zm.append((sx["mean"] - sy["mean"]) / np.hypot(sx["mcse"], sy["mcse"]))
        zs.append((sx["sd"] - sy["sd"]) / np.hypot(_se_sd(x, sx), _se_sd(y, sy)))
    zm, zs = np.abs(zm), np.abs(zs)
    assert np.sum(zm > 3) <= 2 and zm.max() < 4, np.sort(zm)[-5:]
    assert np.sum(zs > 3) <= 2 and zs.max() < 4, np.sort(zs)[-5:]
