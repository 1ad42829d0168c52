"""stansummary statistics on the GPU (gnuts_summary_columns_gpu) against the
reference's stansummary goldens (src/test/interface/stansummary_test.cpp
:481-495 and :622-637) and against the host version on data that exercises
ties, odd chain lengths, constant quantities and thousands of chains."""
import time

import numpy as np
import pytest

from cmdstan_gb300 import gnuts
from test_oracle_golden import BERNOULLI_GOLD, EIGHT_SCHOOLS_GOLD, _fmt, _load

pytestmark = pytest.mark.gpu

KEYS = ["mean", "mcse", "sd", "mad", "q5", "q50", "q95", "ess_bulk", "ess_tail", "rhat"]


@pytest.mark.parametrize("stem,gold", [("bernoulli_chain_1", BERNOULLI_GOLD),
                                       ("eight_schools_output", EIGHT_SCHOOLS_GOLD)])
def test_gpu_summary_matches_goldens(stem, gold):
    names, d = _load(stem)
    cols = [names.index(c) for c in gold]
    res = gnuts.summary_columns(d[None, :, :], cols, gpu=True)
    for (col, line), s in zip(gold.items(), res):
        label = col if "." not in col else "%s[%s]" % tuple(col.split("."))
        assert _fmt(label, s) == line


def _close(a, b, rtol=1e-9):
    for k in KEYS:
        x, y = a[k], b[k]
        if np.isnan(x) or np.isnan(y):
            assert np.isnan(x) and np.isnan(y), (k, x, y)
        else:
            assert np.isclose(x, y, rtol=rtol, atol=1e-12), (k, x, y)


@pytest.mark.parametrize("C,n", [(7, 999), (4, 1000), (1, 11)])
def test_gpu_summary_equals_host(C, n):
    g = np.random.default_rng(C * 1000 + n)
    K = 6
    d = np.cumsum(g.standard_normal((C, n, K)), axis=1) * 0.05 + g.standard_normal((C, n, K))
    d[:, :, 1] = np.round(d[:, :, 1], 1)          # many ties
    d[:, :, 2] = 3.5                               # constant: ESS and R-hat undefined
    d[:, :, 3] = g.integers(0, 3, (C, n))          # discrete
    d[:, :, 4] = -np.abs(d[:, :, 4])               # negative values and zeros
    d[0, 0, 4] = -0.0
    d[:, :, 5] += np.arange(C)[:, None] * 0.5      # chains disagree
    host = gnuts.summary_columns(d, list(range(K)))
    dev = gnuts.summary_columns(d, list(range(K)), gpu=True)
    for j in range(K):
        _close(dev[j], host[j])


def test_gpu_summary_thousands_of_chains():
    """1024 chains x 1000 draws: equal to the host, and reported faster"""
    g = np.random.default_rng(9)
    d = g.standard_normal((1024, 1000, 4)) + np.linspace(0, 0.01, 1024)[:, None, None]
    t = time.perf_counter()
    host = gnuts.summary_columns(d, [0, 1, 2, 3])
    th = time.perf_counter() - t
    t = time.perf_counter()
    dev = gnuts.summary_columns(d, [0, 1, 2, 3], gpu=True)
    tg = time.perf_counter() - t
    for j in range(4):
        _close(dev[j], host[j], rtol=1e-8)
    print("host %.3f s, device %.3f s" % (th, tg))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["corr_gauss", "corr_gauss_depth8", "corr_gauss_depth15", "eight_schools", "mix"])
def test_diagnose_gpu_matches_reference(case):
    """gnuts_diagnose with the ESS / R-hat statistics on the GPU reproduces
    the reference's diagnose reports (src/test/interface/diagnose_test.cpp)."""
    import test_diagnose_cpu as tdc
    draws, names, max_depth, nom = tdc.load_case(case)
    text, _ = gnuts.diagnose(draws, names, max_depth=max_depth, gpu=True)
    assert text == nom


@pytest.mark.gpu
def test_diagnose_gpu_many_chains_matches_host():
    """2048 chains x 1000 draws x 12 parameters: the device statistics give the
    host path's report and counts."""
    import time
    rng = np.random.default_rng(5)
    C, n, P = 2048, 1000, 12
    d = np.zeros((C, n, 7 + P))
    d[:, :, 3] = rng.integers(1, 11, (C, n))
    d[:, :, 5] = rng.random((C, n)) < 1e-4
    d[:, :, 6] = rng.normal(size=(C, n))
    d[:, :, 7:] = rng.normal(size=(C, n, P))
    d[:512, :, 8] += 2.0  # a quarter of the chains off for one parameter: its R-hat is flagged
    names = ["lp__", "accept_stat__", "stepsize__", "treedepth__", "n_leapfrog__", "divergent__", "energy__"] + \
        ["b.%d" % (i + 1) for i in range(P)]
    t = time.perf_counter()
    tg, rg = gnuts.diagnose(d, names, gpu=True)
    tgpu = time.perf_counter() - t
    th, rh = gnuts.diagnose(d, names, gpu=False)
    assert tg == th and rg["n_treedepth_max"] == rh["n_treedepth_max"] and rg["n_high_rhat"] == 1
    print("diagnose of 2048 x 1000 x %d on the GPU: %.3f s" % (P, tgpu))
