"""The oracle is pinned before anything is compared against it.

Summary statistics: the exact CSV goldens of the reference's stansummary
tests (src/test/interface/stansummary_test.cpp:481-495 and :622-637) on the
reference's own example-output draws (extracted into tests/golden/ by
tests/golden/make_golden.py).  Philox: the published Random123 known-answer
vectors.  Gradients: central finite differences with the epsilon / error
defaults of CmdStan's diagnose method (arg_test_grad_eps.hpp:15,
arg_test_grad_err.hpp:15).  NUTS: the analytic Beta posterior of the
bernoulli example and the stansummary_test.cpp:249-253 theta bounds.
"""
import json
import os

import numpy as np
import pytest

import oracle
from cmdstan_gb300 import workloads

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(stem):
    with open(os.path.join(GOLD, stem + ".json")) as f:
        g = json.load(f)
    return g["names"], np.array(g["draws"])


def _fmt(name, s):
    vals = [s["mean"], s["mcse"], s["sd"], s["mad"], s["q5"], s["q50"], s["q95"], s["ess_bulk"], s["ess_tail"],
            s["rhat"]]
    return '"%s",' % name + ",".join("%g" % v for v in vals)


# literal lines of stansummary_test.cpp (check_csv_output, check_csv_output_include_param)
BERNOULLI_GOLD = {
    "lp__": '"lp__",-7.2719,0.0365168,0.768874,0.303688,-8.98426,-6.97009,-6.75007,519.29,503.309,1.00141',
    "energy__": '"energy__",7.78428,0.0508815,1.0314,0.745859,6.80565,7.46758,9.8864,489.874,486.438,1.00495',
    "theta": '"theta",0.256552,0.00610844,0.119654,0.120965,0.0802982,0.24996,0.47034,361.506,395.736,1.00186',
}
EIGHT_SCHOOLS_GOLD = {
    "lp__": '"lp__",-15.5617,0.97319,6.05585,6.3817,-25.3182,-15.7598,-5.47732,41.1897,113.537,1.00153',
    "energy__": '"energy__",20.5888,1.01449,6.43127,6.6161,10.2809,20.8278,30.9921,42.5605,140.171,1.00069',
    "theta.6": '"theta[6]",5.001,0.365016,5.76072,5.37947,-4.95375,5.22746,14.1688,230.645,464.978,1.00054',
    "theta.7": '"theta[7]",8.54125,0.650098,6.22195,5.35785,-0.814388,8.09342,19.2622,92.3075,241.177,1.00244',
}


@pytest.mark.parametrize("stem,gold", [("bernoulli_chain_1", BERNOULLI_GOLD),
                                       ("eight_schools_output", EIGHT_SCHOOLS_GOLD)])
def test_summary_matches_stansummary_goldens(stem, gold):
    names, d = _load(stem)
    for col, line in gold.items():
        s = oracle.summary(d[:, names.index(col)][None, :])
        label = col if "." not in col else "%s[%s]" % tuple(col.split("."))
        assert _fmt(label, s) == line


def test_summary_no_percentile_line():
    # stansummary_test.cpp check_csv_output_no_percentiles: lp__ without quantiles
    names, d = _load("bernoulli_chain_1")
    s = oracle.summary(d[:, names.index("lp__")][None, :])
    got = ",".join("%g" % v for v in (s["mean"], s["mcse"], s["sd"], s["mad"], s["ess_bulk"], s["ess_tail"],
                                      s["rhat"]))
    assert got == "-7.2719,0.0365168,0.768874,0.303688,519.29,503.309,1.00141"


def test_rhat_split_chains_detects_shift():
    g = np.random.default_rng(1)
    x = g.standard_normal((4, 500))
    assert oracle.rhat(x) < 1.01
    x[0] += 2.0
    assert oracle.rhat(x) > 1.1


KAT = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
       ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
       ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
        (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(ctr, key, expect):
    assert oracle.philox(ctr, key) == list(expect)


def _models():
    return [
        ("bernoulli", workloads.bernoulli_reference()),
        ("proper", {}),
        ("test_model", {}),
        ("logistic", workloads.logistic(seed=3, N=200, D=7)),
        ("hier", workloads.hier(seed=4, J=9)),
        ("hier", workloads.eight_schools()),
        ("funnel", workloads.funnel(K=6)),
        ("varint", workloads.varint(seed=5, J=6, K=3)),
        ("horseshoe", workloads.horseshoe(seed=6, N=150, D=9, n_nonzero=3)),
    ]


@pytest.mark.parametrize("mid,data", _models(), ids=lambda v: v if isinstance(v, str) else "")
@pytest.mark.parametrize("jac", [True, False])
def test_oracle_gradient_finite_differences(mid, data, jac):
    m = oracle.OracleModel(mid, data)
    g = np.random.default_rng(11)
    eps, err = 1e-6, 1e-6  # CmdStan diagnose defaults
    for _ in range(3):
        q = g.uniform(-1.5, 1.5, m.dim)
        lp, grad = m.log_prob_grad(q, jac)
        assert np.isfinite(lp)
        fd = np.zeros(m.dim)
        for i in range(m.dim):
            e = np.zeros(m.dim)
            e[i] = eps
            fd[i] = (m.log_prob_grad(q + e, jac)[0] - m.log_prob_grad(q - e, jac)[0]) / (2 * eps)
        scale = np.maximum(1.0, np.abs(grad))
        assert np.all(np.abs(fd - grad) / scale < 1e3 * err), (mid, fd, grad)


def test_oracle_bernoulli_matches_analytic_posterior():
    m = oracle.OracleModel("bernoulli", workloads.bernoulli_reference())
    draws, eps, minv, ng = m.run_chains(4, threads=4, seed=1234)
    theta = 1.0 / (1.0 + np.exp(-draws[:, :, 7]))
    s = oracle.summary(theta)
    # posterior Beta(3, 9): mean 0.25, sd sqrt(27/1872)
    assert abs(s["mean"] - 0.25) < 4 * s["mcse"]
    assert abs(s["sd"] - np.sqrt(27 / 1872)) < 0.01
    assert 0.25 < s["mean"] < 0.27 or abs(s["mean"] - 0.25) < 4 * s["mcse"]
    assert s["rhat"] < 1.01
    assert np.all(np.isfinite(eps)) and np.all(minv > 0)
    # adapted step size / metric in the range of the reference fixture (1.02703 / 0.526879)
    assert 0.4 < np.median(eps) < 2.0 and 0.2 < np.median(minv) < 1.0


def test_oracle_standard_normal_dense_metric():
    m = oracle.OracleModel("test_model", {})
    draws, eps, minv, ng = m.run_chains(2, threads=2, seed=7, metric=1, num_warmup=500, num_samples=1000)
    x = draws[:, :, 7:]
    assert abs(x[:, :, 0].std() - 10.0) < 1.0
    assert abs(x[:, :, 1].std() - 1.0) < 0.1
    assert minv.shape == (2, 4)


def test_oracle_no_adapt_keeps_stepsize():
    m = oracle.OracleModel("proper", {})
    draws, eps, minv, ng = m.run_chains(1, seed=3, adapt_engaged=0, stepsize=0.5, num_warmup=10, num_samples=20)
    assert np.all(draws[:, :, 2] == 0.5)
    assert eps[0] == 0.5


def test_oracle_replay_reversible_energy():
    # a single transition on a standard normal with a tiny step conserves energy
    m = oracle.OracleModel("normal", {"scales": np.ones(5)})
    q0 = np.linspace(-1, 1, 5)
    p0 = np.array([0.3, -0.2, 0.5, 0.1, -0.4])
    q, st, ctr = m.transition(q0, p0, 0.01, inv_metric=np.ones(5), max_depth=4)
    assert st[3] == 4 and st[4] == 15  # hits max depth: 2^4 - 1 leapfrogs
    assert st[1] > 0.999
