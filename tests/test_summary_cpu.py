"""The product's stansummary statistics (gnuts_summary, host C++) against the
reference's stansummary goldens (src/test/interface/stansummary_test.cpp
:481-495 and :622-637) and against the oracle's independent restatement."""
import json
import os

import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import gnuts
import oracle
from test_oracle_golden import BERNOULLI_GOLD, EIGHT_SCHOOLS_GOLD, _fmt, _load


@pytest.mark.parametrize("stem,gold", [("bernoulli_chain_1", BERNOULLI_GOLD),
                                       ("eight_schools_output", EIGHT_SCHOOLS_GOLD)])
def test_product_summary_matches_goldens(stem, gold):
    names, d = _load(stem)
    for col, line in gold.items():
        s = gnuts.summary(d[:, names.index(col)][None, :])
        label = col if "." not in col else "%s[%s]" % tuple(col.split("."))
        assert _fmt(label, s) == line


def test_product_summary_columns_matches_oracle():
    g = np.random.default_rng(3)
    C, n, K = 6, 400, 5
    draws = np.cumsum(g.standard_normal((C, n, K)), axis=1) * 0.05 + g.standard_normal((C, n, K))
    draws[:, :, 2] = np.round(draws[:, :, 2], 1)  # ties
    res = gnuts.summary_columns(draws, [0, 1, 2, 3, 4], threads=3)
    for j in range(K):
        o = oracle.summary(draws[:, :, j])
        for k in o:
            assert np.isclose(res[j][k], o[k], rtol=1e-9, atol=1e-12), (j, k, res[j][k], o[k])


def test_summary_odd_length_and_constant():
    x = np.random.default_rng(1).standard_normal((3, 101))
    s, o = gnuts.summary(x), oracle.summary(x)
    assert np.isclose(s["ess_bulk"], o["ess_bulk"]) and np.isclose(s["rhat"], o["rhat"])
    c = gnuts.summary(np.ones((2, 50)))
    assert np.isnan(c["ess_bulk"]) and c["sd"] == 0
