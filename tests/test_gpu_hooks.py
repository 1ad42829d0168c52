"""The services' interrupt callback and streaming draw sink.

CmdStan passes every service an interrupt callback (src/cmdstan/command.hpp:186,
:609-688) and writers that receive each iteration's row (:191-192).  Here the
sink (gnuts_set_draw_sink) must deliver every row of every chain exactly once,
in order, equal to the draws the same call returns, in round mode (batched
gradient) and fused mode; with keep_draws=False the caller holds no draw
array.  The interrupt (gnuts_set_interrupt) polled between launches stops a
run with GNUTS_ERR_INTERRUPTED, and the next call runs normally.
"""
import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import gnuts, workloads

pytestmark = pytest.mark.gpu


def _collect():
    blocks = []
    return blocks, (lambda first, rows: blocks.append((first, rows)))


@pytest.mark.parametrize("mid,data,C", [("logistic", workloads.logistic(seed=41, N=5000, D=12), 64),
                                         ("hier", workloads.eight_schools(), 16)], ids=["rounds", "fused"])
def test_sink_rows_equal_returned_draws(mid, data, C):
    m = gn.Model(mid, data)
    blocks, sink = _collect()
    fit = m.sample(num_chains=C, num_warmup=150, num_samples=200, seed=9, draw_sink=sink)
    firsts = [f for f, _ in blocks]
    assert firsts == sorted(firsts) and firsts[0] == 0
    rows = np.concatenate([r for _, r in blocks], axis=1)
    assert rows.shape == fit.draws.shape
    np.testing.assert_array_equal(rows, fit.draws)


def test_sink_without_a_draw_array():
    m = gn.Model("logistic", workloads.logistic(seed=42, N=5000, D=8))
    blocks, sink = _collect()
    fit = m.sample(num_chains=32, num_warmup=100, num_samples=100, seed=3, draw_sink=sink, keep_draws=False)
    assert fit.draws.shape[1] == 0
    rows = np.concatenate([r for _, r in blocks], axis=1)
    assert rows.shape == (32, 100, 7 + m.num_constrained)
    assert np.all(np.isfinite(rows))


@pytest.mark.parametrize("mid,data", [("logistic", workloads.logistic(seed=43, N=5000, D=8)),
                                       ("funnel", workloads.funnel(10))], ids=["rounds", "fused"])
def test_interrupt_stops_the_run(mid, data):
    m = gn.Model(mid, data)
    polls = []

    def interrupt():
        polls.append(1)
        return len(polls) >= 3

    blocks, sink = _collect()
    with pytest.raises(gnuts.GnutsError) as e:
        m.sample(num_chains=32, num_warmup=2000, num_samples=2000, seed=4, interrupt=interrupt, draw_sink=sink)
    assert e.value.code == gnuts.ERR_INTERRUPTED
    assert len(polls) == 3
    assert sum(r.shape[1] for _, r in blocks) < 4000
    # the hooks were cleared: the next call completes
    fit = m.sample(num_chains=8, num_warmup=50, num_samples=20, seed=5)
    assert fit.draws.shape[1] == 20
