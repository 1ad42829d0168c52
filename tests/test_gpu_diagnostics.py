"""diagnostic_file rows (CmdStan's diagnostic writers, src/cmdstan/command.hpp:
225-247): per saved iteration the seven sampler columns, the selected point's
unconstrained position q, its momentum p and the gradient g.

Checked against what they must satisfy: the sampler columns are the draws',
write_array(q) is the draw, g is the FP64 gradient at q, and after warmup the
energy column is -lp + p.M^-1.p / 2 with the adapted metric (which pins p);
asking for the rows does not change the draws.
"""
import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mid,data,C", [("logistic", workloads.logistic(seed=51, N=5000, D=9), 32),
                                         ("hier", workloads.eight_schools(), 8)], ids=["rounds", "fused"])
def test_diagnostic_rows_are_consistent(mid, data, C):
    m = gn.Model(mid, data)
    kw = dict(num_chains=C, num_warmup=200, num_samples=100, seed=13)
    fit = m.sample(diagnostics=True, **kw)
    plain = m.sample(**kw)
    np.testing.assert_array_equal(fit.draws, plain.draws)
    dg = fit.diagnostics
    D = m.dim
    assert dg.shape == (C, 100, 7 + 3 * D)
    np.testing.assert_array_equal(dg[:, :, :7], fit.draws[:, :, :7])
    q = dg[:, :, 7:7 + D].reshape(-1, D)
    p = dg[:, :, 7 + D:7 + 2 * D].reshape(C, 100, D)
    g = dg[:, :, 7 + 2 * D:].reshape(-1, D)
    np.testing.assert_allclose(m.write_array(q), fit.draws[:, :, 7:].reshape(-1, m.num_constrained),
                               rtol=1e-12, atol=1e-12)
    lp, g_ref = m.log_prob_grad(q)
    np.testing.assert_allclose(g, g_ref, rtol=1e-9, atol=1e-9 * np.abs(g_ref).max())
    np.testing.assert_allclose(lp, fit.draws[:, :, 0].reshape(-1), rtol=1e-10)
    kin = 0.5 * np.einsum("cnd,cd->cn", p * p, fit.inv_metric)
    energy = -fit.draws[:, :, 0] + kin
    np.testing.assert_allclose(energy, fit.draws[:, :, 6], rtol=1e-9, atol=1e-9)
