"""The allocation-free gradient entry point (gnuts_log_prob_grad_noalloc).

It serves callers that cannot call cudaMalloc (an arena or pool that owns all
device memory, a callback inside another library, an allocator-free loop)
but can pass device buffers they own.  Here the test plays that caller: its
buffers come from torch, and the entry point's results, taken through the C
ABI on two calls in a row, must equal those of the ordinary allocating entry
point gnuts_log_prob_grad (relative 1e-10, the FP64 tolerance of the other
gradient tests).  The file is named to run last, and it creates its own
model, so it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import gnuts, workloads

pytestmark = pytest.mark.gpu


def _noalloc(model, q_dev, lp_dev, g_dev, n, jacobian=True):
    lib = gn.load()
    return lib.gnuts_log_prob_grad_noalloc(model._h, n, ctypes.c_void_p(q_dev.data_ptr()), int(jacobian),
                                           ctypes.c_void_p(lp_dev.data_ptr()), ctypes.c_void_p(g_dev.data_ptr()))


@pytest.mark.parametrize("mid,data,n,jacobian", [
    ("logistic", workloads.logistic(seed=31, N=6000, D=40), 48, True),
    ("horseshoe", workloads.horseshoe(seed=32, N=5000, D=30, n_nonzero=3), 64, True),
    # the horseshoe's constrained scales carry a Jacobian that the finishing
    # kernel removes again when it is off
    ("horseshoe", workloads.horseshoe(seed=32, N=5000, D=30, n_nonzero=3), 64, False),
])
def test_noalloc_matches_allocating_entry_point(mid, data, n, jacobian):
    torch = pytest.importorskip("torch")
    model = gn.Model(mid, data)
    rng = np.random.default_rng(7)
    q = rng.normal(0.0, 0.2, (n, model.dim))
    lp_ref, g_ref = model.log_prob_grad(q, jacobian=jacobian)  # the allocating entry point (also uploads the data)
    q_dev = torch.tensor(q, dtype=torch.float64, device="cuda")
    for call in range(2):
        lp_dev = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        g_dev = torch.full((n, model.dim), float("nan"), dtype=torch.float64, device="cuda")
        rc = _noalloc(model, q_dev, lp_dev, g_dev, n, jacobian)
        assert rc == gnuts.GNUTS_OK, call
        lp, g = lp_dev.cpu().numpy(), g_dev.cpu().numpy()
        np.testing.assert_allclose(lp, lp_ref, rtol=1e-10, atol=0)
        np.testing.assert_allclose(g, g_ref, rtol=1e-10, atol=1e-10 * np.abs(g_ref).max())


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    model = gn.Model("logistic", workloads.logistic(seed=33, N=5000, D=10))
    model.log_prob_grad(np.zeros((1, model.dim)))
    n = gnuts_max = 64 + 1
    q_dev = torch.zeros((n, model.dim), dtype=torch.float64, device="cuda")
    lp_dev = torch.zeros((n,), dtype=torch.float64, device="cuda")
    g_dev = torch.zeros((n, model.dim), dtype=torch.float64, device="cuda")
    rc = _noalloc(model, q_dev, lp_dev, g_dev, gnuts_max)
    assert rc == gnuts.ERR_ARGUMENT
    buf = ctypes.create_string_buffer(512)
    gn.load().gnuts_last_error(buf, 512)
    assert b"GNUTS_NOALLOC_MAX_POINTS" in buf.value
    # a model without a scratch-using kernel is refused too
    small = gn.Model("proper")
    rc = gn.load().gnuts_log_prob_grad_noalloc(small._h, 1, ctypes.c_void_p(q_dev.data_ptr()), 1,
                                                ctypes.c_void_p(lp_dev.data_ptr()),
                                                ctypes.c_void_p(g_dev.data_ptr()))
    assert rc == gnuts.ERR_ARGUMENT
