"""GPU sampler vs the CPU oracle, through the C ABI.

* log_prob_grad of every model: FP64, relative error <= 1e-10 (batched
  round-mode path included for large N).
* One NUTS transition with injected momentum (replay): identical tree depth,
  leapfrog count, divergence flag and RNG consumption; selected point within
  1e-10 relative.
* Whole runs without adaptation on a Gaussian target (linear dynamics, so
  GPU and oracle stay together): every draw equal within 1e-8 relative for
  diag_e, dense_e and unit_e.  With adaptation, the first iterations are
  equal, and the device's adapted metric and step-size sequence are
  re-derived exactly from its own warmup draws.
* Whole runs on nonlinear models: moments within 4 combined MCSE of the
  oracle, R-hat < 1.01, analytic posterior where one exists.
"""
import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import workloads
import oracle

pytestmark = pytest.mark.gpu


def _pair(mid, data):
    return gn.Model(mid, data), oracle.OracleModel(mid, data)


MODELS = [
    ("bernoulli", workloads.bernoulli_reference()),
    ("test_model", {}),
    ("logistic", workloads.logistic(seed=3, N=300, D=7)),
    ("logistic", workloads.logistic(seed=4, N=5000, D=20)),     # batched round-mode path
    ("hier", workloads.eight_schools()),
    ("hier", workloads.hier(seed=5, J=64)),
    ("funnel", workloads.funnel(K=100)),
    ("varint", workloads.varint(seed=6, J=12, K=10)),
    ("horseshoe", workloads.horseshoe(seed=7, N=400, D=30, n_nonzero=4)),
    ("horseshoe", workloads.horseshoe(seed=8, N=5000, D=40, n_nonzero=4)),  # batched
]


@pytest.mark.parametrize("mid,data", MODELS, ids=lambda v: v if isinstance(v, str) else "")
@pytest.mark.parametrize("jac", [True, False])
def test_log_prob_grad_matches_oracle(mid, data, jac):
    gm, om = _pair(mid, data)
    rng = np.random.default_rng(2)
    q = rng.uniform(-1, 1, (5, gm.dim))
    lp, g = gm.log_prob_grad(q, jacobian=jac)
    for i in range(q.shape[0]):
        olp, og = om.log_prob_grad(q[i], jac)
        assert abs(lp[i] - olp) <= 1e-10 * max(1.0, abs(olp))
        np.testing.assert_allclose(g[i], og, rtol=1e-10, atol=1e-10 * max(1.0, np.abs(og).max()))


def test_write_array_matches_oracle():
    for mid, data in MODELS[:1] + MODELS[4:5] + MODELS[7:9]:
        gm, om = _pair(mid, data)
        q = np.random.default_rng(3).uniform(-1, 1, (3, gm.dim))
        out = gm.write_array(q)
        for i in range(3):
            np.testing.assert_allclose(out[i], om.write_array(q[i]), rtol=1e-12)


REPLAY = [
    ("test_model", {}, 0.9, "diag_e"),
    ("test_model", {}, 0.05, "diag_e"),      # long trajectories: max depth
    ("test_model", {}, 40.0, "diag_e"),      # divergences
    ("test_model", {}, 0.7, "dense_e"),
    ("test_model", {}, 0.7, "unit_e"),
    ("bernoulli", workloads.bernoulli_reference(), 1.0, "diag_e"),
    ("hier", workloads.eight_schools(), 0.3, "diag_e"),
    ("hier", workloads.eight_schools(), 0.3, "dense_e"),
    ("funnel", workloads.funnel(K=20), 0.2, "diag_e"),
    ("logistic", workloads.logistic(seed=3, N=300, D=7), 0.1, "diag_e"),
    ("varint", workloads.varint(seed=6, J=5, K=3), 0.05, "diag_e"),
    ("horseshoe", workloads.horseshoe(seed=7, N=200, D=6, n_nonzero=2), 0.05, "diag_e"),
]


@pytest.mark.parametrize("mid,data,eps,metric", REPLAY, ids=lambda v: str(v) if not isinstance(v, dict) else "")
def test_transition_replay_matches_oracle(mid, data, eps, metric):
    gm, om = _pair(mid, data)
    D = gm.dim
    rng = np.random.default_rng(5)
    n = 24
    q0 = rng.uniform(-1, 1, (n, D))
    p0 = rng.standard_normal((n, D))
    mk = gn.METRICS[metric]
    if mk == 0:
        im = rng.uniform(0.5, 2.0, D)
    elif mk == 1:
        A = rng.standard_normal((D, D)) * 0.2
        im = A @ A.T + np.eye(D)
    else:
        im = None
    ids = np.arange(7, 7 + n, dtype=np.uint32)
    ctr = rng.integers(0, 1000, n).astype(np.uint64)
    qo, st, ctr_out = gm.transition(q0, p0, eps, inv_metric=None if im is None else im.ravel(), metric=metric,
                                    max_depth=6, seed=99, chain_ids=ids, counters=ctr.copy())
    for i in range(n):
        oq, ost, octr = om.transition(q0[i], p0[i], eps, inv_metric=None if im is None else im.ravel(), metric=mk,
                                      max_depth=6, seed=99, chain=int(ids[i]), counter=int(ctr[i]))
        assert st[i, 3] == ost[3], "treedepth"
        assert st[i, 4] == ost[4], "n_leapfrog"
        assert st[i, 5] == ost[5], "divergent"
        assert int(ctr_out[i]) == octr, "rng draws consumed"
        np.testing.assert_allclose(qo[i], oq, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(st[i, [0, 1, 6]], ost[[0, 1, 6]], rtol=1e-9, atol=1e-9)


GAUSS = {"scales": np.array([1.0, 3.0, 0.5, 2.0, 1.5])}


@pytest.mark.parametrize("metric", ["diag_e", "dense_e", "unit_e"])
def test_full_run_gaussian_no_adapt_equals_oracle(metric):
    """Fixed step size and metric: Gaussian dynamics are linear, so the whole
    GPU run (momentum draws, trees, multinomial choices, recording) equals the
    oracle run."""
    gm, om = _pair("normal", GAUSS)
    mk = gn.METRICS[metric]
    im = None
    if mk == 0:
        im = np.array([1.0, 9.0, 0.25, 4.0, 2.25])
    elif mk == 1:
        A = np.random.default_rng(0).standard_normal((5, 5)) * 0.3
        im = (A @ A.T + np.diag([1.0, 9.0, 0.25, 4.0, 2.25])).ravel()
    kw = dict(num_warmup=100, num_samples=400, seed=4321, stepsize=0.6, save_warmup=1)
    fit = gm.sample(metric=metric, adapt=False, num_chains=3, chain_id=1, inv_metric=im, **kw)
    od, oeps, ominv, ong = om.run_chains(3, threads=3, first_chain_id=1, metric=mk, adapt_engaged=0,
                                         inv_metric=im, **kw)
    np.testing.assert_array_equal(fit.draws[:, :, 3:6], od[:, :, 3:6])   # treedepth, n_leapfrog, divergent
    np.testing.assert_allclose(fit.draws, od, rtol=1e-8, atol=1e-9)
    assert np.all(fit.n_grad == ong)


def test_team_state_machine_run_equals_oracle():
    """Chains of at least 512 parameters advance as CTA teams of 128 threads
    in round mode (the horseshoe workload's D = 2003 runs this way).  An FP64
    logistic posterior with 520 predictors (D = 521), fixed step size and
    metric, chains started at zero: the transitions equal the oracle's
    (tree depth, leapfrog count, divergence) and the draws agree within 1e-8,
    the team sums differing from the oracle's only in summation order."""
    data = workloads.logistic(seed=31, N=4096, D=520)
    gm, om = _pair("logistic", data)
    kw = dict(num_warmup=0, num_samples=12, seed=77, stepsize=0.01)
    fit = gm.sample(adapt=False, num_chains=4, chain_id=1, inits=np.zeros(gm.dim), **kw)
    od, _, _, ong = om.run_chains(4, threads=4, first_chain_id=1, inits=np.zeros(gm.dim), adapt_engaged=0, **kw)
    assert fit.timing["chains_per_cta"] == 1.0  # one chain per CTA: the team path ran
    np.testing.assert_array_equal(fit.draws[:, :, 3:6], od[:, :, 3:6])
    np.testing.assert_allclose(fit.draws, od, rtol=1e-8, atol=1e-9)
    assert np.all(fit.n_grad == ong)


def test_team_dense_fp64_run_equals_oracle():
    """The team path with an FP64 dense metric (D = 521: team metric product,
    back substitution with team sums per row, the initial Cholesky factor of a
    given SPD inverse metric computed by the warp that initialises the
    chain), fixed step size: the transitions equal the oracle's and the draws
    agree within 1e-8."""
    data = workloads.logistic(seed=32, N=4096, D=520)
    gm, om = _pair("logistic", data)
    D = gm.dim
    rng = np.random.default_rng(3)
    A = rng.standard_normal((D, D)) * (0.3 / np.sqrt(D))
    im = (A @ A.T + np.eye(D)) * 1e-3  # about the posterior scale: sd ~ 0.03
    kw = dict(num_warmup=0, num_samples=6, seed=78, stepsize=0.2)
    fit = gm.sample(metric="dense_e", adapt=False, num_chains=4, chain_id=1, inits=np.zeros(D),
                    inv_metric=im.ravel(), **kw)
    od, _, _, ong = om.run_chains(4, threads=4, first_chain_id=1, inits=np.zeros(D), metric=1, adapt_engaged=0,
                                  inv_metric=im.ravel(), **kw)
    assert fit.timing["chains_per_cta"] == 1.0
    np.testing.assert_array_equal(fit.draws[:, :, 3:6], od[:, :, 3:6])
    np.testing.assert_allclose(fit.draws, od, rtol=1e-8, atol=1e-9)
    assert np.all(fit.n_grad == ong)


def test_dense_metric_team_fp32_matches_fp64():
    """dense_e on the mixed path for a chain of at least 512 parameters: its
    team forms M^-1 p from an FP32 copy of the metric, draws the momentum by a
    blocked FP32 solve with the Cholesky factor and accumulates the Welford
    covariance in FP32 (the factorisation stays FP64).  Adaptation runs
    through a metric update; the posterior moments agree with an FP64 diag_e
    run of the same posterior within 4.5 combined MCSE."""
    data = workloads.logistic(seed=33, N=4096, D=520)
    gm, _ = _pair("logistic", data)
    kw = dict(num_chains=64, num_warmup=150, num_samples=150, seed=8)
    fd = gm.sample(metric="dense_e", precision=gn.PRECISION_MIXED, **kw)
    assert np.all(fd.status == 0) and np.all(np.isfinite(fd.draws))
    assert fd.timing["chains_per_cta"] == 1.0
    # the adapted dense metric is a covariance: symmetric, positive diagonal
    im = fd.inv_metric.reshape(64, gm.dim, gm.dim)
    assert np.allclose(im, np.transpose(im, (0, 2, 1))) and np.all(np.diagonal(im, axis1=1, axis2=2) > 0)
    fr = gm.sample(metric="diag_e", **kw)
    bad = []
    for j in range(0, gm.num_constrained, 13):
        sx, sy = oracle.summary(fd.draws[:, :, 7 + j]), oracle.summary(fr.draws[:, :, 7 + j])
        assert sx["rhat"] < 1.05, (j, sx["rhat"])
        if abs(sx["mean"] - sy["mean"]) >= 4.5 * np.hypot(sx["mcse"], sy["mcse"]):
            bad.append(j)
    assert len(bad) <= 1, bad


@pytest.mark.parametrize("metric", ["diag_e", "dense_e", "unit_e"])
def test_adaptive_run_starts_identical_to_oracle(metric):
    """With adaptation on, ulp differences of libm vs CUDA math are amplified
    by the dual-averaging feedback (x = mu - s_bar sqrt(t) / gamma); the first
    iterations (init, step-size search, first transitions) still coincide."""
    gm, om = _pair("normal", GAUSS)
    kw = dict(num_warmup=300, num_samples=50, seed=4321, save_warmup=1)
    fit = gm.sample(metric=metric, num_chains=3, chain_id=1, **kw)
    od, _, _, _ = om.run_chains(3, threads=3, first_chain_id=1, metric=gn.METRICS[metric], **kw)
    np.testing.assert_array_equal(fit.draws[:, :25, 3:6], od[:, :25, 3:6])
    np.testing.assert_allclose(fit.draws[:, :25], od[:, :25], rtol=1e-6, atol=1e-7)


def _windows(nw, ib=75, tb=50, base=25):
    """Slow-window ends of windowed adaptation for nw warmup iterations."""
    if nw < 20:
        return []
    if ib + base + tb > nw:
        ib, tb = int(0.15 * nw), int(0.1 * nw)
        base = nw - (ib + tb)
    ends, size, nxt = [], base, ib + base - 1
    for counter in range(nw):
        if counter == nxt and counter != nw:
            ends.append(counter)
            if nxt == nw - tb - 1:
                break
            size *= 2
            nxt = counter + size
            if nxt != nw - tb - 1 and nxt + 2 * size >= nw - tb:
                nxt = nw - tb - 1
    return ends


@pytest.mark.parametrize("metric", ["diag_e", "dense_e"])
def test_device_adaptation_rederived_from_its_draws(metric):
    """Re-derive, from the device's own saved warmup draws, the windowed
    Welford metric (n/(n+5) var + 1e-3 * 5/(n+5)) and the dual-averaging
    step-size sequence; both must equal what the device produced."""
    gm = gn.Model("normal", GAUSS)
    nw = 300
    fit = gm.sample(metric=metric, num_chains=2, num_warmup=nw, num_samples=20, seed=99, save_warmup=1)
    ends = _windows(nw)
    assert ends == [99, 149, 249]
    for c in range(2):
        q = fit.draws[c, :nw, 7:]
        lo = ends[-2] + 1
        w = q[lo:ends[-1] + 1]
        n = len(w)
        if metric == "diag_e":
            v = w.var(axis=0, ddof=1)
            expect = n / (n + 5.0) * v + 1e-3 * 5.0 / (n + 5.0)
            np.testing.assert_allclose(fit.inv_metric[c], expect, rtol=1e-10)
        else:
            v = np.cov(w.T, ddof=1)
            expect = n / (n + 5.0) * v + 1e-3 * 5.0 / (n + 5.0) * np.eye(5)
            np.testing.assert_allclose(fit.inv_metric[c], expect, rtol=1e-9, atol=1e-12)
        # dual averaging over the last segment (after the last metric update)
        acc = fit.draws[c, :nw, 1]
        eps = fit.draws[c, :nw, 2]
        t0, gamma, kappa, delta = 10.0, 0.05, 0.75, 0.8
        start = ends[-1] + 1
        mu = np.log(10 * eps[start])
        sbar = xbar = 0.0
        for t in range(1, nw - start + 1):
            a = min(1.0, acc[start + t - 1])
            eta = 1.0 / (t + t0)
            sbar = (1 - eta) * sbar + eta * (delta - a)
            x = mu - sbar * np.sqrt(t) / gamma
            xe = t ** (-kappa)
            xbar = (1 - xe) * xbar + xe * x
            if start + t < nw:
                assert abs(eps[start + t] - np.exp(x)) <= 1e-10 * np.exp(x)
        assert abs(fit.stepsize[c] - np.exp(xbar)) <= 1e-10 * np.exp(xbar)
        assert np.all(fit.draws[c, nw:, 2] == fit.stepsize[c])


def test_full_run_save_warmup_thin_and_no_adapt():
    gm, om = _pair("normal", GAUSS)
    kw = dict(num_warmup=120, num_samples=90, seed=77, save_warmup=1, thin=4, stepsize=0.5)
    fit = gm.sample(adapt=False, num_chains=2, **kw)
    od, oeps, _, _ = om.run_chains(2, threads=2, adapt_engaged=0, **kw)
    assert fit.draws.shape[1] == 30 + 23
    np.testing.assert_allclose(fit.draws, od, rtol=1e-8, atol=1e-9)
    assert np.all(fit.draws[:, :, 2] == 0.5) and np.all(fit.stepsize == 0.5)
    fit = gm.sample(num_chains=2, num_warmup=120, num_samples=90, seed=77, save_warmup=1, thin=4)
    assert fit.draws.shape[1] == 30 + 23


def test_bernoulli_posterior_and_oracle():
    """Beta(3, 9) posterior of the reference's bernoulli example: 64 chains
    give an MCSE near 0.0008, so the analytic moments are checked tightly."""
    gm, om = _pair("bernoulli", workloads.bernoulli_reference())
    fit = gm.sample(num_chains=64, seed=1234)
    th = fit.column("theta")
    s = oracle.summary(th)
    sd = np.sqrt(3 * 9 / (12 ** 2 * 13))
    assert abs(s["mean"] - 0.25) < 4 * s["mcse"], s
    assert abs(s["sd"] / sd - 1) < 0.03, s
    assert s["rhat"] < 1.01
    od, oeps, ominv, _ = om.run_chains(64, threads=16, seed=1234)
    os_ = oracle.summary(1 / (1 + np.exp(-od[:, :, 7])))
    assert abs(s["mean"] - os_["mean"]) < 4 * np.hypot(s["mcse"], os_["mcse"])
    assert abs(np.median(fit.stepsize) / np.median(oeps) - 1) < 0.1
    assert abs(np.median(fit.inv_metric) / np.median(ominv) - 1) < 0.15
    assert np.all(fit.draws[:, :, 3] >= 1) and np.all(fit.draws[:, :, 4] >= 1)
    # sampler diagnostics agree in distribution
    assert abs(fit.draws[:, :, 4].mean() / od[:, :, 4].mean() - 1) < 0.05


@pytest.mark.parametrize("mid,data,kw", [
    ("hier", workloads.eight_schools(), dict(delta=0.95)),
    ("funnel", workloads.funnel(K=10), dict(delta=0.9)),
    ("logistic", workloads.logistic(seed=3, N=500, D=5), {}),
    ("logistic", workloads.logistic(seed=4, N=5000, D=10), {}),
    ("varint", workloads.varint(seed=9, J=8, K=3), {}),
    ("horseshoe", workloads.horseshoe(seed=10, N=300, D=8, n_nonzero=2), dict(delta=0.95)),
], ids=lambda v: v if isinstance(v, str) else "")
def test_moments_match_oracle(mid, data, kw):
    gm, om = _pair(mid, data)
    C = 8
    fit = gm.sample(num_chains=C, seed=2024, **kw)
    od, _, _, _ = om.run_chains(C, threads=8, seed=2024, **kw)
    cons = np.array([[om.write_array(od[c, i, 7:]) for i in range(od.shape[1])] for c in range(C)])
    checked = 0
    for j in range(min(gm.num_constrained, 12)):
        x, y = fit.draws[:, :, 7 + j], cons[:, :, j]
        sx, sy = oracle.summary(x), oracle.summary(y)
        if mid != "funnel" and mid != "hier":
            assert sx["rhat"] < 1.01, (j, sx["rhat"])
        tol = 4.5 * np.hypot(sx["mcse"], sy["mcse"])
        assert abs(sx["mean"] - sy["mean"]) < tol, (gm.param_names[j], sx["mean"], sy["mean"], tol)
        checked += 1
    assert checked > 0


def test_seed_determinism():
    gm = gn.Model("hier", workloads.eight_schools())
    a = gm.sample(num_chains=2, seed=11, num_warmup=200, num_samples=100)
    b = gm.sample(num_chains=2, seed=11, num_warmup=200, num_samples=100)
    c = gm.sample(num_chains=2, seed=12, num_warmup=200, num_samples=100)
    assert np.array_equal(a.draws, b.draws)
    assert not np.array_equal(a.draws, c.draws)
    lg = gn.Model("logistic", workloads.logistic(seed=4, N=5000, D=10))
    a = lg.sample(num_chains=4, seed=3, num_warmup=100, num_samples=50)
    b = lg.sample(num_chains=4, seed=3, num_warmup=100, num_samples=50)
    assert np.array_equal(a.draws, b.draws)


def test_autotuned_launch_shape_does_not_change_draws():
    """With 64 chains or more the fused driver times several launch shapes
    (chains per CTA, shared-memory cache) on the run's first gradients and
    keeps the fastest; every chain computes the same numbers under any shape,
    so runs are bitwise reproducible and equal to each chain run alone."""
    gm = gn.Model("hier", workloads.eight_schools())
    a = gm.sample(num_chains=96, seed=21, num_warmup=150, num_samples=60)
    b = gm.sample(num_chains=96, seed=21, num_warmup=150, num_samples=60)
    assert a.timing["chains_per_cta"] in (1, 2, 4)
    assert np.array_equal(a.draws, b.draws)
    # chain 40 alone (below the tuning threshold: the default shape) gives the same draws
    solo = gm.sample(num_chains=1, chain_id=41, seed=21, num_warmup=150, num_samples=60)
    assert np.array_equal(solo.draws[0], a.draws[40])


def test_chain_ids_offset_draws():
    gm = gn.Model("proper")
    a = gm.sample(num_chains=3, chain_id=10, seed=5, num_warmup=50, num_samples=20)
    b = gm.sample(num_chains=1, chain_id=11, seed=5, num_warmup=50, num_samples=20)
    np.testing.assert_array_equal(a.draws[1], b.draws[0])


def test_init_failure_reports_error():
    gm = gn.Model("funnel", workloads.funnel(K=3))
    with pytest.raises(gn.GnutsError) as e:
        gm.sample(num_chains=1, inits=np.array([-1e4, 1.0, 1.0, 1.0]), num_warmup=10, num_samples=10)
    assert e.value.code == gn.gnuts.ERR_INIT
    assert "Initialization failed" in e.value.msg


def test_user_inits_and_init_zero():
    gm = gn.Model("test_model")
    fit = gm.sample(num_chains=2, inits=np.array([1.0, -1.0]), adapt=False, num_warmup=0, num_samples=5, seed=1)
    assert fit.draws.shape == (2, 5, 9)
    fit = gm.sample(num_chains=1, init_radius=0.0, num_warmup=30, num_samples=5, seed=1)
    assert np.all(np.isfinite(fit.draws))


@pytest.mark.parametrize("N,D,n", [(10000, 100, 300), (4500, 37, 128), (8193, 103, 1)])
def test_tensor_core_gradient_close_to_fp64(N, D, n):
    """Tensor-core contraction (tcgen05) vs the FP64 oracle: coefficients
    split hi/lo in BF16 (lp), residuals in BF16 (gradient).  Tolerances: lp
    relative 1e-4 and gradient 2e-3 of its largest component at random points
    far from the mode; near the mode lp 1e-5 and gradient 3e-3."""
    data = workloads.logistic(seed=N, N=N, D=D)
    gm, om = _pair("logistic", data)
    rng = np.random.default_rng(N)
    q = rng.normal(0, 0.3, (n, gm.dim))
    lp, g = gm.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    for i in list(range(min(n, 6))) + [n - 1]:
        olp, og = om.log_prob_grad(q[i])
        assert abs(lp[i] - olp) <= 1e-4 * abs(olp), (i, lp[i], olp)
        assert np.max(np.abs(g[i] - og)) <= 2e-3 * np.max(np.abs(og)), (i, np.max(np.abs(g[i] - og)))
    # near the posterior mode the error is far smaller than the gradient noise scale
    qm = np.zeros((2, gm.dim))
    lp, g = gm.log_prob_grad(qm, precision=gn.PRECISION_MIXED)
    olp, og = om.log_prob_grad(qm[0])
    assert abs(lp[0] - olp) <= 1e-5 * abs(olp)
    assert np.max(np.abs(g[0] - og)) <= 3e-3 * np.max(np.abs(og))


@pytest.mark.parametrize("mid,data", [
    ("horseshoe", workloads.horseshoe(seed=11, N=8192, D=256, n_nonzero=6)),
    ("logistic", workloads.logistic(seed=12, N=8192, D=136)),
], ids=["horseshoe_256", "logistic_136"])
def test_wide_gradient_close_to_fp64(mid, data):
    """Designs wider than k_glm_tc's tile go through the two-kernel tcgen05
    path (k_wide_eta: eta with the likelihood epilogue fused, residuals BF16;
    k_wide_xtr: X^T r), coefficients split hi/lo, FP32 accumulation.  Same
    tolerances as the narrow tcgen05 path: lp relative 1e-4, gradient 2e-3 of
    its largest component; the FP64 path of the same points stays at 1e-10."""
    gm, om = _pair(mid, data)
    rng = np.random.default_rng(17)
    q = rng.normal(0, 0.3, (9, gm.dim))
    lp, g = gm.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    lp64, g64 = gm.log_prob_grad(q)
    for i in range(q.shape[0]):
        olp, og = om.log_prob_grad(q[i])
        assert abs(lp[i] - olp) <= 1e-4 * abs(olp), (i, lp[i], olp)
        assert np.max(np.abs(g[i] - og)) <= 2e-3 * np.max(np.abs(og)), (i, np.max(np.abs(g[i] - og)))
        assert abs(lp64[i] - olp) <= 1e-10 * abs(olp)


def test_wide_gradient_ragged_shapes():
    """Row count off every tile size (3001 rows: 256-row blocks of the eta
    kernel, 64-row chunks of the X^T r kernel), predictors off the 64-column
    chunk (200), and 130 chains: a second chain tile holding two chains."""
    data = workloads.logistic(seed=14, N=3001, D=200)
    gm, om = _pair("logistic", data)
    q = np.random.default_rng(19).normal(0, 0.2, (130, gm.dim))
    lp, g = gm.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    assert np.all(np.isfinite(lp)) and np.all(np.isfinite(g))
    for i in (0, 1, 63, 127, 128, 129):
        olp, og = om.log_prob_grad(q[i])
        assert abs(lp[i] - olp) <= 1e-4 * abs(olp), (i, lp[i], olp)
        assert np.max(np.abs(g[i] - og)) <= 2e-3 * np.max(np.abs(og)), (i, np.max(np.abs(g[i] - og)))
    # same points again: the kernels' sums run in a fixed order
    lp2, g2 = gm.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    assert np.array_equal(lp, lp2) and np.array_equal(g, g2)


def test_wide_sampler_moments_match_oracle():
    """NUTS on the tcgen05 wide-design gradient: moments agree with the
    FP64 oracle's chains within 4.5 combined MCSE."""
    data = workloads.logistic(seed=22, N=8192, D=136)
    gm, om = _pair("logistic", data)
    fit = gm.sample(num_chains=64, seed=5, precision=gn.PRECISION_MIXED, num_warmup=300, num_samples=300)
    od, _, _, _ = om.run_chains(16, threads=16, seed=5, num_warmup=300, num_samples=300)
    for j in range(0, gm.num_constrained, 7):
        x, y = fit.draws[:, :, 7 + j], od[:, :, 7 + j]
        sx, sy = oracle.summary(x), oracle.summary(y)
        assert sx["rhat"] < 1.02
        assert abs(sx["mean"] - sy["mean"]) < 4.5 * np.hypot(sx["mcse"], sy["mcse"]), gm.param_names[j]


def test_tensor_core_sampler_moments_match_oracle():
    data = workloads.logistic(seed=21, N=6000, D=10)
    gm, om = _pair("logistic", data)
    C = 128
    fit = gm.sample(num_chains=C, seed=5, precision=gn.PRECISION_MIXED, num_warmup=500, num_samples=500)
    od, _, _, _ = om.run_chains(16, threads=16, seed=5, num_warmup=500, num_samples=500)
    for j in range(gm.num_constrained):
        x, y = fit.draws[:, :, 7 + j], od[:, :, 7 + j]
        sx, sy = oracle.summary(x), oracle.summary(y)
        assert sx["rhat"] < 1.01
        assert abs(sx["mean"] - sy["mean"]) < 4.5 * np.hypot(sx["mcse"], sy["mcse"]), gm.param_names[j]
        assert abs(sx["sd"] / sy["sd"] - 1) < 0.1


def test_fp32_batched_gradient_close_to_fp64():
    data = workloads.logistic(seed=4, N=8192, D=32)
    gm, om = _pair("logistic", data)
    q = np.random.default_rng(1).normal(0, 0.2, (3, gm.dim))
    fit = gm.sample(num_chains=4, seed=1, num_warmup=150, num_samples=100, precision=gn.PRECISION_MIXED)
    assert np.all(np.isfinite(fit.draws))
    lp, g = gm.log_prob_grad(q)
    for i in range(3):
        olp, og = om.log_prob_grad(q[i])
        assert abs(lp[i] - olp) < 1e-9 * abs(olp)
