"""The learned preconditioner on the GPU against the FP64 flow oracle.

The device flow computes in FP32 with BF16 weight matrices; the oracle is
given the same BF16-rounded matrices (and FP32-rounded biases, shifts and
log-scales), so the comparison measures FP32 arithmetic error only.
Tolerances: forward map 1e-4 relative, log-determinant 2e-3 absolute (a sum
of L * d FP32 log-scales), gradients 3e-3 of the largest component.  Then
the sampler on z is checked for exactness on a target with known moments,
training is checked to reduce the reverse-KL loss, and the learned service's
gain over plain NUTS (pilot ESS per gradient) and its judge rule are checked
on config 4's two models."""
import numpy as np
import pytest

import oracle
import cmdstan_gb300 as gn
from cmdstan_gb300 import workloads

pytestmark = pytest.mark.gpu


def _layout(fl):
    """(kind array) 0 = weight matrix entry (BF16 on the device), 1 = FP32 parameter."""
    d, L, H = fl.d, fl.L, fl.H
    kinds = []
    for l in range(L):
        nb = int(fl.mask(l).sum())
        na = d - nb
        kinds += [0] * (nb * H) + [1] * H + [0] * (H * 2 * na) + [1] * (2 * na)
    kinds += [1] * (2 * d)
    return np.array(kinds)


def _random_theta(fl, rng, w2=0.05, rho=0.2):
    kinds = _layout(fl)
    th = np.zeros(fl.n_params)
    o = 0
    for l in range(fl.L):
        nb = int(fl.mask(l).sum())
        na = fl.d - nb
        H = fl.H
        th[o:o + nb * H] = rng.normal(0, 0.7 / np.sqrt(nb), nb * H)
        o += nb * H
        th[o:o + H] = rng.normal(0, 0.1, H)
        o += H
        th[o:o + H * 2 * na] = rng.normal(0, w2, H * 2 * na)
        o += H * 2 * na
        th[o:o + 2 * na] = rng.normal(0, 0.05, 2 * na)
        o += 2 * na
    th[o:o + fl.d] = rng.normal(0, 0.5, fl.d)
    th[o + fl.d:] = rng.normal(0, rho, fl.d)
    # what the device holds: BF16 weight matrices, FP32 everything else
    th = np.where(kinds == 0, workloads.round_bf16(th), th.astype(np.float32).astype(np.float64))
    return th


@pytest.mark.parametrize("d,hidden", [(66, 128), (101, 128), (9, 32)])
def test_forward_inverse_logdet_match_oracle(d, hidden):
    rng = np.random.default_rng(d)
    of = oracle.OracleFlow(d, layers=8, hidden=hidden, clamp=4.0)
    f = gn.Flow(d, layers=8, hidden=hidden, clamp=4.0)
    assert f.n_params == of.n_params
    th = _random_theta(of, rng)
    f.set_params(th)
    assert np.array_equal(f.get_params(), th)
    z = rng.normal(size=(37, d))  # 37 points: a partial last CTA
    x, ld = f.forward(z)
    for i in range(z.shape[0]):
        ox, old = of.forward(th, z[i].astype(np.float32).astype(np.float64))
        assert np.allclose(x[i], ox, rtol=1e-4, atol=1e-4 * np.abs(ox).max()), i
        assert abs(ld[i] - old) < 2e-3, (i, ld[i], old)
    z2, ld2 = f.inverse(x)
    assert np.allclose(z2, z, atol=2e-4 * max(1.0, np.abs(z).max()))
    assert np.allclose(ld2, ld, atol=2e-3)


@pytest.mark.parametrize("model_id", ["funnel", "hier"])
def test_log_prob_grad_matches_oracle(model_id):
    rng = np.random.default_rng(11)
    data = workloads.funnel(100) if model_id == "funnel" else workloads.hier(seed=3)
    m, om = gn.Model(model_id, data), oracle.OracleModel(model_id, data)
    d = m.dim
    of = oracle.OracleFlow(d, layers=8, hidden=128, clamp=4.0)
    f = gn.Flow(d, layers=8, hidden=128, clamp=4.0)
    th = _random_theta(of, rng, w2=0.03, rho=0.1)
    f.set_params(th)
    z = rng.normal(0, 0.7, (6, d)).astype(np.float32).astype(np.float64)
    lp, gz, gth = f.log_prob_grad(m, z, param_grad=True)
    gsum = np.zeros(of.n_params)
    for i in range(z.shape[0]):
        olp, ogz, ogth, ox, olpx = of.log_prob_grad(om, th, z[i], param_grad=True)
        assert abs(lp[i] - olp) <= 1e-4 * abs(olp) + 1e-3, (i, lp[i], olp)
        assert np.abs(gz[i] - ogz).max() <= 3e-3 * np.abs(ogz).max(), i
        gsum += ogth
    assert np.abs(gth - gsum).max() <= 3e-3 * np.abs(gsum).max()


@pytest.mark.parametrize("model_id,hidden,n", [("funnel", 128, 37), ("hier", 128, 19), ("hier", 64, 5),
                                               ("funnel", 32, 3)])
def test_tensor_core_pass_matches_oracle(model_id, hidden, n):
    """The sampler's gradient pass (mma.sync contractions on BF16 weights with
    activations carried as three BF16 parts, FP32 accumulation) holds the
    same tolerances as the FP32 SIMT pass: lp 1e-4 relative + 1e-3, gradient
    3e-3 of its largest component; and it agrees with the SIMT pass."""
    rng = np.random.default_rng(hidden + n)
    data = workloads.funnel(100) if model_id == "funnel" else workloads.hier(seed=3)
    m, om = gn.Model(model_id, data), oracle.OracleModel(model_id, data)
    d = m.dim
    of = oracle.OracleFlow(d, layers=8, hidden=hidden, clamp=4.0)
    f = gn.Flow(d, layers=8, hidden=hidden, clamp=4.0)
    th = _random_theta(of, rng, w2=0.03, rho=0.1)
    f.set_params(th)
    z = rng.normal(0, 0.7, (n, d)).astype(np.float32).astype(np.float64)
    lp, gz = f.log_prob_grad_tc(m, z)
    lps, gzs = f.log_prob_grad(m, z)
    for i in range(n):
        olp, ogz = of.log_prob_grad(om, th, z[i])
        assert abs(lp[i] - olp) <= 1e-4 * abs(olp) + 1e-3, (i, lp[i], olp)
        assert np.abs(gz[i] - ogz).max() <= 3e-3 * np.abs(ogz).max(), i
    assert np.allclose(lp, lps, rtol=1e-5, atol=1e-3)
    assert np.abs(gz - gzs).max() <= 1e-3 * np.abs(gzs).max()


def test_adam_step_matches_oracle():
    rng = np.random.default_rng(5)
    of = oracle.OracleFlow(12, layers=4, hidden=32)
    f = gn.Flow(12, layers=4, hidden=32)
    th = _random_theta(of, rng)
    f.set_params(th)
    ref, m, v = th.copy(), np.zeros_like(th), np.zeros_like(th)
    for t in (1, 2, 3):
        g = rng.normal(size=th.size)
        f.adam_step(g, t, lr=1e-2)
        oracle.adam(ref, m, v, g, t, lr=1e-2)
    got = f.get_params()
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)


def test_training_reduces_reverse_kl_on_funnel():
    m = gn.Model("funnel", workloads.funnel(100))
    f = gn.Flow(m.dim, layers=8, hidden=128)
    scale = np.r_[3.0, np.full(100, 2.0)]
    f.init_affine(np.zeros(m.dim), scale, seed=1)
    trace = f.train(m, steps=400, batch=256, learning_rate=2e-3, seed=7, base_scale=1.0, anneal_fraction=0.0)
    assert np.all(np.isfinite(trace))
    first, last = trace[:20].mean(), trace[-20:].mean()
    assert last < first - 5.0, (first, last)


def test_flow_sampler_is_exact_on_gaussian():
    """NUTS on z through a non-trivial (random, untrained) flow must still
    sample the model's own distribution: x ~ N(0, diag(s^2))."""
    rng = np.random.default_rng(2)
    scales = np.array([0.1, 0.5, 1.0, 2.0, 5.0, 10.0])
    m = gn.Model("normal", {"scales": scales})
    of = oracle.OracleFlow(6, layers=4, hidden=32, clamp=2.0)
    f = gn.Flow(6, layers=4, hidden=32, clamp=2.0)
    th = _random_theta(of, rng, w2=0.05, rho=0.0)
    th[-6:] = np.log(scales)  # x = scale * u: the couplings perturb a unit-scale target
    f.set_params(th)
    fit = m.sample_flow(f, num_chains=64, num_warmup=400, num_samples=400, seed=3)
    assert np.all(fit.status == 0)
    for k, s in enumerate(scales):
        x = fit.draws[:, :, 7 + k]
        st = gn.summary(x)
        assert abs(st["mean"]) < 4.5 * st["mcse"] + 1e-12, (k, st)
        assert abs(st["sd"] / s - 1) < 0.08, (k, st["sd"], s)
        assert st["rhat"] < 1.05
    # lp__ is the model's lp at x: -0.5 sum (x/s)^2
    xs = fit.draws[:, :, 7:]
    assert np.allclose(fit.draws[:, :, 0], -0.5 * ((xs / scales) ** 2).sum(axis=2), rtol=1e-9, atol=1e-9)


def _judge_expects(rep, tol=4.0, rhat_max=1.01):
    clean = rep["plain_divergence_rate"] <= 1e-3
    return int(rep["flow_ess_per_grad"] >= rep["plain_ess_per_grad"]
               and rep["flow_divergence_rate"] <= rep["plain_divergence_rate"]
               and rep["flow_max_rhat"] <= max(rhat_max, rep["plain_max_rhat"])
               and (not clean or rep["max_moment_z"] <= tol))


@pytest.mark.parametrize("model_id", ["hier", "funnel"])
def test_learned_map_gain_and_judge(model_id):
    """Config 4, 256 chains: plain diag_e NUTS vs the learned coupling map (8
    layers, hidden 128) trained during warmup.  What the trained network
    gains is measured on the judge's pilots (min bulk-ESS per gradient); the
    map produces the draws only if the judge's rule holds, and the draws are
    valid either way."""
    data = workloads.hier(seed=0) if model_id == "hier" else workloads.funnel(100)
    m = gn.Model(model_id, data)
    fit, rep = m.sample_learned(num_chains=256, num_warmup=1000, num_samples=300, seed=21)
    assert rep["loss_last"] < rep["loss_first"], rep
    if model_id == "hier":
        # the centered hierarchy: the pulled-back space is far easier for NUTS
        assert rep["flow_ess_per_grad"] > 2.0 * rep["plain_ess_per_grad"], rep
    assert rep["used_flow"] == _judge_expects(rep), rep
    assert fit.draws.shape == (256, 300, 7 + m.num_constrained)
    assert np.all(np.isfinite(fit.draws))
    assert rep["final_grads"] == int(fit.n_leapfrog.sum())


def test_learned_judge_applies_its_rule():
    m = gn.Model("hier", workloads.eight_schools())
    fit, rep = m.sample_learned(num_chains=32, num_warmup=300, num_samples=100, seed=4,
                                learned=dict(train=dict(steps=100), pilot_samples=60, flow_warmup=60, hidden=32,
                                             layers=4))
    assert rep["used_flow"] == _judge_expects(rep), rep
    assert fit.draws.shape == (32, 100, 7 + m.num_constrained)
    assert np.all(np.isfinite(fit.draws))
