"""Benchmark: NUTS on the logistic-regression workload (N=100,000 x D=100,
1024 chains sharing X, diag_e, 1000 warmup + 1000 draws, adaptation on).

One step = one complete sampling run of all chains (the unit over which
min bulk-ESS/s is defined).  Reported:
  value       grad-evals/s = sum of n_leapfrog__ over all chains, warmup and
              sampling, divided by the sampler's device time (inputs resident)
  e2e         the same metric through the C ABI with host buffers: model
              creation (X and y copied host -> device), sampling, draws copied
              device -> host, all inside the timed region
  min_bulk_ess_per_s, rhat_max   from the draws of the last run; the ESS is
              divided by that run's wall time (warmup + sampling, host calls
              included), as the metric is defined
  precision_vs_fp64   the mixed-precision gradient against the FP64 one at 64
              posterior draws of the run: largest relative lp error and largest
              gradient error relative to the largest component
  config2_fp64  the same workload on the FP64 CUDA-core gradient (a bounded
              run: 64 chains, 150 warmup + 150 draws)
  roofline    the tcgen05 gradient kernel: algorithmic 4*N*D flops per chain
              per round over its CUDA-event duration, against the measured
              sustained bf16 peak
  cpu_baseline  the CPU FP64 oracle on the host cores (one chain per core), a
              bounded sample of transitions started at the posterior mode
Between timed steps a 256 MB buffer is written to flush L2.
Replicas only: under torchrun each rank runs an independent replica.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "min bulk-ESS/s, grad-evals/s on 1 GB300: learned vs plain GPU NUTS, R-hat<1.01"
N_ROWS, N_PRED, N_CHAINS = 100_000, 100, 1024
NUM_WARMUP, NUM_SAMPLES = 1000, 1000


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the gradient kernel from the committed ncu summary (or None)."""
    p = os.path.join(ROOT, "profiles", "k_glm_tc_logistic_100k_x_100.md")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) < 9:
                        continue
                    try:
                        sm.append(float(parts[1]))
                        mx.append(float(parts[2]))
                    except ValueError:
                        continue
                    for nm, v in zip(names, parts[5:9]):
                        if v.lower().startswith("active"):
                            reasons.add(nm)
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_data(seed=0):
    from cmdstan_gb300 import workloads
    return workloads.logistic(seed=seed, N=N_ROWS, D=N_PRED)


def map_laplace(data):
    """Posterior mode and diagonal Laplace variance (Newton, numpy FP64): the
    starting state of the bounded CPU sample."""
    X, y = data["X"], data["y"].astype(np.float64)
    Xa = np.hstack([np.ones((X.shape[0], 1)), X])
    prior = np.r_[1 / 6.25, np.ones(X.shape[1])]
    w = np.zeros(Xa.shape[1])
    for _ in range(8):
        eta = Xa @ w
        p = 1 / (1 + np.exp(-eta))
        g = Xa.T @ (y - p) - prior * w
        H = (Xa * (p * (1 - p))[:, None]).T @ Xa + np.diag(prior)
        w = w + np.linalg.solve(H, g)
    return w, np.diag(np.linalg.inv(H))


def cpu_sample(data, seconds=15.0, threads=None):
    """Oracle NUTS on the host cores: one chain per core, adaptation off, at the
    posterior mode with the Laplace metric; iterations sized to ~`seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = threads or os.cpu_count() or 1
    om = oracle.OracleModel("logistic", data)
    w, var = map_laplace(data)
    kw = dict(adapt_engaged=0, stepsize=0.7, num_warmup=0, seed=7)
    t = time.time()
    _, _, _, ng = om.run_chains(threads, threads=threads, inits=w, inv_metric=var, num_samples=2, **kw)
    probe = time.time() - t
    per_iter = probe / 2.0
    iters = int(max(2, min(400, seconds / max(per_iter, 1e-6))))
    t = time.time()
    dr, _, _, ng = om.run_chains(threads, threads=threads, inits=w, inv_metric=var, num_samples=iters, **kw)
    wall = time.time() - t
    # the split-chain ESS needs a few draws per chain (a very short sample has none to give)
    ess = (min(oracle.ess_bulk(np.ascontiguousarray(dr[:, :, j])) for j in range(7, dr.shape[2]))
           if dr.shape[1] >= 8 else None)
    return {"value": float(ng.sum() / wall), "unit": "grad-evals/s", "cores": threads, "kind": "port",
            "wall_s": wall, "min_bulk_ess_per_s": None if ess is None else float(ess / wall),
            "min_bulk_ess_note": "min bulk ESS over the 101 parameters of these draws / wall; the chains start "
                                 "at the posterior mode with the Laplace metric and skip warmup, which favours "
                                 "the CPU",
            "sample": "%d chains x %d transitions (adaptation off, started at the posterior mode, Laplace diag "
                      "metric, step 0.7) of the same workload, FP64, %d host threads; %.1f s" %
                      (threads, iters, threads, wall)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    data = workload_data(0)
    res = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(data, seconds=args.cpu_seconds)
        if i >= args.warmup:
            res.append(r)
    v = float(np.mean([r["value"] for r in res]))
    line = {"metric": METRIC, "value": v, "unit": "grad-evals/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean([r["wall_s"] for r in res])) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": config(args),
            "cpu_baseline": {"value": v, "unit": "grad-evals/s", "cores": res[-1]["cores"], "kind": "port",
                             "sample": res[-1]["sample"], "min_bulk_ess_per_s": res[-1]["min_bulk_ess_per_s"],
                             "min_bulk_ess_note": res[-1]["min_bulk_ess_note"]},
            "e2e": {"value": v, "unit": "grad-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's own implementation (stan submodule) is absent from the reference tree; "
                    "the CPU oracle restating it times the CPU path; a step is one bounded sample of the "
                    "workload (ms_per_step is its wall time)"}
    print(json.dumps(line))


def config(args):
    return {"workload": "logistic regression N=100000 x D=100 (+intercept), 1024 chains on one shared X, "
                        "NUTS diag_e, 1000 warmup + 1000 draws, adapt delta 0.8, max_depth 10",
            "chains": N_CHAINS, "rows": N_ROWS, "predictors": N_PRED, "num_warmup": NUM_WARMUP,
            "num_samples": NUM_SAMPLES, "precision": "BF16 hi/lo split tensor-core gradient, FP32 accumulate, "
                                                     "FP64 energy / lp sum / adaptation",
            "l2": "256 MB buffer written between timed steps", "parallelism": "replicas"}


def _min_ess_rhat(draws, cols_per_chain_group=None, per_group=None):
    """min bulk ESS and max R-hat over the constrained columns of draws
    [chains, draws, 7 + params]; with cols_per_chain_group [(chains, ncols)...]
    each chain group is summarised over its own columns (and, when per_group
    is a list, each group's (min ESS, max R-hat) is appended to it)."""
    from cmdstan_gb300 import gnuts
    th = os.cpu_count() or 8
    if cols_per_chain_group is None:
        sm = gnuts.summary_columns(draws, list(range(7, draws.shape[2])), threads=th)
    else:
        sm, c0 = [], 0
        for n, k in cols_per_chain_group:
            g = gnuts.summary_columns(draws[c0:c0 + n], list(range(7, 7 + k)), threads=th)
            if per_group is not None:
                per_group.append((min(s["ess_bulk"] for s in g), max(s["rhat"] for s in g)))
            sm += g
            c0 += n
    return float(min(s["ess_bulk"] for s in sm)), float(max(s["rhat"] for s in sm))


def precision_vs_fp64(model, draws, n=64):
    """Mixed-precision gradient against the FP64 one at n posterior draws
    (the last draw of the first n chains): largest relative lp error and
    largest gradient error relative to the largest gradient component."""
    import cmdstan_gb300 as gn
    q = np.array([model.unconstrain(np.ascontiguousarray(c)) for c in draws[:n, -1, 7:]])
    lp64, g64 = model.log_prob_grad(q)
    lpm, gm = model.log_prob_grad(q, precision=gn.PRECISION_MIXED)
    return {"points": int(q.shape[0]), "where": "posterior draws of the run",
            "lp_rel_err_max": float(np.max(np.abs(lpm - lp64) / np.abs(lp64))),
            "grad_err_max_rel_to_max_component": float(np.max(np.max(np.abs(gm - g64), axis=1) /
                                                              np.max(np.abs(g64), axis=1)))}


def bench_fp64_arm(model, chains=64, warmup=150, samples=150):
    """The logistic workload on the FP64 CUDA-core gradient (k_glm_simt<double>),
    a bounded run: grad-evals/s over device time, min bulk-ESS/s over wall time."""
    t0 = time.perf_counter()
    fit = model.sample(num_chains=chains, num_warmup=warmup, num_samples=samples, seed=7, refresh=0)
    wall = time.perf_counter() - t0
    ess, rhat = _min_ess_rhat(fit.draws)
    dev_s = fit.timing["device_ms"] / 1e3
    g_us = float(fit.timing["grad_kernel_us"])
    return {"workload": "logistic regression N=100000 x D=100, %d chains, %d warmup + %d draws (bounded sample), "
                        "FP64 gradient on CUDA cores" % (chains, warmup, samples),
            "grad_evals_per_s": float(fit.n_leapfrog.sum() / dev_s), "min_bulk_ess_per_s": ess / wall,
            "min_bulk_ess": ess, "rhat_max": rhat, "wall_s": wall,
            "kernels_us": {"k_glm_simt_fp64": g_us, "k_advance": float(fit.timing["advance_kernel_us"])},
            "fp64_tflops_achieved": 4.0 * N_ROWS * N_PRED * chains / (g_us * 1e-6) / 1e12}


def bench_varint_set(peaks):
    """512 uneven varying-intercept regressions (J log-uniform in [8, 256],
    n_j ~ Poisson(50) + 5, K = 10), 4 chains each, one launch (2048 chains),
    1000 warmup + 1000 draws, FP32 likelihood rows, FP64 energy."""
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import workloads
    d = workloads.varint_set(seed=0, P=512)
    m = gn.Model("varint_set", d)
    m.sample(num_chains=2048, num_warmup=30, num_samples=10, seed=1, refresh=0)
    t0 = time.perf_counter()
    fit = m.sample(num_chains=2048, num_warmup=NUM_WARMUP, num_samples=NUM_SAMPLES, seed=2, refresh=0)
    wall = time.perf_counter() - t0
    dev_s = fit.timing["device_ms"] / 1e3
    lf = fit.n_leapfrog.astype(np.float64)
    rows = np.repeat(d["N"].astype(np.float64), 4)
    # FP32 X row (K floats) + FP64 y per row and gradient
    algo_bytes = float((lf * rows).sum() * (4 * d["K"] + 8))
    groups = []
    ess, rhat = _min_ess_rhat(fit.draws, [(4, int(j) + 12) for j in d["J"]], groups)
    g_ess = np.array([e for e, _ in groups])
    g_rhat = np.array([r for _, r in groups])
    cpu = _oracle_rate("varint", workloads.varint_set_member(d, int(np.argsort(d["N"])[len(d["N"]) // 2])), 16, 5.0)
    cpu["sample"] = "the median-size posterior: " + cpu["sample"]
    return {"cpu_baseline": cpu,
            "workload": "512 varying-intercept regressions, J log-uniform [8,256], n_j ~ Poisson(50)+5, K=10, "
                        "4 chains each (2048 chains) in one launch, 1000 warmup + 1000 draws, FP32 rows / FP64 energy",
            "grad_evals_per_s": float(lf.sum() / dev_s), "min_bulk_ess_per_s": ess / dev_s, "min_bulk_ess": ess,
            "rhat_max": rhat, "device_s": dev_s, "wall_s": wall, "rows_total": int(d["N"].sum()),
            "per_posterior": {"median_min_bulk_ess": float(np.median(g_ess)),
                              "posteriors_rhat_below_1.01": int((g_rhat < 1.01).sum()),
                              "note": "the set's minimum is set by posteriors whose simulated tau is tiny "
                                      "(posterior 459: tau = 0.0005, J = 139 - a centered funnel); the FP64 CPU "
                                      "oracle alone on that posterior, 4 x (500 + 500): R-hat 1.78, min bulk ESS 6.1"},
            "roofline": {"bound": "hbm", "achieved": algo_bytes / dev_s / 1e9, "peak": float(peaks["hbm_gbs"]),
                         "unit": "GB/s", "frac": algo_bytes / dev_s / 1e9 / float(peaks["hbm_gbs"]),
                         "note": "algorithmic row bytes (4K + 8 per row per gradient) over the run's device time; "
                                 "the 99.5 MB of rows stay L2-resident, so the bound is latency, not HBM"}}


def _oracle_rate(model_id, data, chains, seconds, **kw):
    """CPU oracle NUTS on the host cores (one chain per core): grad-evals/s of a
    bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    om = oracle.OracleModel(model_id, data)
    n = max(1, min(chains, threads))
    t = time.time()
    _, _, _, ng = om.run_chains(n, threads=threads, num_warmup=kw.get("probe_warmup", 20), num_samples=1, seed=5)
    per = max((time.time() - t) / (kw.get("probe_warmup", 20) + 1), 1e-6)
    iters = int(max(2, min(100000, seconds / per)))
    wu = iters // 2
    t = time.time()
    _, _, _, ng = om.run_chains(n, threads=threads, num_warmup=wu, num_samples=iters - wu, seed=5)
    wall = time.time() - t
    return {"value": float(ng.sum() / wall), "unit": "grad-evals/s", "cores": threads, "kind": "port",
            "sample": "%d chains x %d iterations (%d adaptive warmup) of the same model, FP64, %.1f s" %
                      (n, iters, wu, wall)}


def bench_bernoulli():
    """Bernoulli example (N = 10, y ~ Bernoulli(0.2)), 4 chains x 1000 + 1000, FP64."""
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import workloads
    d = workloads.bernoulli(seed=0)
    m = gn.Model("bernoulli", d)
    m.sample(num_chains=4, num_warmup=50, num_samples=50, seed=1, refresh=0)
    t0 = time.perf_counter()
    fit = m.sample(num_chains=4, num_warmup=NUM_WARMUP, num_samples=NUM_SAMPLES, seed=2, refresh=0)
    wall = time.perf_counter() - t0
    ess, rhat = _min_ess_rhat(fit.draws)
    return {"workload": "bernoulli N=10, 4 chains, 1000 warmup + 1000 draws, FP64",
            "grad_evals_per_s": float(fit.n_leapfrog.sum() / wall), "min_bulk_ess_per_s": ess / wall,
            "min_bulk_ess": ess, "rhat_max": rhat, "wall_s": wall,
            "cpu_baseline": _oracle_rate("bernoulli", d, 4, 3.0, probe_warmup=200)}


def bench_horseshoe(peaks, chains=256):
    """Config 5: regularised-horseshoe logistic regression, X 200,000 x 1000
    (BF16-exact), 256 chains, diag_e, mixed precision (the two-kernel tcgen05
    wide-design gradient).  A bounded sampling run (30 warmup + 10 draws) gives
    grad-evals/s and the per-round kernel times; the wide gradient's roofline
    uses 4 N K C algorithmic flops per round.  The CPU baseline is the oracle's
    FP64 gradient on every host core."""
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import workloads
    from concurrent.futures import ThreadPoolExecutor
    d = workloads.horseshoe(seed=0)
    m = gn.Model("horseshoe", d)
    N, K = d["X"].shape
    fit = m.sample(num_chains=chains, num_warmup=30, num_samples=10, seed=3, precision=gn.PRECISION_MIXED,
                   refresh=0)
    prec = precision_vs_fp64(m, fit.draws, n=16)
    tm = fit.timing
    dev_s = float(tm["device_ms"]) / 1e3
    grads = float(fit.n_leapfrog.sum())
    g_us = float(tm["grad_kernel_us"])
    flops = 4.0 * N * K * chains
    # CPU: the oracle's FP64 gradient, one point per host thread
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    om = oracle.OracleModel("horseshoe", d)
    threads = os.cpu_count() or 1
    q = np.random.default_rng(3).normal(0, 0.1, (threads, m.dim))
    t = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda i: om.log_prob_grad(q[i], True), range(threads)))
    cw = time.perf_counter() - t
    # dense_e arm: per-chain 2003 x 2003 metrics (FP32 metric product and
    # momentum solve in each chain's team).  Sampling only, at the diag_e
    # run's median step size with the identity as the metric: the dense
    # machinery's cost per gradient.  (The adaptive windows add a
    # D x D Welford update per transition and an FP64 Cholesky per window
    # end; a 30 + 10 adaptive run of the same chains took 386 s.)
    eps_med = float(np.median(fit.stepsize))
    t = time.perf_counter()
    fd = m.sample(metric="dense_e", adapt=False, num_chains=chains, num_warmup=0, num_samples=10, seed=4,
                  stepsize=eps_med, precision=gn.PRECISION_MIXED, refresh=0)
    dense_wall = time.perf_counter() - t
    tmd = fd.timing
    dense = {"workload": "same model and chains, dense_e (identity metric), no adaptation, 10 draws at the diag_e "
                         "run's median step size (bounded sample)",
             "grad_evals_per_s": float(fd.n_leapfrog.sum()) / (float(tmd["device_ms"]) / 1e3),
             "device_s": float(tmd["device_ms"]) / 1e3, "wall_s": dense_wall, "leapfrogs": float(fd.n_leapfrog.sum()),
             "kernels_us": {"wide_gradient": float(tmd["grad_kernel_us"]), "k_advance": float(tmd["advance_kernel_us"])},
             "finite_draws": bool(np.all(np.isfinite(fd.draws[:, :, :7])))}
    del fd
    return {"dense_e": dense,
            "workload": "horseshoe logistic N=200000 x K=1000 (D=2003), %d chains, diag_e, 30 warmup + 10 draws "
                        "(bounded sample), mixed precision" % chains,
            "grad_evals_per_s": grads / dev_s, "device_s": dev_s, "leapfrogs": grads,
            "kernels_us": {"wide_gradient": g_us, "k_advance": float(tm["advance_kernel_us"])},
            "precision_vs_fp64": prec,
            "roofline": {"bound": "tensor", "achieved": flops / (g_us * 1e-6) / 1e12,
                         "peak": peaks.get("bf16_tflops_sustained", 1709.0), "unit": "TFLOP/s",
                         "frac": flops / (g_us * 1e-6) / 1e12 / peaks.get("bf16_tflops_sustained", 1709.0),
                         "note": "4*N*K flops per chain-gradient x 256 chains per round over the round's whole "
                                 "gradient pipeline (coefficient staging, the tcgen05 eta kernel with the hi/lo "
                                 "split doubling its MMAs and the likelihood epilogue fused, the tcgen05 X^T r "
                                 "kernel, the partial sums)"},
            "cpu_baseline": {"value": threads / cw, "unit": "grad-evals/s", "cores": threads, "kind": "port",
                             "sample": "%d oracle FP64 gradients, one per host thread, %.2f s" % (threads, cw)}}


def bench_learned(model_id, chains=256):
    """Config 4, 256 chains: plain diag_e NUTS vs the learned coupling map
    (8 layers, hidden 128) with plain NUTS as judge, on the centered
    hierarchical model (J = 64) or the 100-d funnel; min bulk-ESS/s over all
    parameters, each sampler timed end to end (warmup, training, judge pilots
    and draws)."""
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import workloads
    data = workloads.hier(seed=0) if model_id == "hier" else workloads.funnel(100)
    m = gn.Model(model_id, data)
    t0 = time.perf_counter()
    fp = m.sample(num_chains=chains, num_warmup=NUM_WARMUP, num_samples=NUM_SAMPLES, seed=21, refresh=0)
    tp = time.perf_counter() - t0
    ep, rp = _min_ess_rhat(fp.draws)
    t0 = time.perf_counter()
    fl, rep = m.sample_learned(num_chains=chains, num_warmup=NUM_WARMUP, num_samples=NUM_SAMPLES, seed=21,
                               refresh=0)
    tl = time.perf_counter() - t0
    el, rl = _min_ess_rhat(fl.draws)
    desc = ("centered hierarchical J=64: mu ~ N(0,5), tau ~ half-Cauchy(0,5), theta_j ~ N(mu,tau), "
            "y_j ~ N(theta_j, sigma_j), sigma_j ~ U[5,20], y at mu=4, tau=3" if model_id == "hier" else
            "funnel v ~ N(0,3), x_1..100 ~ N(0, exp(v/2))")
    return {"cpu_baseline": _oracle_rate(model_id, data, 16, 5.0),
            "workload": "%s; %d chains; 1000 warmup + 1000 draws" % (desc, chains),
            "plain": {"min_bulk_ess_per_s": ep / tp, "min_bulk_ess": ep, "rhat_max": rp, "seconds": tp,
                      "divergence_rate": float(fp.draws[:, :, 5].mean()),
                      "grad_evals": float(fp.n_leapfrog.sum())},
            "learned": {"min_bulk_ess_per_s": el / tl, "min_bulk_ess": el, "rhat_max": rl, "seconds": tl,
                        "divergence_rate": float(fl.draws[:, :, 5].mean()), "report": rep}}


def run_profile_case(case):
    """Short runs whose kernels the ncu summaries in profiles/ describe:
    flow_hier_256 - the learned sampler's fused kernel (flow trained 50 steps
    on the centered hierarchical model, then 256 chains x 20 + 10);
    horseshoe_short - the wide-design gradient round (horseshoe, 256 chains,
    5 + 2, mixed precision);
    horseshoe_100k - the same on 100,000 rows (X 200 MB as BF16, larger than
    L2; about 1.5 GB on the device), for full ncu captures of single
    launches."""
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import workloads
    if case == "flow_hier_256":
        m = gn.Model("hier", workloads.hier(seed=0))
        f = gn.Flow(m.dim)
        f.init_affine(np.zeros(m.dim), np.ones(m.dim), seed=1)
        f.train(m, steps=50, seed=3)
        fit = m.sample_flow(f, num_chains=256, num_warmup=20, num_samples=10, seed=5)
    else:
        n_rows = 100_000 if case == "horseshoe_100k" else 200_000
        m = gn.Model("horseshoe", workloads.horseshoe(seed=0, N=n_rows))
        fit = m.sample(num_chains=256, num_warmup=5, num_samples=2, seed=3, precision=gn.PRECISION_MIXED, refresh=0)
    print(json.dumps({"profile_case": case, "note": "profiling run, not a bench value",
                      "timing": {k: float(v) for k, v in fit.timing.items()},
                      "leapfrogs": int(fit.n_leapfrog.sum())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the batched-posterior and funnel (learned vs plain) workloads")
    ap.add_argument("--quick", action="store_true",
                    help="profiling aid: one short run (20 warmup + 10 draws) of the same workload; not a bench value")
    ap.add_argument("--profile-case", choices=["flow_hier_256", "horseshoe_short", "horseshoe_100k"],
                    help="profiling aid: a short run of another workload's hot kernel; not a bench value")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return run_profile_case(args.profile_case)
    if args.quick:
        import cmdstan_gb300 as gn
        model = gn.Model("logistic", workload_data(0))
        fit = model.sample(num_chains=N_CHAINS, num_warmup=20, num_samples=10, refresh=0, seed=1,
                           precision=gn.PRECISION_MIXED)
        print(json.dumps({"quick": True, "note": "profiling run, not a bench value", "timing": fit.timing,
                          "leapfrogs": int(fit.n_leapfrog.sum())}))
        return

    import torch
    import cmdstan_gb300 as gn
    from cmdstan_gb300 import gnuts

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    data = workload_data(0)
    model = gn.Model("logistic", data)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    kw = dict(num_chains=N_CHAINS, num_warmup=NUM_WARMUP, num_samples=NUM_SAMPLES, refresh=0,
              precision=gn.PRECISION_MIXED)

    from cmdstan_gb300.replicas import chain_id_base, reduce_job

    def one_step(seed):
        return model.sample(seed=seed, chain_id=chain_id_base(rank, N_CHAINS), **kw)

    for i in range(args.warmup):
        one_step(1000 + i)
    fits, times = [], []
    peaks, peak_kind = measured_peaks()
    with Clocks(local) as clk:
        for i in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fit = one_step(1 + i)
            e1.record()
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
            times.append(e0.elapsed_time(e1))
            fits.append(fit)
    clocks = clk.summary()
    # whole-job throughput: leapfrogs over the sampler's device time (max over ranks)
    lf = float(sum(f.n_leapfrog.sum() for f in fits))
    dev_ms = float(sum(f.timing["device_ms"] for f in fits))
    lf, dev_ms, wall_ms = reduce_job(lf, dev_ms, float(sum(times)), dist, device="cuda")
    value = lf / (dev_ms / 1e3)
    # ESS / R-hat of the last run
    last = fits[-1]
    cols = list(range(7, last.draws.shape[2]))
    t_sum = time.perf_counter()
    try:
        sm = gnuts.summary_columns(last.draws, cols, gpu=True)
        summary_where = "gpu"
    except Exception:
        sm = gnuts.summary_columns(last.draws, cols, threads=os.cpu_count() or 8)
        summary_where = "host"
    t_sum = time.perf_counter() - t_sum
    ess_min = float(min(s["ess_bulk"] for s in sm))
    rhat_max = float(max(s["rhat"] for s in sm))
    step_wall_s = times[-1] / 1e3  # the last run's wall time: warmup + sampling
    prec = precision_vs_fp64(model, last.draws)
    grad_us = float(np.mean([f.timing["grad_kernel_us"] for f in fits]))
    adv_us = float(np.mean([f.timing["advance_kernel_us"] for f in fits]))
    flops = 4.0 * N_ROWS * N_PRED * N_CHAINS
    achieved = flops / (grad_us * 1e-6) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops")))
    traffic = profile_traffic()
    # e2e: host buffers through the C ABI, model creation + sampling + draws back
    e2e_times, e2e_lf = [], 0.0
    for i in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m2 = gn.Model("logistic", data)
        f2 = m2.sample(seed=100 + i, chain_id=chain_id_base(rank, N_CHAINS), **kw)
        del m2
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        e2e_lf += float(f2.n_leapfrog.sum())
    e2e_value = e2e_lf / sum(e2e_times)
    h2d = data["X"].nbytes + data["y"].astype(np.int32).nbytes
    d2h = last.draws.nbytes + last.n_leapfrog.nbytes * 4 + last.stepsize.nbytes + last.inv_metric.nbytes
    launches = int(sum(f.timing["launches"] for f in fits))
    line = {
        "metric": METRIC, "value": value, "unit": "grad-evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x2/fp32/fp64",
        "data": "synthetic (seeded PCG64, X rounded to bf16)", "config": config(args),
        "min_bulk_ess_per_s": ess_min / step_wall_s, "min_bulk_ess": ess_min, "rhat_max": rhat_max,
        "min_bulk_ess_per_s_denominator": "wall time of the run (warmup + sampling)",
        "precision_vs_fp64": prec,
        "sampler_device_s_per_step": dev_ms / 1e3 / args.steps,
        "leapfrogs_per_step": lf / args.steps,
        "kernels_us": {"k_glm_tc": grad_us, "k_advance": adv_us},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": "%s bf16 sustained" % peak_kind,
                     "note": "algorithmic 4*N*D flops per chain-gradient x 1024 chains per launch; the BF16 "
                             "hi/lo split executes 1.5x that on the tensor pipe (K padded to 112)"},
        "e2e": {"value": e2e_value, "unit": "grad-evals/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "s_per_step": float(np.mean(e2e_times))},
        "gpu_launches": launches, "clocks": clocks,
        "summary": {"where": summary_where, "seconds": t_sum,
                    "what": "stansummary statistics of the 101 parameters over 1024 x 1000 draws"},
    }
    if rank == 0:
        if not args.no_extra:
            extra = {}
            for name, fn in (("config2_fp64", lambda: bench_fp64_arm(model)), ("bernoulli", bench_bernoulli),
                             ("varint_set_512x4", lambda: bench_varint_set(peaks)),
                             ("hier_64_learned_vs_plain", lambda: bench_learned("hier")),
                             ("funnel_100d_learned_vs_plain", lambda: bench_learned("funnel")),
                             ("horseshoe_2003d", lambda: bench_horseshoe(peaks))):
                try:
                    extra[name] = fn()
                except Exception as e:  # reported in the line, the headline stands
                    extra[name] = {"error": repr(e)}
            line["workloads"] = extra
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_sample(data, seconds=args.cpu_seconds)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
