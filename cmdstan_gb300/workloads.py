"""Seeded synthetic data for the sampling workloads.

There is no public dataset behind these workloads: each one is generated
from a seed with numpy's PCG64, with the shapes and value distributions the
workload is defined by.  Design matrices are rounded to bfloat16-representable
values, so the FP64, FP32 and BF16 copies on the device hold the same matrix
and the mixed-precision path is exact on X (its error comes only from the
chains' coefficients and the accumulation).
"""
import numpy as np


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def round_bf16(x):
    """Round float64 values to the nearest bfloat16 (ties to even), as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bernoulli(seed=0, N=10, p=0.2):
    """theta ~ beta(1,1), y ~ bernoulli(theta); y drawn Bernoulli(p)."""
    y = (_rng(seed).random(N) < p).astype(np.int32)
    return {"N": N, "y": y}


def bernoulli_reference():
    """The bernoulli example data of the reference's test models (bern.data.json)."""
    return {"N": 10, "y": np.array([0, 1, 0, 0, 0, 0, 0, 0, 0, 1], dtype=np.int32)}


def logistic(seed=0, N=100_000, D=100, alpha=0.5):
    """X iid N(0,1) (bf16-representable), beta ~ N(0, 1/D), y ~ Bernoulli(inv_logit(alpha + X beta))."""
    g = _rng(seed)
    X = round_bf16(g.standard_normal((N, D)))
    beta = g.standard_normal(D) / np.sqrt(D)
    eta = alpha + X @ beta
    y = (g.random(N) < 1.0 / (1.0 + np.exp(-eta))).astype(np.int32)
    return {"N": N, "D": D, "X": X, "y": y}


def hier(seed=0, J=64, mu=4.0, tau=3.0):
    """Centered hierarchical normal: theta_j ~ N(mu, tau), sigma_j ~ U[5,20], y_j ~ N(theta_j, sigma_j)."""
    g = _rng(seed)
    theta = mu + tau * g.standard_normal(J)
    sigma = g.uniform(5.0, 20.0, J)
    y = theta + sigma * g.standard_normal(J)
    return {"J": J, "y": y, "sigma": sigma}


def eight_schools():
    """Data of the reference's eight_schools test model (eight_schools.data.json)."""
    return {"J": 8, "y": np.array([28., 8, -3, 7, -1, 1, 18, 12]),
            "sigma": np.array([15., 10, 16, 11, 9, 11, 10, 18])}


def funnel(K=100):
    return {"K": K}


def varint(seed=0, J=None, K=10, Jmin=8, Jmax=256):
    """One varying-intercept regression: J ~ log-uniform[Jmin, Jmax], n_j ~ Poisson(50)+5,
    x iid N(0,1), sigma_y ~ half-N(0,1), tau ~ half-N(0,1), y simulated."""
    g = _rng(seed)
    if J is None:
        J = int(round(np.exp(g.uniform(np.log(Jmin), np.log(Jmax)))))
    n = g.poisson(50, J) + 5
    N = int(n.sum())
    group = np.repeat(np.arange(1, J + 1), n).astype(np.int32)
    X = g.standard_normal((N, K))
    sigma_y = abs(g.standard_normal())
    tau = abs(g.standard_normal())
    alpha = tau * g.standard_normal(J)
    beta = g.standard_normal(K)
    y = alpha[group - 1] + X @ beta + sigma_y * g.standard_normal(N)
    return {"N": N, "J": J, "K": K, "group": group, "X": X, "y": y}


def horseshoe(seed=0, N=200_000, D=1000, n_nonzero=20):
    """Sparse logistic regression: X iid N(0,1) (bf16), 20 nonzero beta ~ N(0,2), rest 0."""
    g = _rng(seed)
    X = round_bf16(g.standard_normal((N, D)))
    beta = np.zeros(D)
    idx = g.choice(D, n_nonzero, replace=False)
    beta[idx] = 2.0 * g.standard_normal(n_nonzero)
    eta = X @ beta
    y = (g.random(N) < 1.0 / (1.0 + np.exp(-eta))).astype(np.int32)
    return {"N": N, "D": D, "X": X, "y": y, "scale_global": 0.01, "slab_scale": 2.0, "slab_df": 4.0}


def varint_set(seed=0, P=512, K=10, Jmin=8, Jmax=256):
    """P independent varying-intercept regressions (each drawn by varint() with
    its own seed) concatenated for one batched launch: rows of posterior p
    follow those of posterior p - 1."""
    parts = [varint(seed=1_000_003 * (seed + 1) + p, K=K, Jmin=Jmin, Jmax=Jmax) for p in range(P)]
    return {"P": P, "K": K, "J": np.array([q["J"] for q in parts], dtype=np.int32),
            "N": np.array([q["N"] for q in parts], dtype=np.int32),
            "group": np.concatenate([q["group"] for q in parts]).astype(np.int32),
            "X": np.concatenate([q["X"] for q in parts]), "y": np.concatenate([q["y"] for q in parts])}


def varint_set_member(data, p):
    """Posterior p of a varint_set data dict as a stand-alone varint data dict."""
    off = int(np.sum(data["N"][:p]))
    n = int(data["N"][p])
    return {"N": n, "J": int(data["J"][p]), "K": int(data["K"]), "group": data["group"][off:off + n],
            "X": data["X"][off:off + n], "y": data["y"][off:off + n]}
