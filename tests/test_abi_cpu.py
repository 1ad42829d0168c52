"""C-ABI checks that need no GPU: the library loads, exports every symbol of
include/gnuts.h, parses Stan JSON data, names parameters like CmdStan's CSV
header, and rejects bad arguments with CmdStan's messages."""
import ctypes
import os
import re

import numpy as np
import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import gnuts

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    lib = gn.load()
    with open(os.path.join(ROOT, "include", "gnuts.h")) as f:
        header = f.read()
    declared = set(re.findall(r"\b(gnuts_[a-z0-9_]+)\s*\(", header))
    assert declared == set(gnuts.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.gnuts_version().decode().startswith("gnuts")


def test_defaults_match_cmdstan():
    a = gn.default_args()
    # arg_sample.hpp / arg_adapt.hpp / arg_hmc.hpp / arg_nuts.hpp / arg_init.hpp defaults
    assert (a.num_samples, a.num_warmup, a.save_warmup, a.thin) == (1000, 1000, 0, 1)
    assert (a.gamma, a.delta, a.kappa, a.t0) == (0.05, 0.8, 0.75, 10.0)
    assert (a.init_buffer, a.term_buffer, a.window) == (75, 50, 25)
    assert (a.max_depth, a.stepsize, a.stepsize_jitter, a.init_radius) == (10, 1.0, 0.0, 2.0)
    assert a.refresh == 100


def test_json_data_and_names():
    # the bernoulli example data file of the reference's test models
    m = gn.Model("bernoulli", json_text='{\n    "N" : 10,\n    "y" : [0,1,0,0,0,0,0,0,0,1]\n}\n')
    assert (m.dim, m.num_constrained, m.param_names, m.name) == (1, 1, ["theta"], "bernoulli_model")
    m = gn.Model("hier", json_text='{"J" : 8, "y" : [28,8,-3,7,-1,1,18,12], '
                                   '"sigma" : [15,10,16,11,9,11,10,18], "tau" : 25}')
    assert m.param_names == ["mu"] + ["theta.%d" % j for j in range(1, 9)] + ["tau"]
    m = gn.Model("logistic", json_text='{"N":2,"D":3,"X":[[1,2,3],[4,5,6.5]],"y":[0,1]}')
    assert m.param_names == ["alpha", "beta.1", "beta.2", "beta.3"]
    m = gn.Model("test_model")
    assert m.param_names == ["mu1", "mu2"]
    m = gn.Model("horseshoe", {"N": 3, "D": 2, "X": np.ones((3, 2)), "y": np.array([0, 1, 1])})
    assert m.dim == 7 and m.num_constrained == 9
    assert m.param_names[-2:] == ["beta.1", "beta.2"]


def test_json_special_values_and_errors():
    m = gn.Model("hier", json_text='{"J":2,"y":[1.5,"Infinity"],"sigma":[1,2]}')
    assert m.dim == 4
    with pytest.raises(gn.GnutsError, match="ragged"):
        gn.Model("logistic", json_text='{"N":2,"D":2,"X":[[1,2],[3]],"y":[0,1]}')
    with pytest.raises(gn.GnutsError, match="variable name=y"):
        gn.Model("bernoulli", json_text='{"N":2}')
    with pytest.raises(gn.GnutsError, match="dimension"):
        gn.Model("bernoulli", json_text='{"N":3,"y":[0,1]}')
    with pytest.raises(gn.GnutsError, match="interval"):
        gn.Model("bernoulli", {"N": 2, "y": np.array([0, 2])})
    with pytest.raises(gn.GnutsError, match="unknown model"):
        gn.Model("no_such_model", {})


def test_unconstrain():
    m = gn.Model("hier", {"J": 2, "y": np.array([1.0, 2.0]), "sigma": np.array([1.0, 1.0])})
    q = m.unconstrain([0.5, 1.0, 2.0, 3.0])
    np.testing.assert_allclose(q, [0.5, 1.0, 2.0, np.log(3.0)])
    with pytest.raises(gn.GnutsError):
        m.unconstrain([0.5, 1.0, 2.0, -1.0])
    b = gn.Model("bernoulli", {"N": 1, "y": np.array([1])})
    with pytest.raises(gn.GnutsError, match="interval"):
        b.unconstrain([1.5])


@pytest.mark.parametrize("kw,msg", [
    (dict(num_warmup=0), "num_warmup"),          # command.hpp:569-574
    (dict(thin=0), "thin"),
    (dict(stepsize=0.0), "stepsize"),
    (dict(stepsize_jitter=1.5), "jitter"),
    (dict(max_depth=0), "max_depth"),
    (dict(delta=1.0), "delta"),
    (dict(num_chains=0), "num_chains"),
])
def test_argument_validation(kw, msg):
    m = gn.Model("proper")
    with pytest.raises(gn.GnutsError, match=msg) as e:
        m.sample(**kw)
    assert e.value.code == gnuts.ERR_ARGUMENT


def test_no_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    m = gn.Model("proper")
    with pytest.raises(gn.GnutsError) as e:
        m.sample(num_warmup=10, num_samples=10)
    assert e.value.code == gnuts.ERR_CUDA


def test_posterior_set_model_layout():
    """A posterior set is built on the host: shared parameters first, alpha
    columns up to the largest posterior."""
    from cmdstan_gb300 import workloads
    d = workloads.varint_set(seed=3, P=5, Jmax=30)
    m = gn.Model("varint_set", d)
    assert m.dim == int(d["J"].max()) + 12
    assert m.param_names[:12] == ["beta.%d" % k for k in range(1, 11)] + ["sigma_y", "tau"]
    assert m.param_names[12:] == ["alpha.%d" % j for j in range(1, int(d["J"].max()) + 1)]
    bad = dict(d)
    bad["group"] = d["group"].copy()
    bad["group"][0] = 1000
    with pytest.raises(gn.GnutsError):
        gn.Model("varint_set", bad)
