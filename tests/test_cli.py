"""The gnuts-sample command line: CmdStan argument grammar and Stan CSV output.

Mirrors the reference's interface tests: argument errors and exit codes
(src/test/interface/command_test.cpp, arguments/*_test.cpp), the CSV layout of
src/test/interface/example_output/bernoulli_chain_1.csv (config header,
column header, adaptation block, elapsed-time trailer; kept as a golden
fixture), output file naming for several chains (file.hpp make_filenames),
the metric JSON (save_metric_json_test.cpp) and metric files with
adaptation off (metric_test.cpp).
"""
import json
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "cmdstan_gb300", "_lib", "gnuts-sample")
GOLDEN = os.path.join(ROOT, "tests", "golden", "bernoulli_chain_1.json")
BERN_DATA = {"N": 10, "y": [0, 1, 0, 0, 0, 0, 0, 0, 0, 1]}


def run(args, cwd):
    r = subprocess.run([EXE] + args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    return r.returncode, r.stdout, r.stderr


def key_lines(lines):
    """config lines reduced to indent + key (values and (Default) dropped)"""
    out = []
    for l in lines:
        l = l[2:] if l.startswith("# ") else l
        out.append(l.split(" = ")[0].rstrip())
    return out


def is_subsequence(small, big):
    it = iter(big)
    return all(any(x == y for y in it) for x in small)


# ------------------------------------------------------------------ CPU
def test_no_arguments_prints_usage_and_fails(tmp_path):
    rc, out, _ = run(["model=bernoulli"], tmp_path)
    assert rc == 1 and "Usage" in out


def test_help_exits_zero(tmp_path):
    rc, out, _ = run(["model=bernoulli", "sample", "help"], tmp_path)
    assert rc == 0 and "Usage" in out


@pytest.mark.parametrize("args,msg", [
    (["sample", "num_samples=-1"], '-1 is not a valid value for "num_samples"'),
    (["sample", "adapt", "delta=1.5"], '1.5 is not a valid value for "delta"'),
    (["sample", "thin=0"], '0 is not a valid value for "thin"'),
    (["sample", "algorithm=hmc", "metric=diagonal"], 'diagonal is not a valid value for "metric"'),
    (["sample", "save_warmup=maybe"], 'maybe is not a valid value for "save_warmup"'),
    (["sample", "bogus=1"], "bogus=1 is either mistyped or misplaced."),
    (["num_samples=10"], "num_samples=10 is either mistyped or misplaced."),
    (["data", "file=x.json"], "A method must be specified!"),
    (["sample", "random", "seed=-5"], '-5 is not a valid value for "seed"'),
])
def test_argument_errors(tmp_path, args, msg):
    rc, _, err = run(["model=bernoulli"] + args, tmp_path)
    assert rc == 1
    assert msg in err
    if "method" not in msg:
        assert "Failed to parse command arguments, cannot run model." in err


def test_adapt_requires_warmup(tmp_path):
    rc, _, err = run(["model=bernoulli", "sample", "num_warmup=0"], tmp_path)
    assert rc == 1
    assert "must be greater than zero if adaptation is enabled" in err


def test_save_metric_requires_adaptation(tmp_path):
    rc, _, err = run(["model=bernoulli", "sample", "adapt", "engaged=0", "save_metric=1"], tmp_path)
    assert rc == 1 and "can only be enabled when adaptation is engaged" in err


def test_other_methods_are_refused(tmp_path):
    for m in ("optimize", "variational", "pathfinder"):
        rc, _, err = run(["model=bernoulli", m], tmp_path)
        assert rc == 1 and "not provided" in err


def test_missing_data_fails(tmp_path):
    rc, _, err = run(["model=bernoulli", "sample"], tmp_path)
    assert rc == 1 and "variable name=N" in err


def test_config_echo_follows_the_reference_tree(tmp_path):
    """The argument tree printed at start-up (and into the CSV header) holds
    every key of the reference's CSV header in the same order and nesting."""
    golden = json.load(open(GOLDEN))
    ref_keys = [k for k in key_lines(golden["config"])
                if not k.startswith(("stan_version", "model"))]
    _, out, _ = run(["model=bernoulli", "sample", "num_warmup=0", "adapt", "engaged=1"], tmp_path)
    ours = key_lines([l for l in out.splitlines() if l.strip()])
    assert is_subsequence(ref_keys, ours), (ref_keys, ours)


def test_config_echo_values(tmp_path):
    _, out, _ = run(["model=bernoulli", "method=sample", "num_samples=20", "num_warmup=0", "adapt", "delta=0.9",
                     "algorithm=hmc", "engine=nuts", "max_depth=7", "metric=dense_e", "num_chains=3",
                     "random", "seed=42", "output", "refresh=0"], tmp_path)
    lines = out.splitlines()
    assert "    num_samples = 20" in lines
    assert "      delta = 0.9" in lines
    assert "      gamma = 0.05 (Default)" in lines
    assert "            max_depth = 7" in lines
    assert "        metric = dense_e" in lines
    assert "    num_chains = 3" in lines
    assert "  seed = 42" in lines
    assert "  refresh = 0" in lines
    # unvalued options (metric choices) print no line of their own
    assert not any(l.strip() == "dense_e" for l in lines)


# ------------------------------------------------------------------ GPU
def write_json(path, obj):
    with open(path, "w") as f:
        json.dump(obj, f)
    return str(path)


def read_csv(path):
    config, adapt, trailer, rows, names = [], [], [], [], None
    for line in open(path):
        line = line.rstrip("\n")
        if line.startswith("#"):
            (config if names is None else adapt if not rows else trailer).append(line)
        elif names is None:
            names = line.split(",")
        else:
            rows.append([float(v) for v in line.split(",")])
    return config, names, adapt, rows, trailer


@pytest.mark.gpu
def test_bernoulli_csv_layout_matches_reference(tmp_path):
    golden = json.load(open(GOLDEN))
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, out, err = run(["model=bernoulli", "sample", "data", "file=" + data, "random", "seed=1234",
                        "output", "file=b_out.csv"], tmp_path)
    assert rc == 0, err
    assert "Iteration: 2000 / 2000 [100%]  (Sampling)" in out
    config, names, adapt, rows, trailer = read_csv(tmp_path / "b_out.csv")
    assert names == golden["names"]
    assert config[0] == "# stan_version_major = 2"
    assert "# model = bernoulli_model" in config
    assert "#   file = " + data in config
    assert "#   seed = 1234" in config
    assert is_subsequence([k for k in key_lines(golden["config"]) if k != "model"], key_lines(config))
    # adaptation block: same four lines, numbers in the same format
    assert len(adapt) == len(golden["adaptation"]) == 4
    for ours, ref in zip(adapt, golden["adaptation"]):
        pat = re.sub(r"-?\d+(\.\d+)?(e[-+]\d+)?", "NUM", ref)
        assert re.sub(r"-?\d+(\.\d+)?(e[-+]\d+)?", "NUM", ours) == pat
    # trailer: blank comment, three elapsed-time lines, blank comment
    assert len(trailer) == len(golden["trailer"]) == 5
    for ours, ref in zip(trailer, golden["trailer"]):
        assert re.sub(r"\d+(\.\d+)?(e[-+]\d+)?", "T", ours) == re.sub(r"\d+(\.\d+)?(e[-+]\d+)?", "T", ref)
    assert len(rows) == 1000
    # draws: sampler columns in range, theta posterior Beta(3, 9)
    theta = [r[7] for r in rows]
    assert all(0 < t < 1 for t in theta)
    assert all(0 <= r[1] <= 1 and r[3] >= 1 and r[4] >= 1 and r[5] in (0, 1) for r in rows)
    mean = sum(theta) / len(theta)
    assert 0.2 < mean < 0.31
    # default output: 6 significant digits
    raw = [l for l in open(tmp_path / "b_out.csv") if l[0] not in "#l"]
    assert all(len(v.replace("-", "").replace(".", "").split("e")[0].lstrip("0")) <= 6
               for v in raw[0].strip().split(","))


@pytest.mark.gpu
def test_several_chains_write_numbered_files_and_metric_json(tmp_path):
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, out, err = run(["model=bernoulli", "sample", "num_samples=100", "num_warmup=200", "adapt", "save_metric=1",
                        "algorithm=hmc", "metric=dense_e", "num_chains=3", "id=7", "data", "file=" + data,
                        "output", "file=out.csv", "refresh=0", "sig_figs=9"], tmp_path)
    assert rc == 0, err
    for k in (7, 8, 9):
        config, names, adapt, rows, _ = read_csv(tmp_path / ("out_%d.csv" % k))
        assert len(rows) == 100
        assert adapt[2] == "# Elements of inverse mass matrix:"
        m = json.load(open(tmp_path / ("out_metric_%d.json" % k)))
        assert m["metric_type"] == "dense_e" and m["stepsize"] > 0
        assert len(m["inv_metric"]) == 1 and len(m["inv_metric"][0]) == 1
        txt = open(tmp_path / ("out_metric_%d.json" % k)).read()
        assert txt.count("[") == 2
        # the CSV's step size and the JSON's agree
        assert abs(float(adapt[1].split("=")[1]) - m["stepsize"]) <= 1e-5 * m["stepsize"]
    assert not os.path.exists(tmp_path / "out.csv")
    # sig_figs=9 widens the printed values
    line = [l for l in open(tmp_path / "out_7.csv") if l[0] not in "#l"][0]
    assert any(len(v.replace("-", "").replace(".", "")) > 7 for v in line.split(","))


@pytest.mark.gpu
@pytest.mark.parametrize("model,metric,inv,expected", [
    ("proper", "diag_e", [1.5], "# Diagonal elements of inverse mass matrix:\n# 1.5"),
    ("proper", "dense_e", [[1.5]], "# Elements of inverse mass matrix:\n# 1.5"),
    ("test_model", "diag_e", [1.5, 1.8], "# Diagonal elements of inverse mass matrix:\n# 1.5, 1.8"),
    ("test_model", "dense_e", [[1.5, 1], [1, 1.5]], "# Elements of inverse mass matrix:\n# 1.5, 1\n# 1, 1.5"),
])
def test_metric_file_without_adaptation(tmp_path, model, metric, inv, expected):
    """metric_test.cpp: with adaptation off the metric file's values and the
    given step size are written back unchanged."""
    mf = write_json(tmp_path / ("%s.%s_metric.json" % (model, metric)), {"inv_metric": inv})
    for warm in ("0", "100"):
        rc, _, err = run(["model=" + model, "method=sample", "num_samples=100", "num_warmup=" + warm, "adapt",
                          "engaged=0", "algorithm=hmc", "engine=nuts", "metric=" + metric, "metric_file=" + mf,
                          "stepsize=0.5", "output", "file=o.csv", "refresh=0"], tmp_path)
        assert rc == 0, err
        text = open(tmp_path / "o.csv").read()
        assert text.count(expected) == 1
        assert text.count("# Step size = 0.5") == 1
        assert "# Adaptation terminated" not in text


@pytest.mark.gpu
def test_init_file_and_bad_init(tmp_path):
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    good = write_json(tmp_path / "bern_init.json", {"theta": 0.1})
    rc, _, err = run(["model=bernoulli", "sample", "num_samples=50", "num_warmup=50", "data", "file=" + data,
                      "init=" + good, "output", "refresh=0"], tmp_path)
    assert rc == 0, err
    bad = write_json(tmp_path / "bern_init_bad.json", {"theta": 2.0})
    rc, _, err = run(["model=bernoulli", "sample", "num_samples=50", "num_warmup=50", "data", "file=" + data,
                      "init=" + bad, "output", "refresh=0"], tmp_path)
    assert rc == 1 and "theta" in err
    missing = write_json(tmp_path / "bern_init_missing.json", {"phi": 0.3})
    rc, _, err = run(["model=bernoulli", "sample", "data", "file=" + data, "init=" + missing], tmp_path)
    assert rc == 1 and "theta" in err


@pytest.mark.gpu
def test_per_chain_init_files(tmp_path):
    """get_vec_var_context: init=<base>.json with several chains reads
    <base>_<id+i>.json when the first of them exists."""
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    for k in (1, 2):
        write_json(tmp_path / ("bi_%d.json" % k), {"theta": 0.2 * k})
    rc, _, err = run(["model=bernoulli", "sample", "num_samples=20", "num_warmup=20", "num_chains=2", "data",
                      "file=" + data, "init=" + str(tmp_path / "bi.json"), "output", "refresh=0"], tmp_path)
    assert rc == 0, err
    assert os.path.exists(tmp_path / "output_1.csv") and os.path.exists(tmp_path / "output_2.csv")


# ------------------------------------------------------------------ log_prob / diagnose
def test_log_prob_needs_exactly_one_parameter_file(tmp_path):
    """log_prob_test.cpp:165-174 (no parameters) and command.hpp:422-431 (both given)"""
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, _, err = run(["model=bernoulli", "method=log_prob", "data", "file=" + data], tmp_path)
    assert rc == 1 and "No input parameter files provided" in err
    up = write_json(tmp_path / "up.json", {"params_r": [0.1]})
    rc, _, err = run(["model=bernoulli", "method=log_prob", "unconstrained_params=" + up,
                      "constrained_params=" + up, "data", "file=" + data], tmp_path)
    assert rc == 1 and "Cannot specify both" in err


@pytest.mark.gpu
def test_log_prob_constrained_csv_matches_oracle(tmp_path):
    """log_prob_test.cpp:140-163: the bernoulli model on the reference's
    fitted-parameters CSV (1000 draws, kept as tests/golden/bern_fitted_params.json)
    gives 1000 rows of lp__, g_theta; every value equals the FP64 oracle's at
    logit(theta) (the Jacobian included, as jacobian=true by default)."""
    import numpy as np
    import oracle
    with open(os.path.join(ROOT, "tests", "golden", "bern_fitted_params.json")) as f:
        g = json.load(f)
    csv = tmp_path / "fitted.csv"
    with open(csv, "w") as f:
        f.write("# fitted parameters\n" + ",".join(g["names"]) + "\n")
        for row in g["draws"]:
            f.write(",".join(repr(v) for v in row) + "\n")
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, out, err = run(["model=bernoulli", "method=log_prob", "constrained_params=" + str(csv), "data",
                        "file=" + data, "output", "file=lp.csv", "sig_figs=15"], tmp_path)
    assert rc == 0, err
    config, names, _, rows, _ = read_csv(tmp_path / "lp.csv")
    assert names == ["lp__", "g_theta"]
    assert len(rows) == 1000
    om = oracle.OracleModel("bernoulli", BERN_DATA)
    theta = np.array(g["draws"])[:, g["names"].index("theta")]
    for th, (lp, gt) in zip(theta, rows):
        olp, og = om.log_prob_grad([np.log(th / (1 - th))], jacobian=True)
        assert abs(lp - olp) <= 1e-12 * abs(olp) + 1e-12 and abs(gt - og[0]) <= 1e-12 * max(1, abs(og[0]))
    assert any("method = log_prob" in l for l in config)


@pytest.mark.gpu
def test_log_prob_unconstrained_json_and_jacobian(tmp_path):
    """params_r as one vector or an array of vectors (command_helper.hpp:520-558);
    jacobian=0 drops the change-of-variables term"""
    import numpy as np
    import oracle
    from cmdstan_gb300 import workloads
    d = workloads.eight_schools()
    data = write_json(tmp_path / "es.json", {k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in d.items()})
    rng = np.random.default_rng(2)
    q = rng.uniform(-1, 1, (3, 10))
    up = write_json(tmp_path / "up.json", {"params_r": q.tolist()})
    om = oracle.OracleModel("hier", d)
    for jac in (1, 0):
        rc, _, err = run(["model=hier", "method=log_prob", "unconstrained_params=" + up, "jacobian=%d" % jac,
                          "data", "file=" + data, "output", "file=lp%d.csv" % jac, "sig_figs=15"], tmp_path)
        assert rc == 0, err
        _, names, _, rows, _ = read_csv(tmp_path / ("lp%d.csv" % jac))
        assert names[0] == "lp__" and len(names) == 11 and names[1] == "g_mu"
        for qi, row in zip(q, rows):
            olp, og = om.log_prob_grad(qi, jacobian=bool(jac))
            assert abs(row[0] - olp) <= 1e-12 * abs(olp) + 1e-12
            assert np.allclose(row[1:], og, rtol=1e-12, atol=1e-12)
    bad = write_json(tmp_path / "short.json", {"params_r": [0.1, 0.2]})
    rc, _, err = run(["model=hier", "method=log_prob", "unconstrained_params=" + bad, "data", "file=" + data],
                     tmp_path)
    assert rc == 1 and "Incorrect number of unconstrained parameters" in err


@pytest.mark.gpu
def test_diagnose_gradient_report(tmp_path):
    """method=diagnose test=gradient (arg_test_gradient.hpp): the model
    gradient against central finite differences at the initial point; every
    error is within the default threshold for a correct model"""
    from cmdstan_gb300 import workloads
    d = workloads.eight_schools()
    data = write_json(tmp_path / "es.json", {k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in d.items()})
    rc, out, err = run(["model=hier", "method=diagnose", "test=gradient", "epsilon=1e-6", "error=1e-6", "data",
                        "file=" + data, "random", "seed=7", "output", "file=diag.csv"], tmp_path)
    assert rc == 0, err
    assert "TEST GRADIENT MODE" in out and "Log probability=" in out
    lines = [l for l in out.splitlines() if re.match(r"^\s+\d+\s", l)]
    assert len(lines) == 10
    for l in lines:
        idx, value, model, fd, error = l.split()
        assert abs(float(error)) < 1e-5, l
        assert abs(float(model) - float(fd)) < 1e-5 * max(1.0, abs(float(model))), l
    text = open(tmp_path / "diag.csv").read()
    assert "# TEST GRADIENT MODE" in text and "method = diagnose" in text


# ------------------------------------------------------------------ gpu options
def test_gpu_group_echo_and_learned_needs_diag_adapt(tmp_path):
    """The sampler's own options sit in a `gpu` group after CmdStan's
    arguments; learned=1 is refused outside diag_e with adaptation."""
    _, out, _ = run(["model=bernoulli", "sample", "num_warmup=0", "adapt", "engaged=1"], tmp_path)
    keys = key_lines([l for l in out.splitlines() if l.strip()])
    assert keys[-3:] == ["gpu", "  precision", "  learned"]
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, _, err = run(["model=bernoulli", "sample", "algorithm=hmc", "metric=dense_e", "data", "file=" + data,
                      "gpu", "learned=1"], tmp_path)
    assert rc == 1 and "learned=1 needs metric=diag_e" in err


@pytest.mark.gpu
def test_gpu_learned_run_writes_stan_csv(tmp_path):
    from cmdstan_gb300 import workloads
    d = workloads.eight_schools()
    data = write_json(tmp_path / "es.json", {k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in d.items()})
    rc, out, err = run(["model=hier", "sample", "num_samples=100", "num_warmup=200", "num_chains=32", "data",
                        "file=" + data, "random", "seed=3", "output", "file=lr.csv", "refresh=0", "gpu",
                        "learned=1"], tmp_path)
    assert rc == 0, err
    assert "Learned preconditioner:" in out
    config, names, adapt, rows, _ = read_csv(tmp_path / "lr_1.csv")
    assert names[:7] == ["lp__", "accept_stat__", "stepsize__", "treedepth__", "n_leapfrog__", "divergent__",
                         "energy__"] and names[7] == "mu"
    assert len(rows) == 100
    assert any(l.startswith("#   learned = true") or l.startswith("# ") and "learned = true" in l for l in config)


@pytest.mark.gpu
def test_diagnostic_file_per_chain(tmp_path):
    """diagnostic_file (command.hpp:225-247, multi_chain_test.cpp): one file per
    chain named like the output files, columns lp__ .. energy__, the
    unconstrained parameters, p_ and g_ of each; rows as the output file's."""
    data = write_json(tmp_path / "bern.data.json", BERN_DATA)
    rc, out, err = run(["model=bernoulli", "id=10", "sample", "num_samples=50", "num_warmup=100", "num_chains=2",
                        "data", "file=" + data, "output", "file=b.csv", "diagnostic_file=b_diag.csv", "refresh=0"],
                       tmp_path)
    assert rc == 0, err
    for k in (10, 11):
        _, names, _, rows, _ = read_csv(tmp_path / ("b_%d.csv" % k))
        lines = [l.strip() for l in open(tmp_path / ("b_diag_%d.csv" % k)) if not l.startswith("#")]
        header = lines[0].split(",")
        assert header[:7] == names[:7]
        assert header[7:] == ["theta", "p_theta", "g_theta"]
        drows = [[float(v) for v in l.split(",")] for l in lines[1:]]
        assert len(drows) == len(rows) == 50
        for d, r in zip(drows, rows):
            assert d[:7] == r[:7]
            # theta = inv_logit(q) (6 significant digits in both files)
            assert abs(1 / (1 + pow(2.718281828459045, -d[7])) - r[7]) <= 1e-5
