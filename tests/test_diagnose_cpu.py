"""gnuts_diagnose against the reference's diagnose-tool goldens.

src/test/interface/diagnose_test.cpp:11-98 runs bin/diagnose on the example
CSVs of src/test/interface/example_output and expects the .nom report texts;
tests/golden/make_golden.py extracted those draws (diag_<case>.npz) and texts
(<case>.nom).  Every case must reproduce its report exactly: treedepth
saturation at max_depth 10 / 8 / 15, the eight-schools divergences and
E-BFMI of 0.26, the two-chain mixture's R-hat list.
"""
import os

import numpy as np
import pytest

from cmdstan_gb300 import gnuts

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["corr_gauss", "corr_gauss_depth8", "corr_gauss_depth15", "eight_schools", "mix"]


def load_case(case):
    z = np.load(os.path.join(GOLD, "diag_%s.npz" % case))
    with open(os.path.join(GOLD, case + ".nom")) as f:
        nom = f.read()
    return z["draws"].astype(np.float64), [str(n) for n in z["names"]], int(z["max_depth"]), nom


@pytest.mark.parametrize("case", CASES)
def test_diagnose_report_matches_reference(case):
    draws, names, max_depth, nom = load_case(case)
    text, res = gnuts.diagnose(draws, names, max_depth=max_depth)
    assert text == nom, "\n--- got\n%s--- expected\n%s" % (text, nom)
    assert res["has_problems"] == (0 if "no problems detected" in nom else 1)


def test_diagnose_counts():
    draws, names, max_depth, _ = load_case("eight_schools")
    _, res = gnuts.diagnose(draws, names, max_depth=max_depth)
    assert res["n_divergent"] == 7 and res["n_treedepth_max"] == 0
    assert abs(res["e_bfmi"] - 0.26) < 0.005
    draws, names, max_depth, _ = load_case("corr_gauss_depth8")
    _, res = gnuts.diagnose(draws, names, max_depth=max_depth)
    assert res["n_treedepth_max"] == 424
    draws, names, max_depth, _ = load_case("mix")
    _, res = gnuts.diagnose(draws, names, max_depth=max_depth)
    assert res["n_high_rhat"] == 4 and res["n_low_ess"] == 0


def test_diagnose_flags_low_ess():
    # a parameter stuck at a few values in every chain: ESS per draw far below 0.001
    rng = np.random.default_rng(0)
    C, n = 4, 2000
    d = np.zeros((C, n, 8))
    d[:, :, 3] = 3
    d[:, :, 6] = rng.normal(size=(C, n))
    d[:, :, 7] = np.repeat(np.cumsum(rng.normal(size=(C, n // 500)), axis=1), 500, axis=1)
    names = ["lp__", "accept_stat__", "stepsize__", "treedepth__", "n_leapfrog__", "divergent__", "energy__", "x"]
    text, res = gnuts.diagnose(d, names)
    assert res["n_low_ess"] == 1 and "fewer than 0.001 effective draws per transition:\n  x\n" in text


def _write_csv(path, names, rows, max_depth):
    with open(path, "w") as f:
        f.write("# method = sample (Default)\n#             max_depth = %d\n" % max_depth)
        f.write(",".join(names) + "\n")
        for r in rows:
            f.write(",".join("%.9g" % v for v in r) + "\n")
        f.write("# \n#  Elapsed Time: 0.1 seconds (Warm-up)\n")


@pytest.mark.parametrize("case", ["eight_schools", "mix", "corr_gauss_depth8"])
def test_diagnose_cli_matches_reference(case, tmp_path):
    import subprocess
    draws, names, max_depth, nom = load_case(case)
    files = []
    for c in range(draws.shape[0]):
        p = tmp_path / ("out_%d.csv" % (c + 1))
        _write_csv(p, names, draws[c], max_depth)
        files.append(str(p))
    exe = os.path.join(os.path.dirname(gnuts.LIB_PATH), "gnuts-diagnose")
    r = subprocess.run([exe] + files, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout == nom


def test_diagnose_cli_usage_and_errors(tmp_path):
    import subprocess
    exe = os.path.join(os.path.dirname(gnuts.LIB_PATH), "gnuts-diagnose")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("USAGE:  diagnose <filename 1>")
    r = subprocess.run([exe, str(tmp_path / "missing.csv")], capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout == "File %s not found\nNo valid input files, exiting.\n" % (tmp_path / "missing.csv")
    bad = tmp_path / "bad.csv"
    bad.write_text("lp__,x\n1,2\n3\n")
    r = subprocess.run([exe, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith("Cannot parse input csv file: %s" % bad)
