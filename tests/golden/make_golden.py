"""Extract the reference's example-output draws into compact golden fixtures.

Reads the Stan CSV fixtures that the reference's stansummary / diagnose tests
use (src/test/interface/example_output/*.csv under the reference checkout
given as argv[1]) and the fitted-parameters CSV of its log_prob tests
(src/test/test-models/bern_fitted_params.csv), and writes, for each, a JSON
file with the column names,
the draw matrix and the comment blocks (config header, adaptation block,
elapsed-time trailer).  The expected summary numbers are
the literal goldens of src/test/interface/stansummary_test.cpp (:481-495,
:622-637) and are written into the tests themselves.

It also writes the fixtures of the diagnose tool's tests
(src/test/interface/diagnose_test.cpp:11-98): for each case the sampler
columns and parameter draws of its example CSV files as a compressed array
(diag_<case>.npz: draws [chains, iterations, columns] in float32 -- the CSV
values carry six significant digits -- column names, max_depth from the
config block) and the expected report text (<case>.nom).

Usage: python tests/golden/make_golden.py <path of the reference checkout>
"""
import json
import os
import re
import sys

import numpy as np


def parse_stan_csv(path):
    """Column names, draws, and the comment blocks: the config header before
    the column names, the adaptation block between the names and the first
    draw, and the trailer after the last draw."""
    names, rows, config, adapt, trailer = None, [], [], [], []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if line.startswith("#"):
                if names is None:
                    config.append(line)
                elif not rows:
                    adapt.append(line)
                else:
                    trailer.append(line)
                continue
            if not line.strip():
                continue
            if names is None:
                names = line.split(",")
                continue
            rows.append([float(v) for v in line.split(",")])
    return names, rows, config, adapt, trailer


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    fixtures = [("src/test/interface/example_output", "bernoulli_chain_1"),
                ("src/test/interface/example_output", "eight_schools_output"),
                # the fitted-parameters CSV of the log_prob method tests (log_prob_test.cpp:140-163)
                ("src/test/test-models", "bern_fitted_params")]
    for sub, stem in fixtures:
        names, rows, config, adapt, trailer = parse_stan_csv(os.path.join(ref, sub, stem + ".csv"))
        out = {
            "source": "%s/%s.csv" % (sub, stem),
            "names": names,
            "draws": rows,
            "config": config,
            "adaptation": adapt,
            "trailer": trailer,
        }
        with open(os.path.join(here, stem + ".json"), "w") as f:
            json.dump(out, f, separators=(",", ":"))
        print(stem, len(rows), "draws x", len(names), "columns")


DIAGNOSE_CASES = [("corr_gauss", ["corr_gauss_output"]), ("corr_gauss_depth8", ["corr_gauss_output_depth8"]),
                  ("corr_gauss_depth15", ["corr_gauss_output_depth15"]), ("eight_schools", ["eight_schools_output"]),
                  ("mix", ["mix_output.1", "mix_output.2"])]


def diagnose_fixtures(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    ex = os.path.join(ref, "src/test/interface/example_output")
    for case, stems in DIAGNOSE_CASES:
        chains, names, max_depth = [], None, None
        for stem in stems:
            nm, rows, config, _, _ = parse_stan_csv(os.path.join(ex, stem + ".csv"))
            for line in config:
                m = re.search(r"max_depth = (\d+)", line)
                if m:
                    max_depth = int(m.group(1))
            names = nm
            chains.append(np.asarray(rows, dtype=np.float32))
        np.savez_compressed(os.path.join(here, "diag_%s.npz" % case), draws=np.stack(chains),
                            names=np.array(names), max_depth=np.int32(max_depth))
        with open(os.path.join(ex, case + ".nom")) as f, open(os.path.join(here, case + ".nom"), "w") as g:
            g.write(f.read())
        print("diagnose", case, np.stack(chains).shape, "max_depth", max_depth)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
    diagnose_fixtures(sys.argv[1])
