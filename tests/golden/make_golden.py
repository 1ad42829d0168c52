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

Usage: python tests/golden/make_golden.py /root/reference
"""
import json
import os
import sys


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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
