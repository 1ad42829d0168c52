"""Extract the reference's example-output draws into compact golden fixtures.

Reads the Stan CSV fixtures that the reference's stansummary / diagnose tests
use (src/test/interface/example_output/*.csv under the reference checkout
given as argv[1]) and writes, for each, a JSON file with the column names,
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
    src = os.path.join(ref, "src", "test", "interface", "example_output")
    for stem in ("bernoulli_chain_1", "eight_schools_output"):
        names, rows, config, adapt, trailer = parse_stan_csv(os.path.join(src, stem + ".csv"))
        out = {
            "source": "src/test/interface/example_output/%s.csv" % stem,
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
