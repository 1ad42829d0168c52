"""The Python binding's ctypes mirrors of the C-ABI structs (include/gnuts.h)
have the C layout: a small C program built against the header prints each
struct's size and field offsets, and they must equal the ctypes ones.  Also
the learned-sampler defaults as the library sets them.  No GPU needed."""
import ctypes
import os
import shutil
import subprocess

import pytest

import cmdstan_gb300 as gn
from cmdstan_gb300 import gnuts

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "gnuts_diagnosis": gnuts.Diagnosis,
    "gnuts_sample_args": gnuts.SampleArgs,
    "gnuts_var": gnuts.Var,
    "gnuts_output": gnuts.Output,
    "gnuts_train_args": gnuts.TrainArgs,
    "gnuts_learned_args": gnuts.LearnedArgs,
    "gnuts_learned_report": gnuts.LearnedReport,
}


def _c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gnuts.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    return got


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_ctypes_structs_match_the_header(tmp_path):
    c = _c_layout(tmp_path)
    for cname, py in STRUCTS.items():
        assert c[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert c[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_learned_defaults():
    la = gnuts.learned_args()
    assert (la.layers, la.hidden, la.clamp) == (8, 128, 6.0)
    assert (la.flow_warmup, la.flow_delta, la.pilot_samples) == (300, 0.95, 200)
    assert la.moment_tolerance == 4.0 and la.rhat_max == 1.01
    with pytest.raises(TypeError):
        gnuts.learned_args(not_a_field=1)
    assert gn.default_args().num_chains >= 1
