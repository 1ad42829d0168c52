"""Every CUDA / C++ source of the library is compiled by the build recipe
(cmdstan_gb300/build.py), exactly once per variant list, and every source the
recipe names exists; build() links them into libgnuts.so."""
import os

from cmdstan_gb300 import build

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cmdstan_gb300", "csrc")


def test_every_source_is_built_once():
    listed = list(build.CU_SOURCES) + list(build.CU_KIND_SOURCES) + [build.ADVANCE_SOURCE] + list(build.CPP_SOURCES)
    assert len(listed) == len(set(listed))
    on_disk = {f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))}
    assert set(listed) == on_disk, (sorted(on_disk - set(listed)), sorted(set(listed) - on_disk))


def test_variant_lists():
    # one round-mode state-machine object per (metric, team width): diag, dense, unit x warp, team
    assert sorted(build.ADVANCE_VARIANTS) == sorted((m, tw) for m in (0, 1, 2) for tw in (32, 128))
    assert build.N_KINDS == 7
