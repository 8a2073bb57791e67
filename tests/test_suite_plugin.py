"""The b200 target as a suite plug-in: assembly, discovery by the harness.

Needs the reference tree (assemble_suite.sh copies it); skipped where it is
absent.  Without a GPU the b200 programs stop at the device and the harness
reports their rows as FAIL; the test checks the harness found and ran them.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITE = os.path.join(ROOT, "kernelgen-perf-tests_gb300", "suite")
sys.path.insert(0, ROOT)
from __graft_entry__ import reference_tree  # noqa: E402

REFERENCE = reference_tree()
TESTS = ["laplacian", "divergence", "gradient", "uxx1", "wave13pt", "tricubic", "tricubic2",
         "jacobi", "lapgsrb", "gaussblur", "gameoflife"]


def test_overlay_files():
    for t in TESTS:
        assert open(os.path.join(SUITE, t, "b200", "kernel")).read().strip() == t
        mk = open(os.path.join(SUITE, t, "b200", "makefile")).read()
        assert "test:" in mk and "all:" in mk
        if t in ("jacobi", "gaussblur", "gameoflife"):
            assert "$$(($(NY) * $(NS)))" in mk


@pytest.mark.skipif(not os.path.isdir(REFERENCE), reason="reference tree not present")
def test_assemble_and_run_harness(tmp_path):
    out = tmp_path / "suite"
    subprocess.run([os.path.join(SUITE, "assemble_suite.sh"), REFERENCE, str(out)], check=True)
    assert (out / "laplacian" / "b200" / "makefile").exists()
    bench = (out / "benchmark").read_text()
    assert bench.count('($target eq "b200")') == 4
    res = subprocess.run(["./benchmark", "8", "8", "8", "1", "1", "b200"], cwd=out,
                         capture_output=True, text=True, timeout=600)
    for t in TESTS:
        assert "Found test %s" % t in res.stdout
    rows = [ln for ln in res.stdout.splitlines() if "|                  b200 |" in ln]
    assert len(rows) >= len(TESTS)
