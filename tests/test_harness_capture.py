"""The suite's harness parsing a b200 program's real GB300 output.

tests/golden/b200_stdout_*.txt hold the stdout of b200 programs run at the
suite's size on a GB300 with PROFILING_FNAME set (capture_b200_stdout.sh).
Here the suite is assembled with the b200 target, the program of each test is
replaced by one that prints its capture, and the patched `benchmark` runs its
own report_test on it (benchmark:137-282).  Its b200 row must carry t_krn
(the mean of the "kernel time" lines, benchmark:174-178), nreg_krn (the
regcount line, :207-216), i_mean and f_mean from the capture.  The capture's
kernel times are host wall times around launch and device synchronisation,
as the reference's launch interposer measures them (cuda_profiling.cu:
239-249), so each is at least the sweep's device time printed beside it.

Needs the reference tree (the harness and the tests' sources); skipped where
it is absent.
"""
import os
import re
import stat
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITE = os.path.join(ROOT, "kernelgen-perf-tests_gb300", "suite")
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
from __graft_entry__ import reference_tree  # noqa: E402

REFERENCE = reference_tree()
CAPTURES = {   # test -> (capture, command line of the suite's size)
    "laplacian": ("b200_stdout_laplacian_512x256x256x10.txt", (512, 256, 256, 10)),
    "gameoflife": ("b200_stdout_gameoflife_512x65536x10.txt", (512, 256, 256, 10)),
    "tricubic2": ("b200_stdout_tricubic2_graph_512x256x256x10.txt", (512, 256, 256, 10)),
}


def floats(text, pattern):
    return [float(m) for m in re.findall(pattern, text)]


@pytest.mark.parametrize("name", sorted(CAPTURES))
def test_capture_lines(name):
    text = open(os.path.join(GOLDEN, CAPTURES[name][0])).read()
    krn = floats(text, r"%s kernel time = ([0-9.eE+-]+)" % name)
    dev = floats(text, r"%s device time = ([0-9.eE+-]+)" % name)
    assert len(krn) == len(dev) >= 1
    for k, d in zip(krn, dev):
        assert k >= d > 0
    assert re.search(r"%s regcount = \d+" % name, text)
    assert re.search(r"final mean = -?[0-9.]+\s", text)


@pytest.mark.skipif(not os.path.isdir(REFERENCE), reason="reference tree not present")
def test_harness_parses_captures(tmp_path):
    out = tmp_path / "suite"
    subprocess.run([os.path.join(SUITE, "assemble_suite.sh"), REFERENCE, str(out)], check=True,
                   capture_output=True)
    # a package stand-in whose b200 programs print the captures
    fake = tmp_path / "pkg"
    (fake / "build" / "bin").mkdir(parents=True)
    for name, (cap, _) in CAPTURES.items():
        prog = fake / "build" / "bin" / ("%s_b200" % name)
        prog.write_text("#!/bin/sh\ncat '%s'\n" % os.path.join(GOLDEN, cap))
        prog.chmod(prog.stat().st_mode | stat.S_IEXEC)
    (fake / "Makefile").write_text("all drivers:\n\t@true\n")   # the programs are already there
    (out / "makefile.b200.in").write_text("KG_ROOT ?= %s\n" % fake)
    # only the captured tests keep their b200 directory
    for d in os.listdir(out):
        b = out / d / "b200"
        if b.is_dir() and d not in CAPTURES:
            subprocess.run(["rm", "-r", str(b)], check=True)
    nx, ny, ns, nt = CAPTURES["laplacian"][1]
    res = subprocess.run(["./benchmark", str(nx), str(ny), str(ns), str(nt), "1", "b200"], cwd=out,
                         capture_output=True, text=True, timeout=600)
    rows = {}
    for ln in res.stdout.splitlines():
        f = [x.strip() for x in ln.split("|")]
        if len(f) >= 13 and f[2] == "b200":
            rows[f[1]] = f
    assert sorted(rows) == sorted(CAPTURES), res.stdout[-2000:]
    for name, (cap, _) in CAPTURES.items():
        text = open(os.path.join(GOLDEN, cap)).read()
        f = rows[name]
        i_mean, t_krn, nreg, f_mean = f[3], f[8], f[9], f[12]
        krn = floats(text, r"%s kernel time = ([0-9.eE+-]+)" % name)
        assert abs(float(t_krn) - sum(krn) / len(krn)) <= 1e-6 + 1e-3 * float(t_krn), (name, t_krn)
        assert int(float(nreg)) == int(re.search(r"%s regcount = (\d+)" % name, text).group(1))
        assert abs(float(i_mean) - float(re.search(r"initial mean = (-?[0-9.]+)", text).group(1))) < 1e-6
        assert abs(float(f_mean) - float(re.search(r"final mean = (-?[0-9.]+)", text).group(1))) < 1e-6
