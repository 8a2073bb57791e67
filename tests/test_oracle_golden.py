"""Pin the oracle (CPU restatement) against the reference itself.

Fixtures under tests/golden/ were produced by tests/golden/make_golden.py from
the reference's own C sources compiled unmodified: array hashes from a strict
IEEE build of each kernel, printed checksum lines from the suite's gcc target
binary, and README.md's published checksum column.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as ol

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ARRAYS = json.load(open(os.path.join(GOLDEN, "reference_arrays.json")))
SUMS = json.load(open(os.path.join(GOLDEN, "reference_checksums.json")))


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def print_float(v):
    """benchmark:27-52: a value as the harness table prints it (8 chars)."""
    for width in range(6, -1, -1):
        s = "%.*g" % (width, v)
        if len(s) <= 8:
            return s
    raise ValueError(v)


def coef_lines(test, coef):
    if test == "laplacian":
        return ["alpha = %f, beta = %f" % tuple(coef)]
    if test in ("divergence", "gradient"):
        return ["alpha = %f, beta = %f, gamma = %f" % tuple(coef)]
    if test == "uxx1":
        return ["c1 = %f, c2 = %f" % tuple(coef)]
    if test == "wave13pt":
        return ["m0 = %f, m1 = %f, m2 = %f" % tuple(coef)]
    if test == "lapgsrb":
        return ["c0 = %f, c1 = %f, c2 = %f, c3 = %f" % tuple(coef)]
    if test == "gaussblur":
        return ["s0 = %f, s1 = %f, s2 = %f" % tuple(coef[:3]), "s4 = %f, s5 = %f, s8 = %f" % tuple(coef[3:])]
    return []


SMALL = [(t, i) for t in ARRAYS for i in range(len(ARRAYS[t]))]


@pytest.mark.parametrize("test,idx", SMALL, ids=["%s-%d" % x for x in SMALL])
def test_restatement_bitwise_vs_reference_kernel(test, idx):
    fx = ARRAYS[test][idx]
    case = ol.Case(test, fx["shape"])
    assert case.coef == fx["coef"]
    assert [sha(b) for b in case.arrays()] == fx["input_sha256"], "rand() draw order differs"
    case.run(fx["nt"])
    assert [sha(b) for b in case.arrays()] == fx["output_sha256"]
    assert case.final_mean() == fx["final_mean"]


SMALL_RUNS = [(t, r) for t in SUMS["runs"] for r in SUMS["runs"][t] if not r.get("readme_config")]


def expected_lines(test, case):
    lines = coef_lines(test, case.coef) + ["initial mean = %f" % case.initial_mean()]
    return lines


@pytest.mark.parametrize("test,run", SMALL_RUNS, ids=["%s-%s" % (t, "x".join(map(str, r["args"]))) for t, r in SMALL_RUNS])
def test_checksum_lines_vs_reference_binary(test, run):
    """The reference gcc binary (fast-math) prints the same lines as the oracle."""
    args = run["args"]
    shape, nt = args[:-1], args[-1]
    case = ol.Case(test, shape)
    pre = expected_lines(test, case)
    case.run(nt)
    got = pre + ["final mean = %f" % case.final_mean()]
    ref = [ln.rstrip() for ln in run["lines"]]
    assert sorted(got) == sorted(ref)


def test_bernoulli_conway_is_the_reference_rule():
    """Bernoulli(0.3) 0/1 cells: the reference FP64 rule thresholded at 0.5
    equals B3/S23 on bytes, sweep after sweep (bit-exact)."""
    nx, ny = 67, 45
    case = ol.Case("gameoflife", (nx, ny), variant=ol.INIT_BERNOULLI)
    u0, u1 = [b.copy() for b in case.arrays()]
    b0, b1 = ol.bernoulli_u8(nx * ny)
    assert np.array_equal(b0, u0.astype(np.uint8)) and np.array_equal(b1, u1.astype(np.uint8))
    for _ in range(12):
        case.run(1)
        b0, b1 = ol.conway_u8(b0, b1, nx, ny), b0
        newest = case.arrays()[0]
        assert np.array_equal((newest > 0.5).astype(np.uint8), b0)
        alive = newest[newest > 0.5]
        assert np.all(alive == 1.0)
        assert np.all(newest[newest <= 0.5] < 1e-19)


@pytest.mark.slow
@pytest.mark.parametrize("test", list(SUMS["runs"].keys()))
def test_readme_config_checksums(test):
    """benchmark 512 256 256 10: the oracle prints the reference binary's lines,
    and (where README.md has a row) the harness-formatted f_mean/i_mean of
    README.md:113-128."""
    run = [r for r in SUMS["runs"][test] if r.get("readme_config")][0]
    args = run["args"]
    case = ol.Case(test, args[:-1])
    pre = expected_lines(test, case)
    i_mean = case.initial_mean()
    case.run(args[-1])
    f_mean = case.final_mean()
    got = pre + ["final mean = %f" % f_mean]
    assert sorted(got) == sorted(ln.rstrip() for ln in run["lines"])
    row = SUMS["readme_cuda_t500"].get(test)
    if row and row["f_mean"] != "FAIL":
        # The harness parses the %f-printed line, then prints it with print_float.
        assert print_float(float("%f" % f_mean)) == row["f_mean"]
        assert print_float(float("%f" % i_mean)) == row["i_mean"]
