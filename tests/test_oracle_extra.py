"""The oracle of the suite's other tests against the reference itself (CPU).

vecadd, matvec and whispering: the restatement (reference draws, time loop,
rotation, means) reproduces, bit for bit, the arrays of the reference kernel
compiled unmodified in strict mode, and the checksum lines its gcc target
prints (tests/golden/reference_extra.json, made by make_golden_extra.py);
the suite-size lines also equal README.md's published matvec and vecadd
rows.  matmul and sincos (Fortran kernels) are checked for their defining
properties only: parity unpinned.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest

import oracle_lib as ol

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_extra.json")))


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


CASES = [(t, i) for t in GOLD for i in range(len(GOLD[t]["cases"]))]


@pytest.mark.parametrize("test,idx", CASES, ids=["%s-%d" % c for c in CASES])
def test_extra_oracle_matches_reference_kernel(test, idx):
    case = GOLD[test]["cases"][idx]
    a, coef, im, fm = ol.extra_program(test, case["args"])
    assert [sha(x) for x in a] == case["output_sha256"]
    assert im == case["initial_mean"] and fm == case["final_mean"]
    if test == "whispering":
        assert coef == case["coef"]


RUNS = [(t, i) for t in GOLD for i in range(len(GOLD[t]["runs"])) if not GOLD[t]["runs"][i].get("readme_config")]


@pytest.mark.parametrize("test,idx", RUNS, ids=["%s-%d" % c for c in RUNS])
def test_extra_oracle_prints_reference_lines(test, idx):
    run = GOLD[test]["runs"][idx]
    a, coef, im, fm = ol.extra_program(test, run["args"])
    want = [ln for ln in run["lines"] if not ln.startswith("mu")]
    got = ["initial mean = %f" % im, "final mean = %f" % fm]
    for w, g in zip(want, got):
        # The gcc target is a fast-math build; whispering's fields grow to
        # 1e5 and more, where its last printed digit may differ.
        wv, gv = float(w.split("=")[1]), float(g.split("=")[1])
        assert w == g or abs(wv - gv) <= 1e-10 * abs(wv) + 1e-6, (w, g)


def test_readme_rows():
    """The suite-size gcc lines equal README.md's published cuda rows
    (i_mean, f_mean) for vecadd and matvec."""
    assert GOLD["vecadd"]["runs"][-1]["lines"] == ["initial mean = 0.000024", "final mean = -0.003702"]
    assert GOLD["matvec"]["runs"][-1]["lines"] == ["initial mean = 0.022473", "final mean = -0.036188"]


def test_matmul_oracle_properties():
    """C accumulates nt times the product, summed in k order."""
    a, _, im, fm = ol.extra_program("matmul", (7, 5, 3, 2))
    A = a[0].reshape(5, 7).T       # column-major A(i,k)
    B = a[1].reshape(3, 5).T       # B(k,j)
    C = a[2].reshape(3, 7).T
    assert np.allclose(C, 2 * (A @ B), rtol=1e-14, atol=1e-14)
    # k order: one column equals the sequential sum
    c = 0.0
    for k in range(5):
        c = c + A[2, k] * B[k, 1]
    c2 = c
    for k in range(5):
        c2 = c2 + A[2, k] * B[k, 1]
    assert C[2, 1] == c2


def test_sincos_oracle_properties():
    a, _, im, fm = ol.extra_program("sincos", (9, 4, 3, 2))
    x, y, xy = a
    assert np.array_equal(xy, np.array([math.sin(u) + math.cos(v) for u, v in zip(x, y)]))
