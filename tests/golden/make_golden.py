#!/usr/bin/env python3
"""Generate the golden fixtures of this directory from the reference itself.

Needs the reference tree (KG_REFERENCE_TREE, else the build's default) and the builds
of its own C sources made by ``make -C oracle ref`` (oracle/_ref/).  The
fixtures are committed; nothing at test time reads the reference tree.

Outputs:
  reference_arrays.json     for small cases: SHA-256 of every buffer after nt
                            sweeps of the reference kernel compiled unmodified
                            in strict IEEE mode (-O2 -ffp-contract=off), driven
                            with the reference main()'s rand() order and
                            pointer rotation; plus the final mean, and the
                            normwise gap max|fast-strict|/max|strict| of the
                            suite's fast-math build of the same kernel.
  reference_checksums.json  stdout lines (coefficients, initial mean, final
                            mean) of the suite's gcc target binary (the
                            reference main(), makefile.in:28-29 flags) for the
                            small cases and for ``benchmark 512 256 256 10``,
                            plus README.md's published f_mean/i_mean column.
"""
import ctypes
import hashlib
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BUILD = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, ROOT)
from __graft_entry__ import reference_tree  # noqa: E402

REFERENCE = reference_tree()

libc = ctypes.CDLL("libc.so.6")
RAND_MAX = 2147483647

# name, number of arrays, coefficient draws (divisors), 2D?
TESTS = {
    "laplacian": (2, [1, 1], False),
    "divergence": (4, [1, 1, 1], False),
    "gradient": (4, [1, 1, 1], False),
    "uxx1": (6, [1, 1], False),
    "wave13pt": (3, [1, 6.0, 6.0], False),
    "tricubic": (5, [], False),
    "tricubic2": (5, [], False),
    "lapgsrb": (2, [1, 6.0, 12.0, 6.0], False),
    "gaussblur": (2, [1, 1, 1, 1, 1, 1], True),
    "gameoflife": (2, [], True),
}

SMALL_3D = [(3, 3, 3, 1), (4, 4, 4, 2), (5, 5, 5, 2), (7, 6, 5, 3), (33, 17, 9, 4),
            (64, 32, 32, 10), (129, 35, 20, 3)]
SMALL_2D = [(3, 3, 1), (5, 5, 2), (7, 9, 3), (33, 70, 4), (64, 1024, 10), (129, 300, 3)]


def real_rand():
    # laplacian/laplacian.c:112 with real = double
    return ((libc.rand() / float(RAND_MAX)) - 0.5) * 2


def make_inputs(test, shape):
    narr, divs, _ = TESTS[test]
    libc.srand(1)
    coef = []
    for d in divs:
        v = real_rand()
        coef.append(v / d if d != 1 else v)
    n = int(np.prod(shape))
    arrs = [np.empty(n, dtype=np.float64) for _ in range(narr)]
    for i in range(n):
        for q in range(narr):
            arrs[q][i] = real_rand()
    return coef, arrs


def call_kernel(lib, test, shape, coef, a):
    P = [x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for x in a]
    I = [ctypes.c_int(s) for s in shape]
    D = [ctypes.c_double(c) for c in coef]
    fn = getattr(lib, test)
    fn.restype = None
    fn(*I, *D, *P)


def run_case(lib, test, shape, nt, coef, arrs):
    a = [x.copy() for x in arrs]
    for _ in range(nt):
        call_kernel(lib, test, shape, coef, a)
        if test in ("divergence", "gradient"):
            pass
        elif test == "wave13pt":
            a = [a[1], a[2], a[0]]
        else:
            a[0], a[1] = a[1], a[0]
    return a


def final_mean(test, a):
    n = a[0].size
    if test == "gradient":
        s = 0.0
        for i in range(n):
            s += a[1][i] + a[2][i] + a[3][i]
        return s / n / 3
    slot = 0 if test == "divergence" else 1
    s = 0.0
    for v in a[slot]:
        s += float(v)
    return s / n


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def run_binary(test, args):
    exe = os.path.join(REF_BUILD, test + "_gcc")
    env = {k: v for k, v in os.environ.items() if k != "NO_TIMING"}
    out = subprocess.run([exe] + [str(x) for x in args], capture_output=True, text=True,
                         check=True, env=env).stdout
    keep = [ln for ln in out.splitlines()
            if re.match(r"^(initial mean|final mean|alpha|c0|c1|m0|s0|s4)\b", ln)]
    return keep


def readme_table():
    rows = {}
    with open(os.path.join(REFERENCE, "README.md")) as f:
        for ln in f:
            m = re.match(r"^\|\s*(\w+)\s*\|\s*cuda\s*\|(.*)\|\s*$", ln)
            if m:
                cols = [c.strip() for c in m.group(2).split("|")]
                rows[m.group(1)] = {"i_mean": cols[0], "t_krn": cols[5], "f_mean": cols[-1]}
    return rows


def main():
    arrays = {}
    sums = {}
    for test, (narr, divs, is2d) in TESTS.items():
        strict = ctypes.CDLL(os.path.join(REF_BUILD, "lib%s_strict.so" % test))
        fast = ctypes.CDLL(os.path.join(REF_BUILD, "lib%s_fast.so" % test))
        cases = SMALL_2D if is2d else SMALL_3D
        arrays[test] = []
        sums[test] = []
        for case in cases:
            shape, nt = case[:-1], case[-1]
            coef, arrs = make_inputs(test, shape)
            a = run_case(strict, test, shape, nt, coef, arrs)
            b = run_case(fast, test, shape, nt, coef, arrs)
            gap = 0.0
            for x, y in zip(a, b):
                m = float(np.max(np.abs(x))) if x.size else 0.0
                if m > 0:
                    gap = max(gap, float(np.max(np.abs(x - y))) / m)
            arrays[test].append({
                "shape": list(shape), "nt": nt, "coef": coef,
                "input_sha256": [sha(x) for x in arrs],
                "output_sha256": [sha(x) for x in a],
                "final_mean": final_mean(test, a),
                "fast_vs_strict_normwise": gap,
            })
            sums[test].append({"args": list(shape) + [nt], "lines": run_binary(test, list(shape) + [nt])})
            print(test, shape, nt, "gap %.3g" % gap, flush=True)
        full = [512, 256 * 256, 10] if is2d else [512, 256, 256, 10]
        sums[test].append({"args": full, "lines": run_binary(test, full), "readme_config": True})
        print(test, "full", sums[test][-1]["lines"], flush=True)
    with open(os.path.join(HERE, "reference_arrays.json"), "w") as f:
        json.dump(arrays, f, indent=1)
    with open(os.path.join(HERE, "reference_checksums.json"), "w") as f:
        json.dump({"runs": sums, "readme_cuda_t500": readme_table()}, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
