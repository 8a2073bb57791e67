#!/usr/bin/env python3
"""Golden fixtures of the suite's other C tests (vecadd, matvec, whispering)
from the reference itself.

Needs the reference tree (KG_REFERENCE_TREE, else the build's default) and
``make -C oracle ref``.  Writes reference_extra.json: for small cases, the
SHA-256 of every array after nt steps of the reference kernel compiled
unmodified in strict IEEE mode (driven with the reference main()'s rand()
order, time loop and pointer rotation), the initial and final means; and the
checksum lines of the suite's gcc target binary for those cases and for the
suite's own problem size (vecadd 512 256 256 10; matvec and whispering
512 65536 10).  matmul and sincos have Fortran kernels and are not built.
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
libc = ctypes.CDLL("libc.so.6")
RAND_MAX = 2147483647

CASES = {
    "vecadd": [(3, 3, 3, 1), (5, 4, 3, 2), (33, 17, 9, 4), (64, 32, 32, 10)],
    "matvec": [(1, 1, 1), (3, 5, 2), (33, 70, 3), (512, 300, 10), (100, 1000, 2)],
    "whispering": [(3, 3, 1), (5, 7, 2), (33, 70, 4), (64, 1024, 10), (129, 300, 3)],
}
FULL = {"vecadd": [512, 256, 256, 10], "matvec": [512, 65536, 10], "whispering": [512, 65536, 10]}


def real_rand():
    return ((libc.rand() / float(RAND_MAX)) - 0.5) * 2


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def P(x):
    return x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def serial_mean_terms(*cols):
    """sum over i of (((c0 + c1) + c2) ...) accumulated in order, as the C loop."""
    s = 0.0
    for vals in zip(*cols):
        t = vals[0]
        for v in vals[1:]:
            t = t + v
        s = s + t
    return s


def run_vecadd(lib, nx, ny, ns, nt):
    n = nx * ny * ns
    libc.srand(1)
    w = [np.empty(n) for _ in range(3)]
    for i in range(n):
        for q in range(3):
            w[q][i] = real_rand()
    imean = serial_mean_terms(w[0], w[1], w[2]) / n / 3
    ins = [sha(x) for x in w]
    fn = lib.vecadd
    fn.restype = None
    for _ in range(nt):
        fn(ctypes.c_int(nx), ctypes.c_int(ny), ctypes.c_int(ns), P(w[0]), P(w[1]), P(w[2]))
        w = [w[1], w[2], w[0]]
    fmean = serial_mean_terms(w[1]) / n
    return ins, [sha(x) for x in w], imean, fmean


def run_matvec(lib, nx, ny, nt):
    libc.srand(1)
    A, x, y = np.empty(nx * ny), np.empty(nx), np.empty(ny)
    for i in range(nx * ny):
        A[i] = real_rand()
    for i in range(nx):
        x[i] = real_rand()
    for i in range(ny):
        y[i] = real_rand()
    imean = serial_mean_terms(A) / (nx * ny) + serial_mean_terms(x) / nx + serial_mean_terms(y) / ny
    ins = [sha(v) for v in (A, x, y)]
    fn = lib.matvec
    fn.restype = None
    for _ in range(nt):
        fn(ctypes.c_int(nx), ctypes.c_int(ny), P(A), P(x), P(y))
    return ins, [sha(v) for v in (A, x, y)], imean, serial_mean_terms(y) / ny


def run_whispering(lib, nx, ny, nt):
    n = nx * ny
    libc.srand(1)
    mu, eps = real_rand(), real_rand()
    a = [np.empty(2 * n)] + [np.empty(n) for _ in range(8)]
    for i in range(n):
        a[0][2 * i] = real_rand()
        a[0][2 * i + 1] = real_rand()
        for q in range(1, 9):
            a[q][i] = real_rand()
    imean = serial_mean_terms(a[0][0::2], a[0][1::2], *a[1:]) / n / 12
    ins = [sha(v) for v in a]
    fn = lib.whispering
    fn.restype = None
    for _ in range(nt):
        fn(ctypes.c_int(nx), ctypes.c_int(ny), ctypes.c_double(mu), ctypes.c_double(eps), *[P(v) for v in a])
        a[1], a[2] = a[2], a[1]
        a[3], a[4] = a[4], a[3]
    fmean = serial_mean_terms(a[0][0::2], a[0][1::2], a[2], a[4]) / n / 4
    return ins, [sha(v) for v in a], imean, fmean, [mu, eps]


def run_binary(test, args):
    exe = os.path.join(REF_BUILD, test + "_gcc")
    env = {k: v for k, v in os.environ.items() if k != "NO_TIMING"}
    out = subprocess.run([exe] + [str(x) for x in args], capture_output=True, text=True,
                         check=True, env=env).stdout
    return [ln for ln in out.splitlines() if re.match(r"^(initial mean|final mean|mu)\b", ln)]


def main():
    res = {}
    for test, cases in CASES.items():
        lib = ctypes.CDLL(os.path.join(REF_BUILD, "lib%s_strict.so" % test))
        res[test] = {"cases": [], "runs": []}
        for case in cases:
            if test == "vecadd":
                ins, outs, im, fm = run_vecadd(lib, *case)
                extra = {}
            elif test == "matvec":
                ins, outs, im, fm = run_matvec(lib, *case)
                extra = {}
            else:
                ins, outs, im, fm, coef = run_whispering(lib, *case)
                extra = {"coef": coef}
            res[test]["cases"].append(dict(args=list(case), input_sha256=ins, output_sha256=outs,
                                           initial_mean=im, final_mean=fm, **extra))
            res[test]["runs"].append({"args": list(case), "lines": run_binary(test, list(case))})
            print(test, case, flush=True)
        res[test]["runs"].append({"args": FULL[test], "lines": run_binary(test, FULL[test]), "readme_config": True})
        print(test, "full", res[test]["runs"][-1]["lines"], flush=True)
    with open(os.path.join(HERE, "reference_extra.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
