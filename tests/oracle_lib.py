"""ctypes binding of the oracle (oracle/kg_oracle.c): test infrastructure.

Only tests, the smoke check and bench.py's CPU baseline leg use the oracle;
the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")

TESTS = ["laplacian", "divergence", "gradient", "uxx1", "wave13pt", "tricubic",
         "tricubic2", "jacobi", "lapgsrb", "gaussblur", "gameoflife"]
TEST_ID = {t: i for i, t in enumerate(TESTS)}
NARR = [2, 4, 4, 6, 3, 5, 5, 2, 2, 2, 2]
NCOEF = [2, 3, 3, 2, 3, 0, 0, 3, 4, 6, 0]
IS2D = {"jacobi", "gaussblur", "gameoflife"}

INIT_REFERENCE, INIT_BERNOULLI, INIT_UNIT_OFFSETS = 0, 1, 2


class OrCase(ctypes.Structure):
    _fields_ = [("test", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("ns", ctypes.c_int), ("narr", ctypes.c_int), ("ncoef", ctypes.c_int),
                ("coef", ctypes.c_double * 6), ("arr", ctypes.c_void_p * 6),
                ("order", ctypes.c_int * 6)]


_libs = {}


def load(flavour="strict"):
    """Load build/liboracle.so (strict) or build/liboracle_fast.so (fast)."""
    if flavour in _libs:
        return _libs[flavour]
    name = "liboracle.so" if flavour == "strict" else "liboracle_fast.so"
    path = os.path.join(ORACLE_DIR, "build", name)
    if not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    lib = ctypes.CDLL(path)
    lib.or_init.argtypes = [ctypes.POINTER(OrCase), ctypes.c_int, ctypes.c_uint]
    lib.or_sweep.argtypes = [ctypes.POINTER(OrCase)]
    lib.or_set_threads.argtypes = [ctypes.c_int]
    lib.or_set_threads.restype = None
    lib.or_run.argtypes = [ctypes.POINTER(OrCase), ctypes.c_int]
    lib.or_initial_mean.argtypes = [ctypes.POINTER(OrCase)]
    lib.or_initial_mean.restype = ctypes.c_double
    lib.or_final_mean.argtypes = [ctypes.POINTER(OrCase)]
    lib.or_final_mean.restype = ctypes.c_double
    lib.or_final_slot.argtypes = [ctypes.POINTER(OrCase)]
    lib.or_final_slot.restype = ctypes.c_int
    lib.or_conway_u8.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_init_bernoulli_u8.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_double, ctypes.c_uint]
    lib.or_rbsor_sweep.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_void_p, ctypes.c_void_p]
    lib.or_residual_norm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_residual_norm.restype = ctypes.c_double
    _libs[flavour] = lib
    return lib


def rbsor_sweeps(u, f, shape, omega, nsweeps):
    lib = load()
    nx, ny, ns = shape
    for _ in range(nsweeps):
        lib.or_rbsor_sweep(nx, ny, ns, omega, u.ctypes.data, f.ctypes.data)
    return u


def residual_norm(u, f, shape):
    nx, ny, ns = shape
    return load().or_residual_norm(nx, ny, ns, u.ctypes.data, f.ctypes.data)


class Case:
    """A test program's state: arrays (numpy, float64) + coefficients."""

    def __init__(self, test, shape, variant=INIT_REFERENCE, seed=1, flavour="strict"):
        self.test = test
        self.lib = load(flavour)
        tid = TEST_ID[test]
        if len(shape) == 2:
            nx, ny, ns = shape[0], shape[1], 1
        else:
            nx, ny, ns = shape
        self.shape = (nx, ny, ns)
        n = nx * ny * ns
        self.buffers = [np.zeros(n, dtype=np.float64) for _ in range(NARR[tid])]
        self.c = OrCase()
        self.c.test, self.c.nx, self.c.ny, self.c.ns = tid, nx, ny, ns
        for q, b in enumerate(self.buffers):
            self.c.arr[q] = b.ctypes.data
        self.lib.or_init(ctypes.byref(self.c), variant, seed)

    @classmethod
    def from_arrays(cls, test, shape, coef, arrays, flavour="strict"):
        """A case over given inputs (copied), e.g. the product's pulse input."""
        self = cls.__new__(cls)
        self.test = test
        self.lib = load(flavour)
        tid = TEST_ID[test]
        nx, ny, ns = (shape[0], shape[1], 1) if len(shape) == 2 else shape
        self.shape = (nx, ny, ns)
        self.buffers = [np.array(a, dtype=np.float64, copy=True) for a in arrays]
        self.c = OrCase()
        self.c.test, self.c.nx, self.c.ny, self.c.ns = tid, nx, ny, ns
        self.c.narr, self.c.ncoef = NARR[tid], NCOEF[tid]
        for q, b in enumerate(self.buffers):
            self.c.arr[q] = b.ctypes.data
            self.c.order[q] = q
        for q, v in enumerate(list(coef)[:6]):
            self.c.coef[q] = v
        return self

    @property
    def coef(self):
        return [self.c.coef[q] for q in range(NCOEF[TEST_ID[self.test]])]

    def arrays(self):
        """Arrays in their current roles (slot order after rotation)."""
        by_addr = {b.ctypes.data: b for b in self.buffers}
        return [by_addr[self.c.arr[q]] for q in range(len(self.buffers))]

    def sweep(self):
        self.lib.or_sweep(ctypes.byref(self.c))

    def run(self, nt):
        self.lib.or_run(ctypes.byref(self.c), nt)

    def initial_mean(self):
        return self.lib.or_initial_mean(ctypes.byref(self.c))

    def final_mean(self):
        return self.lib.or_final_mean(ctypes.byref(self.c))

    def final_slot(self):
        return self.lib.or_final_slot(ctypes.byref(self.c))


def conway_u8(u0, u1, nx, ny):
    """One B3/S23 sweep u0 -> u1 (interior only; u1's rim is kept)."""
    lib = load()
    out = u1.copy()
    lib.or_conway_u8(nx, ny, u0.ctypes.data, out.ctypes.data)
    return out


def bernoulli_u8(n, p=0.3, seed=1):
    lib = load()
    u0 = np.zeros(n, dtype=np.uint8)
    u1 = np.zeros(n, dtype=np.uint8)
    lib.or_init_bernoulli_u8(n, u0.ctypes.data, u1.ctypes.data, p, seed)
    return u0, u1


# ---- the suite's other tests (oracle/kg_oracle_extra.c) ----------------------

EXTRA = ["vecadd", "matvec", "matmul", "sincos", "whispering"]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def extra_program(test, args, flavour="strict"):
    """Run one of the other tests as the reference main() does.  args as its
    command line (vecadd/sincos/matmul: nx ny ns nt; matvec/whispering: nx
    ny nt).  Returns (arrays in their final roles, coefficients, initial mean,
    final mean); the arrays are those the test allocates, in its order."""
    lib = load(flavour)
    im, fm = ctypes.c_double(), ctypes.c_double()
    coef = []
    if test in ("vecadd", "sincos"):
        nx, ny, ns, nt = args
        n = nx * ny * ns
        a = [np.empty(n) for _ in range(3)]
        if test == "vecadd":
            w = (ctypes.POINTER(ctypes.c_double) * 3)(*[_dp(x) for x in a])
            lib.or_vecadd_program(nx, ny, ns, nt, w, ctypes.byref(im), ctypes.byref(fm))
            order = [next(q for q in range(3) if ctypes.addressof(w[r].contents) == a[q].ctypes.data)
                     for r in range(3)]
            a = [a[q] for q in order]
        else:
            lib.or_sincos_program(nx, ny, ns, nt, _dp(a[0]), _dp(a[1]), _dp(a[2]), ctypes.byref(im), ctypes.byref(fm))
    elif test == "matvec":
        nx, ny, nt = args
        a = [np.empty(nx * ny), np.empty(nx), np.empty(ny)]
        lib.or_matvec_program(nx, ny, nt, _dp(a[0]), _dp(a[1]), _dp(a[2]), ctypes.byref(im), ctypes.byref(fm))
    elif test == "matmul":
        nx, ny, ns, nt = args
        a = [np.empty(nx * ny), np.empty(ny * ns), np.empty(nx * ns)]
        lib.or_matmul_program(nx, ny, ns, nt, _dp(a[0]), _dp(a[1]), _dp(a[2]), ctypes.byref(im), ctypes.byref(fm))
    elif test == "whispering":
        nx, ny, nt = args
        n = nx * ny
        a = [np.empty(2 * n)] + [np.empty(n) for _ in range(8)]
        c = (ctypes.c_double * 2)()
        w = (ctypes.POINTER(ctypes.c_double) * 9)(*[_dp(x) for x in a])
        lib.or_whispering_program(nx, ny, nt, c, w, ctypes.byref(im), ctypes.byref(fm))
        by_addr = {x.ctypes.data: x for x in a}
        a = [by_addr[ctypes.addressof(w[r].contents)] for r in range(9)]
        coef = list(c)
    else:
        raise ValueError(test)
    return a, coef, im.value, fm.value


def extra_step(test, arrays, args, coef=()):
    """One step of the oracle kernel on numpy arrays (in place)."""
    lib = load("strict")
    if test == "vecadd":
        lib.or_vecadd(ctypes.c_size_t(arrays[0].size), *[_dp(x) for x in arrays])
    elif test == "sincos":
        lib.or_sincos(ctypes.c_size_t(arrays[0].size), *[_dp(x) for x in arrays])
    elif test == "matvec":
        lib.or_matvec(args[0], args[1], *[_dp(x) for x in arrays])
    elif test == "matmul":
        lib.or_matmul(args[0], args[1], args[2], *[_dp(x) for x in arrays])
    elif test == "whispering":
        lib.or_whispering(args[0], args[1], ctypes.c_double(coef[0]), ctypes.c_double(coef[1]),
                          *[_dp(x) for x in arrays])
    else:
        raise ValueError(test)
