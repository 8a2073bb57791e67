"""GPU parity of the suite's other tests (vecadd, matvec, matmul, sincos,
whispering) through the C ABI against the oracle.

KG_F64 equals the oracle bit for bit (vecadd, matvec and whispering: the
oracle itself equals the reference's own kernels, tests/test_oracle_extra.py)
except sincos, whose sin/cos come from CUDA's math library (within 2 ulp each
of the correctly rounded value): there the bound is 4 ulp of 2.  KG_F64_FMA
is within 1e-12 normwise; KG_F32 within the stated bounds.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


CASES = {
    "vecadd": [(3, 3, 3, 1), (5, 4, 3, 2), (33, 17, 9, 4), (64, 32, 32, 10), (130, 1, 1, 3)],
    "matvec": [(1, 1, 1), (3, 5, 2), (33, 70, 3), (512, 300, 10), (100, 1000, 2), (0, 7, 1), (1000, 129, 1)],
    "matmul": [(1, 1, 1, 1), (7, 5, 3, 2), (33, 17, 40, 2), (64, 64, 64, 1), (100, 37, 70, 2)],
    "sincos": [(3, 3, 3, 1), (33, 17, 9, 2)],
    "whispering": [(3, 3, 1), (5, 7, 2), (33, 70, 4), (64, 1024, 10), (129, 300, 3)],
}


def gpu_program(test, args, dtype, tdt=torch.float64):
    """The test program on the GPU from the oracle's initial arrays; returns
    the arrays in their final roles (numpy FP64)."""
    nt = args[-1]
    init, coef, _, _ = ol.extra_program(test, tuple(args[:-1]) + (0,))
    bufs = [torch.from_numpy(a.copy()).cuda().to(tdt) for a in init]
    by = {b.data_ptr(): b for b in bufs}
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(nt):
        kgb200.extra_step(test, dtype, args[:-1], ptrs, coef)
        ptrs = kgb200.extra_rotate(test, ptrs)
    torch.cuda.synchronize()
    return [by[p].double().cpu().numpy() for p in ptrs]


def normwise(x, ref):
    m = float(np.max(np.abs(ref))) if ref.size else 0.0
    return float(np.max(np.abs(x - ref))) / m if m > 0 else float(np.max(np.abs(x))) if x.size else 0.0


ALL = [(t, c) for t in CASES for c in CASES[t]]


@pytest.mark.parametrize("test,args", ALL, ids=["%s-%s" % (t, "x".join(map(str, c))) for t, c in ALL])
def test_extra_f64(test, args):
    got = gpu_program(test, args, kgb200.KG_F64)
    want, _, _, _ = ol.extra_program(test, args)
    for q, (g, w) in enumerate(zip(got, want)):
        if test == "sincos":
            assert np.max(np.abs(g - w)) <= 4 * 2.0 ** -52 * 2, q
        else:
            assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), \
                "%s array %d differs (max |d| %g)" % (test, q, np.max(np.abs(g - w)) if g.size else 0)


FORMS = [(t, CASES[t][min(2, len(CASES[t]) - 1)]) for t in CASES]


@pytest.mark.parametrize("test,args", FORMS, ids=[t for t, _ in FORMS])
def test_extra_fma_and_f32(test, args):
    want, _, _, _ = ol.extra_program(test, args)
    got = gpu_program(test, args, kgb200.KG_F64_FMA)
    for g, w in zip(got, want):
        assert normwise(g, w) <= 1e-12
    got = gpu_program(test, args, kgb200.KG_F32, torch.float32)
    # FP32: storage rounding of the inputs plus sums of up to ~100 terms
    tol = {"vecadd": 2e-6, "matvec": 2e-6, "matmul": 2e-6, "sincos": 2e-6, "whispering": 2e-5}[test]
    for g, w in zip(got, want):
        assert normwise(g, w) <= tol, (test, normwise(g, w))


def test_extra_argument_errors():
    lib = kgb200.load()
    a = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = a.data_ptr()
    assert lib.kg_vecadd(kgb200.KG_BF16, 4, 4, 4, p, p, p, None) == 5
    assert lib.kg_vecadd(kgb200.KG_F64, 2, 2, 2, p, p + 8, p, None) == 1      # output overlaps input
    assert lib.kg_matvec(kgb200.KG_F64, -1, 4, p, p, p, None) == 1
    assert lib.kg_matmul(kgb200.KG_F64, 2, 2, 2, p, p + 64, p + 8, None) == 1  # C overlaps A
    assert lib.kg_sincos(kgb200.KG_F64, 1, 1, 1, None, p, p + 8, None) == 1
    n = 9
    e, h0, h1 = p, p + 8 * 2 * n, p + 8 * 3 * n
    assert lib.kg_whispering(kgb200.KG_F64, 3, 3, 1.0, 1.0, e, h0, h0, h0, h1, h0, h0, h0, h0, None) == 1
    nregs = __import__("ctypes").c_int()
    kgb200.check(lib.kg_extra_regcount(b"matmul", kgb200.KG_F64, __import__("ctypes").byref(nregs)))
    assert nregs.value > 0


GOLD = __import__("json").load(open(__import__("os").path.join(
    __import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden", "reference_extra.json")))
BIN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.dirname(
    __import__("os").path.abspath(__file__))), "kernelgen-perf-tests_gb300", "build", "bin")
RUNS = [(t, i) for t in GOLD for i in range(len(GOLD[t]["runs"]))]


def driver_lines(test, args):
    import subprocess
    env = {k: v for k, v in __import__("os").environ.items() if k != "NO_TIMING"}
    out = subprocess.run([__import__("os").path.join(BIN, test + "_b200")] + [str(a) for a in args],
                         capture_output=True, text=True, check=True, env=env).stdout
    return [ln for ln in out.splitlines() if ln.startswith(("initial mean", "final mean", "mu"))]


def same_line(w, g):
    if w == g:
        return True
    # growing whispering fields: the reference gcc build is fast-math
    wv, gv = float(w.split("=")[-1]), float(g.split("=")[-1])
    return abs(wv - gv) <= 1e-10 * abs(wv) + 1e-6


@pytest.mark.parametrize("test,idx", RUNS, ids=["%s-%d" % r for r in RUNS])
def test_b200_extra_driver_prints_reference_lines(test, idx):
    """The b200 program of vecadd, matvec and whispering prints the lines of
    the reference's gcc target (including the suite's own problem size)."""
    run = GOLD[test]["runs"][idx]
    got = driver_lines(test, run["args"])
    assert len(got) == len(run["lines"]) and all(same_line(w, g) for w, g in zip(run["lines"], got)), (run["lines"], got)


@pytest.mark.parametrize("test,args", [("matmul", (33, 17, 40, 2)), ("sincos", (33, 17, 9, 2)),
                                       ("matmul", (512, 256, 256, 10))])
def test_b200_extra_driver_matches_oracle(test, args):
    """matmul and sincos (Fortran kernels in the reference): the b200 program
    prints the oracle program's means."""
    _, _, im, fm = ol.extra_program(test, args)
    assert driver_lines(test, args) == ["initial mean = %f" % im, "final mean = %f" % fm]


def _f32(rng, n):
    return torch.from_numpy(rng.uniform(-1, 1, n).astype(np.float32)).cuda()


@pytest.mark.parametrize("nx,ny", [(4, 1), (32, 64), (36, 65), (100, 1000), (1000, 129), (512, 65536)])
def test_matvec_f32_ring_equals_register_staged(nx, ny):
    """FP32 rows of a multiple of 4 with 16-byte aligned A and x take the
    cp.async ring kernel; an x 4 bytes off alignment takes the register-staged
    kernel.  Both sum each row in the reference's order: equal bit for bit,
    and within FP32 rounding of the FP64 product."""
    lib = kgb200.load()
    rng = np.random.default_rng(nx + ny)
    A = _f32(rng, nx * ny)
    xb = _f32(rng, nx + 4)
    x16, x4 = xb[:nx].clone(), xb[1:1 + nx]
    x4.copy_(x16)
    assert x16.data_ptr() % 16 == 0 and x4.data_ptr() % 16 == 4
    y16 = torch.zeros(ny, dtype=torch.float32, device="cuda")
    y4 = torch.full((ny,), 7.0, dtype=torch.float32, device="cuda")
    kgb200.check(lib.kg_matvec(kgb200.KG_F32, nx, ny, A.data_ptr(), x16.data_ptr(), y16.data_ptr(), None))
    kgb200.check(lib.kg_matvec(kgb200.KG_F32, nx, ny, A.data_ptr(), x4.data_ptr(), y4.data_ptr(), None))
    g16, g4 = y16.cpu().numpy(), y4.cpu().numpy()
    assert np.array_equal(g16.view(np.uint32), g4.view(np.uint32))
    ref = A.double().cpu().numpy().reshape(ny, nx) @ x16.double().cpu().numpy()
    mag = np.abs(A.double().cpu().numpy().reshape(ny, nx)) @ np.abs(x16.double().cpu().numpy())
    assert np.all(np.abs(g16 - ref) <= nx * 2.0 ** -23 * mag + 1e-30)


@pytest.mark.parametrize("n", [1, 4, 7, 4099, 1 << 20])
def test_sincos_f32_vector_equals_scalar(n):
    """Aligned FP32 sincos runs four points a thread; arrays 4 bytes off
    alignment run the scalar kernel: the same bits, within 2 ulp-ish of FP64."""
    lib = kgb200.load()
    rng = np.random.default_rng(n)
    xb, yb = _f32(rng, n + 4) * 8, _f32(rng, n + 4) * 8
    x16, y16 = xb[:n].clone(), yb[:n].clone()
    x4, y4 = xb[1:1 + n], yb[1:1 + n]
    x4.copy_(x16)
    y4.copy_(y16)
    o16 = torch.zeros(n, dtype=torch.float32, device="cuda")
    ob = torch.zeros(n + 4, dtype=torch.float32, device="cuda")
    o4 = ob[1:1 + n]
    kgb200.check(lib.kg_sincos(kgb200.KG_F32, n, 1, 1, x16.data_ptr(), y16.data_ptr(), o16.data_ptr(), None))
    kgb200.check(lib.kg_sincos(kgb200.KG_F32, n, 1, 1, x4.data_ptr(), y4.data_ptr(), o4.data_ptr(), None))
    g16, g4 = o16.cpu().numpy(), o4.cpu().numpy()
    assert np.array_equal(g16.view(np.uint32), g4.view(np.uint32))
    ref = np.sin(x16.double().cpu().numpy()) + np.cos(y16.double().cpu().numpy())
    assert np.max(np.abs(g16 - ref)) <= 4 * 2.0 ** -23 * 2
