"""GPU parity: the sm_103a sweeps through the C ABI against the oracle.

KG_F64 must equal the oracle (a strict IEEE restatement of the reference)
bit for bit, rims included, and equal the SHA-256 of the reference's own
kernels recorded in tests/golden/.  KG_F64_FMA must be within 1e-12
normwise (max|gpu-ref| / max|ref|), the bound the reference's fast-math gcc
build itself meets.  Narrow storage types are checked against FP64 with the
per-type tolerances stated below.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ARRAYS = json.load(open(os.path.join(GOLDEN, "reference_arrays.json")))
SUMS = json.load(open(os.path.join(GOLDEN, "reference_checksums.json")))
BIN = os.path.join(ROOT, "kernelgen-perf-tests_gb300", "build", "bin")

SHAPES_3D = [(3, 3, 3), (5, 5, 5), (7, 6, 5), (33, 17, 9), (64, 32, 32), (129, 35, 20)]
SHAPES_2D = [(3, 3), (5, 5), (7, 9), (33, 70), (64, 1024), (129, 300)]

# Normwise tolerances of the narrow forms after NT_LOW sweeps of the
# reference's random inputs (storage rounding dominates: FP32 2^-24,
# FP16 2^-11, BF16 2^-8 relative per value).
NT_LOW = 2
TOL = {kgb200.KG_F32: 2e-6, kgb200.KG_F16: 4e-3, kgb200.KG_BF16: 3e-2}


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def shapes(name):
    return SHAPES_2D if name in kgb200.IS2D else SHAPES_3D


def gpu_run(name, dtype, shape, coef, arrays, nt, torch_dtype=torch.float64):
    """nt sweeps on the GPU with the reference's rotation; returns numpy FP64
    arrays in their final roles."""
    bufs = [torch.from_numpy(a).to("cuda").to(torch_dtype) for a in arrays]
    ptr2buf = {b.data_ptr(): b for b in bufs}
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(nt):
        kgb200.sweep(kgb200.problem(name, dtype, shape, coef, ptrs))
        ptrs = kgb200.rotate(name, ptrs)
    torch.cuda.synchronize()
    return [ptr2buf[p].to(torch.float64).cpu().numpy() for p in ptrs]


def normwise(x, ref):
    m = float(np.max(np.abs(ref))) if ref.size else 0.0
    return float(np.max(np.abs(x - ref))) / m if m > 0 else float(np.max(np.abs(x))) if x.size else 0.0


CASES = [(n, s) for n in kgb200.STENCILS for s in shapes(n)]


@pytest.mark.parametrize("name,shape", CASES, ids=["%s-%s" % (n, "x".join(map(str, s))) for n, s in CASES])
def test_f64_bitwise_vs_oracle(name, shape):
    case = ol.Case(name, shape)
    arrays = [a.copy() for a in case.arrays()]
    nt = 3
    got = gpu_run(name, kgb200.KG_F64, case.shape, case.coef, arrays, nt)
    case.run(nt)
    for q, (g, w) in enumerate(zip(got, case.arrays())):
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), \
            "%s slot %d differs (max |d| %g)" % (name, q, np.max(np.abs(g - w)))


FIX = [(t, i) for t in ARRAYS for i in range(len(ARRAYS[t]))]


@pytest.mark.parametrize("name,idx", FIX, ids=["%s-%d" % x for x in FIX])
def test_f64_matches_reference_kernel_hashes(name, idx):
    """Outputs hash-equal to the reference's own kernel (strict build)."""
    fx = ARRAYS[name][idx]
    case = ol.Case(name, fx["shape"])
    got = gpu_run(name, kgb200.KG_F64, case.shape, case.coef, case.arrays(), fx["nt"])
    assert [sha(g) for g in got] == fx["output_sha256"]


@pytest.mark.parametrize("name", kgb200.STENCILS)
def test_f64fma_normwise(name):
    shape = (129, 300) if name in kgb200.IS2D else (64, 32, 32)
    case = ol.Case(name, shape)
    nt = 4
    got = gpu_run(name, kgb200.KG_F64_FMA, case.shape, case.coef, [a.copy() for a in case.arrays()], nt)
    case.run(nt)
    for g, w in zip(got, case.arrays()):
        if name == "gameoflife":
            # the smooth rule divides by 1 + x*1e20; compare where it is well conditioned
            assert np.array_equal(g > 0.5, w > 0.5) or normwise(g, w) <= 1e-12
        else:
            assert normwise(g, w) <= 1e-12


LOW = [(n, d) for n in kgb200.STENCILS if n != "gameoflife"
       for d in (kgb200.KG_F32, kgb200.KG_F16, kgb200.KG_BF16)]


@pytest.mark.parametrize("name,dtype", LOW, ids=["%s-%d" % x for x in LOW])
def test_narrow_storage_error_bounds(name, dtype):
    shape = (129, 300) if name in kgb200.IS2D else (64, 32, 32)
    case = ol.Case(name, shape)
    tdt = {kgb200.KG_F32: torch.float32, kgb200.KG_F16: torch.float16, kgb200.KG_BF16: torch.bfloat16}[dtype]
    # The oracle runs on the same rounded inputs, so the error is the sweeps' own.
    rounded = [torch.from_numpy(a).to(tdt).to(torch.float64).numpy() for a in case.arrays()]
    for a, r in zip(case.arrays(), rounded):
        a[:] = r
    if name == "uxx1":
        # uxx1 divides by the mean density d; the reference's d1 in [-1,1] puts
        # d near 0, where any rounding is amplified without bound.  A density
        # in [1,2) (as in the precision-sweep input) keeps the test meaningful.
        d1 = case.arrays()[2]
        d1[:] = torch.from_numpy(1.5 + 0.5 * d1).to(tdt).to(torch.float64).numpy()
    got = gpu_run(name, dtype, case.shape, case.coef, [a.copy() for a in case.arrays()], NT_LOW, tdt)
    case.run(NT_LOW)
    out_slots = [q for q in range(len(got)) if not np.array_equal(got[q], case.arrays()[q])]
    for q in range(len(got)):
        err = normwise(got[q], case.arrays()[q])
        assert err <= TOL[dtype], "%s slot %d error %g (tolerance %g, changed slots %s)" % (
            name, q, err, TOL[dtype], out_slots)


# rows of a multiple of 16 bytes take the 16-cell vector kernel: one vector a
# row (both rims in it), a partial warp, two warps a row, one interior row
@pytest.mark.parametrize("shape", [(3, 3), (5, 7), (67, 45), (512, 1031), (16, 40), (48, 33), (1024, 100),
                                   (32, 3)])
def test_conway_u8_bitwise(shape):
    nx, ny = shape
    b0, b1 = ol.bernoulli_u8(nx * ny)
    d = [torch.from_numpy(b0.copy()).cuda(), torch.from_numpy(b1.copy()).cuda()]
    ptrs = [x.data_ptr() for x in d]
    for _ in range(7):
        kgb200.sweep(kgb200.problem("gameoflife", kgb200.KG_U8, shape, [], ptrs))
        ptrs = ptrs[::-1]
        b0, b1 = ol.conway_u8(b0, b1, nx, ny), b0
    torch.cuda.synchronize()
    by = {x.data_ptr(): x for x in d}
    assert np.array_equal(by[ptrs[0]].cpu().numpy(), b0)
    assert np.array_equal(by[ptrs[1]].cpu().numpy(), b1)


@pytest.mark.parametrize("shape", [(130, 77), (128, 77)])
def test_conway_u8_equals_fp64_reference_rule(shape):
    """Bernoulli(0.3) cells: the FP64 sweep (the reference rule) thresholded
    at 0.5 equals the byte sweep, sweep after sweep (scalar and vector
    kernels)."""
    case = ol.Case("gameoflife", shape, variant=ol.INIT_BERNOULLI)
    f = gpu_run("gameoflife", kgb200.KG_F64, case.shape, [], case.arrays(), 9)
    b0, b1 = (x.astype(np.uint8) for x in case.arrays())
    d = [torch.from_numpy(b0.copy()).cuda(), torch.from_numpy(b1.copy()).cuda()]
    ptrs = [x.data_ptr() for x in d]
    for _ in range(9):
        kgb200.sweep(kgb200.problem("gameoflife", kgb200.KG_U8, shape, [], ptrs))
        ptrs = ptrs[::-1]
    torch.cuda.synchronize()
    by = {x.data_ptr(): x for x in d}
    for q in range(2):
        assert np.array_equal((f[q] > 0.5).astype(np.uint8), by[ptrs[q]].cpu().numpy())


@pytest.mark.parametrize("dtype", [kgb200.KG_F64, kgb200.KG_F32, kgb200.KG_BF16, kgb200.KG_U8])
def test_checksum(dtype):
    n = 3_000_017
    rng = np.random.default_rng(5)
    tdt = {kgb200.KG_F64: torch.float64, kgb200.KG_F32: torch.float32,
           kgb200.KG_BF16: torch.bfloat16, kgb200.KG_U8: torch.uint8}[dtype]
    if dtype == kgb200.KG_U8:
        xs = [torch.from_numpy(rng.integers(0, 2, n).astype(np.uint8)).cuda() for _ in range(2)]
    else:
        xs = [torch.from_numpy(rng.uniform(-1, 1, n)).to(tdt).cuda() for _ in range(3)]
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    kgb200.checksum(dtype, n, [x.data_ptr() for x in xs], out.data_ptr())
    kgb200.checksum(dtype, n, [x.data_ptr() for x in xs], out[1:].data_ptr())
    torch.cuda.synchronize()
    ref = sum(x.to(torch.float64).cpu().numpy() for x in xs)
    want = float(np.sum(ref))
    got = out.cpu().numpy()
    assert got[0] == got[1], "checksum is not deterministic"
    assert abs(got[0] - want) <= 1e-12 * float(np.sum(np.abs(ref))) + 1e-300


def test_error_stats():
    n = 1_000_003
    rng = np.random.default_rng(6)
    ref = rng.uniform(-2, 2, n)
    x = torch.from_numpy(ref).to(torch.float32).cuda()
    r = torch.from_numpy(ref).cuda()
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    kgb200.error_stats(kgb200.KG_F32, n, x.data_ptr(), r.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    d = x.double().cpu().numpy() - ref
    o = out.cpu().numpy()
    assert o[0] == np.max(np.abs(d)) and o[2] == np.max(np.abs(ref))
    assert abs(o[1] - np.sum(d * d)) <= 1e-9 * np.sum(d * d)
    assert abs(o[3] - np.sum(ref * ref)) <= 1e-12 * np.sum(ref * ref)


@pytest.mark.parametrize("name", kgb200.STENCILS)
def test_program_run_host_buffers(name):
    """kg_program_run (host arrays in, nt sweeps, results out) equals the oracle
    run, and leaves the arrays in the reference's final roles."""
    shape = (70, 301) if name in kgb200.IS2D else (40, 33, 21)
    case = ol.Case(name, shape)
    host = [a.copy() for a in case.arrays()]
    p = kgb200.problem(name, kgb200.KG_F64, case.shape, case.coef, [h.ctypes.data for h in host])
    t = kgb200.program_run(p, 5, 0x3F)
    case.run(5)
    by = {h.ctypes.data: h for h in host}
    final = [by[p.arr[q]] for q in range(len(host))]
    for g, w in zip(final, case.arrays()):
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64))
    assert t.kernel_avg > 0 and t.nregs > 0


@pytest.mark.parametrize("name", ["laplacian", "wave13pt", "divergence", "gameoflife"])
def test_graph_plan(name):
    shape = (70, 301) if name in kgb200.IS2D else (40, 33, 21)
    case = ol.Case(name, shape)
    bufs = [torch.from_numpy(a).cuda() for a in case.arrays()]
    p = kgb200.problem(name, kgb200.KG_F64, case.shape, case.coef, [b.data_ptr() for b in bufs])
    plan = kgb200.Plan(p, 6)
    plan.launch()
    torch.cuda.synchronize()
    fin = plan.final_roles()
    plan.close()
    by = {b.data_ptr(): b for b in bufs}
    case.run(6)
    for q, w in enumerate(case.arrays()):
        g = by[fin.arr[q]].cpu().numpy()
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64))


def test_argument_errors_do_not_launch():
    x = torch.zeros(8 * 8 * 8, dtype=torch.float64, device="cuda")
    lib = kgb200.load()
    # output aliases input
    p = kgb200.problem("laplacian", kgb200.KG_F64, (8, 8, 8), [1.0, 1.0], [x.data_ptr(), x.data_ptr()])
    assert lib.kg_sweep(p, None) == 1
    # byte cells only for gameoflife
    y = torch.zeros_like(x)
    p = kgb200.problem("laplacian", kgb200.KG_U8, (8, 8, 8), [1.0, 1.0], [x.data_ptr(), y.data_ptr()])
    assert lib.kg_sweep(p, None) == 5
    # 2D stencil with ns != 1
    p = kgb200.problem("jacobi", kgb200.KG_F64, (8, 8, 8), [1.0, 1.0, 1.0], [x.data_ptr(), y.data_ptr()])
    assert lib.kg_sweep(p, None) == 1
    # empty domain: OK, nothing written
    y.fill_(7.0)
    p = kgb200.problem("wave13pt", kgb200.KG_F64, (4, 4, 4), [1.0, 1.0, 1.0],
                       [x.data_ptr(), x[1:].data_ptr(), y.data_ptr()])
    assert lib.kg_sweep(p, None) == 0
    torch.cuda.synchronize()
    assert bool(torch.all(y == 7.0))


def driver_lines(name, args, env_extra=None):
    env = {k: v for k, v in os.environ.items() if k != "NO_TIMING"}
    env.update(env_extra or {})
    out = subprocess.run([os.path.join(BIN, name + "_b200")] + [str(a) for a in args],
                         capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr
    return out.stdout


def protocol_lines(stdout):
    import re
    return sorted(ln.rstrip() for ln in stdout.splitlines()
                  if re.match(r"^(initial mean|final mean|alpha|c0|c1|m0|s0|s4)\b", ln))


DRV = [(t, r) for t in SUMS["runs"] for r in SUMS["runs"][t]]


@pytest.mark.parametrize("name,run", DRV, ids=["%s-%s" % (t, "x".join(map(str, r["args"]))) for t, r in DRV])
def test_b200_driver_prints_reference_lines(name, run):
    """The b200 target program prints the reference gcc binary's coefficient,
    initial-mean and final-mean lines (full size 512 256 256 10 included)."""
    out = driver_lines(name, run["args"], {"PROFILING_FNAME": name})
    assert protocol_lines(out) == sorted(ln.rstrip() for ln in run["lines"])
    assert "%s regcount = " % name in out
    assert out.count("%s kernel time = " % name) == run["args"][-1]
    for key in ("init time", "device buffer alloc time", "data load time", "compute time",
                "data save time", "device buffer free time"):
        assert key + " = " in out


def test_b200_driver_jacobi_and_graph_mode():
    """jacobi has no reference fixture (Fortran kernel): its final mean must
    equal the oracle's; graph mode must print the same lines as plain mode."""
    case = ol.Case("jacobi", (64, 1024))
    im = case.initial_mean()
    case.run(10)
    out = driver_lines("jacobi", [64, 1024, 10])
    assert "final mean = %f" % case.final_mean() in out
    assert "initial mean = %f" % im in out
    g = driver_lines("laplacian", [64, 32, 32, 10], {"B200_MODE": "graph"})
    p = driver_lines("laplacian", [64, 32, 32, 10])
    assert protocol_lines(g) == protocol_lines(p)


def test_b200_driver_gameoflife_bernoulli_u8():
    """Config: Bernoulli(0.3) int cells on bytes print the FP64 reference
    rule's final mean thresholded (the live-cell fraction)."""
    case = ol.Case("gameoflife", (128, 512), variant=ol.INIT_BERNOULLI)
    case.run(10)
    live = float(np.mean(case.arrays()[1] > 0.5))
    out = driver_lines("gameoflife", [128, 512, 10], {"B200_PREC": "u8", "B200_INIT": "bernoulli"})
    assert "final mean = %f" % live in out




@pytest.mark.parametrize("name", ["tricubic", "tricubic2"])
@pytest.mark.parametrize("shape", [(5, 5, 5), (40, 33, 21), (129, 35, 20)])
def test_tricubic_plan_precomputed_weights(name, shape):
    """Plans of tricubic programs evaluate the loop-invariant weight products
    once per replay (one extra kernel) and sweep from them: bit for bit the
    oracle over two replays of four sweeps (an even count returns the roles,
    so the second replay continues the first); the FMA form stays within
    1e-12 of it."""
    for dt in (kgb200.KG_F64, kgb200.KG_F64_FMA):
        case = ol.Case(name, shape)
        bufs = [torch.from_numpy(a).cuda() for a in case.arrays()]
        p = kgb200.problem(name, dt, case.shape, case.coef, [b.data_ptr() for b in bufs])
        plan = kgb200.Plan(p, 4)
        assert plan.kernels() == 5
        plan.launch()
        plan.launch()
        torch.cuda.synchronize()
        fin = plan.final_roles()
        plan.close()
        case.run(8)
        by = {b.data_ptr(): b for b in bufs}
        for q, w in enumerate(case.arrays()):
            g = by[fin.arr[q]].cpu().numpy()
            if dt == kgb200.KG_F64:
                assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), (name, shape, q)
            else:
                assert normwise(g, w) <= 1e-12, (name, shape, q)
