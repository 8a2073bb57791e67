"""The three sweep engines against each other and against the oracle.

The TMA engine (halo planes moved into shared memory by tiled bulk copies,
own column in registers) evaluates the same expressions as the direct engine,
so its KG_F64 results equal the oracle bit for bit and its other types equal
the automatic engine's.  Shapes keep rows a multiple of 16 bytes, as the bulk
copies need; they include domains smaller than a tile, tiles cut by the
domain's edge in x, y and z, and single-plane runs.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

TDT = {kgb200.KG_F64: torch.float64, kgb200.KG_F64_FMA: torch.float64, kgb200.KG_F64_FF: torch.float64,
       kgb200.KG_F32: torch.float32, kgb200.KG_BF16: torch.bfloat16, kgb200.KG_F16: torch.float16}

SHAPES_3D = [(8, 4, 4), (8, 6, 5), (40, 33, 20), (64, 32, 32), (136, 20, 41)]
SHAPES_2D = [(8, 5), (16, 3), (64, 1024), (136, 300), (264, 77)]


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def shapes(name):
    return SHAPES_2D if name in kgb200.IS2D else SHAPES_3D


def run(name, dtype, shape, coef, arrays, nt, engine):
    tdt = TDT[dtype]
    bufs = [torch.from_numpy(a).to("cuda").to(tdt) for a in arrays]
    ptr2buf = {b.data_ptr(): b for b in bufs}
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(nt):
        kgb200.sweep(kgb200.problem(name, dtype, shape, coef, ptrs, engine=engine))
        ptrs = kgb200.rotate(name, ptrs)
    torch.cuda.synchronize()
    kgb200.engine_status()
    return [ptr2buf[p].to(torch.float64).cpu().numpy() for p in ptrs]


F64_CASES = [(n, s) for n in kgb200.STENCILS for s in shapes(n)]


@pytest.mark.parametrize("name,shape", F64_CASES, ids=["%s-%s" % (n, "x".join(map(str, s))) for n, s in F64_CASES])
def test_tma_f64_bitwise_vs_oracle(name, shape):
    case = ol.Case(name, shape)
    nt = 3
    got = run(name, kgb200.KG_F64, case.shape, case.coef, [a.copy() for a in case.arrays()], nt, "tma")
    case.run(nt)
    for q, (g, w) in enumerate(zip(got, case.arrays())):
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), \
            "%s slot %d differs (max |d| %g)" % (name, q, np.max(np.abs(g - w)))


OTHER = [(n, d, s) for n in kgb200.STENCILS
         for d in (kgb200.KG_F64_FMA, kgb200.KG_F32, kgb200.KG_BF16, kgb200.KG_F16, kgb200.KG_F64_FF)
         for s in shapes(n)[2:4]
         if not (n == "gameoflife" and d in (kgb200.KG_BF16, kgb200.KG_F16))]


@pytest.mark.parametrize("name,dtype,shape", OTHER,
                         ids=["%s-%d-%s" % (n, d, "x".join(map(str, s))) for n, d, s in OTHER])
def test_tma_equals_other_engine(name, dtype, shape):
    """Same arithmetic, same expression: the TMA engine's output equals the
    direct (or, for float-float, the staged) engine's bit for bit."""
    case = ol.Case(name, shape)
    if name == "uxx1":
        d1 = case.arrays()[2]
        d1[:] = 1.5 + 0.5 * d1      # density away from 0, as for the narrow types
    other = "staged" if dtype == kgb200.KG_F64_FF else "direct"
    a = run(name, dtype, case.shape, case.coef, [x.copy() for x in case.arrays()], 3, "tma")
    b = run(name, dtype, case.shape, case.coef, [x.copy() for x in case.arrays()], 3, other)
    for q, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), \
            "%s slot %d: tma and %s differ (max |d| %g)" % (name, q, other, np.max(np.abs(x - y)))


VEC = [(n, d, s) for n in kgb200.STENCILS
       for d in (kgb200.KG_F32, kgb200.KG_BF16, kgb200.KG_F16)
       for s in shapes(n)]


@pytest.mark.parametrize("name,dtype,shape", VEC,
                         ids=["%s-%d-%s" % (n, d, "x".join(map(str, s))) for n, d, s in VEC])
def test_tma_vec_equals_direct(name, dtype, shape):
    """The vector TMA engine (4 consecutive points per thread) evaluates the
    same expressions: its output equals the direct engine's bit for bit,
    rims untouched, on tiles cut by the domain's edges in x, y and z (2D
    stencils: walked down bands of rows, the last band cut by the edge)."""
    case = ol.Case(name, shape)
    if name == "uxx1":
        d1 = case.arrays()[2]
        d1[:] = 1.5 + 0.5 * d1
    a = run(name, dtype, case.shape, case.coef, [x.copy() for x in case.arrays()], 3, "tmavec")
    b = run(name, dtype, case.shape, case.coef, [x.copy() for x in case.arrays()], 3, "direct")
    for q, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), \
            "%s slot %d: tmavec and direct differ (max |d| %g)" % (name, q, np.max(np.abs(x - y)))


def test_auto_engine_falls_back_on_unaligned_rows():
    """AUTO takes the direct engine where rows are not 16-byte multiples."""
    case = ol.Case("laplacian", (33, 17, 9))
    a = run("laplacian", kgb200.KG_F32, case.shape, case.coef, [x.copy() for x in case.arrays()], 2, "auto")
    b = run("laplacian", kgb200.KG_F32, case.shape, case.coef, [x.copy() for x in case.arrays()], 2, "direct")
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
