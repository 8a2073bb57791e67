"""Full-size parity: every stencil at the suite's own size, whole arrays.

`benchmark 512 256 256 10` runs the 3D tests on 512x256x256 and the 2D tests
on 512x65536 (their makefiles pass NY*NS, gameoflife/gcc/makefile:45-46) for
ten sweeps from the reference main()'s rand() draws.  Here every buffer of
every test, rims included, in its final role after those ten sweeps, is
compared with the oracle run on the same inputs:

* KG_F64 through kg_sweep (one call per sweep, the reference loop's shape,
  laplacian/laplacian.c:287-301) and through a plan (the ten sweeps as one
  CUDA graph; tricubic and tricubic2 evaluate their loop-invariant weights
  once into weight planes, the path bench.py times): bit for bit the strict
  oracle, and within 1e-12 normwise of the oracle built with the suite's
  fast-math flags (the gcc target);
* KG_F64_FMA: within 1e-12 normwise of the fast-math oracle;
* the project-defined inputs of the full-suite workload: gameoflife on
  Bernoulli(0.3) byte cells (KG_U8) equals the reference rule on the same
  0/1 cells thresholded at 0.5, and tricubic/tricubic2 with offsets in [0,1)
  equal the strict oracle bit for bit.

The oracle runs on all host cores (OpenMP over planes; every point's
arithmetic is unchanged), a few seconds per test.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

SHAPE3 = (512, 256, 256)
SHAPE2 = (512, 256 * 256)
NT = 10


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def shape_of(name):
    return SHAPE2 if name in kgb200.IS2D else SHAPE3


def normwise(x, ref):
    m = float(np.max(np.abs(ref)))
    return float(np.max(np.abs(x - ref))) / m if m > 0 else float(np.max(np.abs(x)))


def same_bits(a, b):
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


def gpu_sweeps(name, dtype, shape, coef, arrays):
    """NT kg_sweep calls with the reference's rotation; arrays in final roles."""
    bufs = [torch.from_numpy(a).to("cuda") for a in arrays]
    by_ptr = {b.data_ptr(): b for b in bufs}
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(NT):
        kgb200.sweep(kgb200.problem(name, dtype, shape, coef, ptrs))
        ptrs = kgb200.rotate(name, ptrs)
    torch.cuda.synchronize()
    kgb200.engine_status()
    return [by_ptr[p].cpu().numpy() for p in ptrs]


def gpu_plan(name, dtype, shape, coef, arrays):
    """The NT sweeps as one plan (CUDA graph); arrays in final roles."""
    bufs = [torch.from_numpy(a).to("cuda") for a in arrays]
    by_ptr = {b.data_ptr(): b for b in bufs}
    plan = kgb200.Plan(kgb200.problem(name, dtype, shape, coef, [b.data_ptr() for b in bufs]), NT)
    plan.launch()
    torch.cuda.synchronize()
    kgb200.engine_status()
    roles = plan.final_roles()
    plan.close()
    n = kgb200.load().kg_stencil_narrays(kgb200.STENCIL_ID[name])
    out = [by_ptr[roles.arr[q]].cpu().numpy() for q in range(n)]
    del bufs
    torch.cuda.empty_cache()
    return out


def oracle_after(case):
    case.run(NT)
    return [a.copy() for a in case.arrays()]


@pytest.mark.parametrize("name", kgb200.STENCILS)
def test_full_size_f64(name):
    shape = shape_of(name)
    strict = ol.Case(name, shape)
    init = [a.copy() for a in strict.arrays()]
    coef = strict.coef
    fast = ol.Case.from_arrays(name, shape, coef, init, flavour="fast")
    want = oracle_after(strict)
    want_fast = oracle_after(fast)
    for path, got in (("kg_sweep", gpu_sweeps(name, kgb200.KG_F64, strict.shape, coef, init)),
                      ("plan", gpu_plan(name, kgb200.KG_F64, strict.shape, coef, init))):
        for q, (g, w, wf) in enumerate(zip(got, want, want_fast)):
            assert same_bits(g, w), "%s %s slot %d: %d points differ from the strict oracle" % (
                name, path, q, int(np.sum(g.view(np.uint64) != w.view(np.uint64))))
            if name != "gameoflife":
                assert normwise(g, wf) <= 1e-12, (name, path, q, normwise(g, wf))
            else:
                # the smooth rule 1/(1 + x 1e20) amplifies a last-bit difference
                # of x; the cells it makes live or dead must agree
                assert np.array_equal(g > 0.5, wf > 0.5)


@pytest.mark.parametrize("name", kgb200.STENCILS)
def test_full_size_f64fma_vs_fast_oracle(name):
    shape = shape_of(name)
    fast = ol.Case(name, shape, flavour="fast")
    init = [a.copy() for a in fast.arrays()]
    want = oracle_after(fast)
    got = gpu_plan(name, kgb200.KG_F64_FMA, fast.shape, fast.coef, init)
    for q, (g, w) in enumerate(zip(got, want)):
        if name == "gameoflife":
            assert np.array_equal(g > 0.5, w > 0.5)
        else:
            assert normwise(g, w) <= 1e-12, (name, q, normwise(g, w))


def test_full_size_gameoflife_u8_bernoulli():
    """512x65536 Bernoulli(0.3) cells (both buffers, rims included), ten
    sweeps: the byte kernel's B3/S23 cells equal the reference rule run on
    the same cells as doubles, thresholded at 0.5, sweep after sweep."""
    shape = SHAPE2
    case = ol.Case("gameoflife", shape, variant=ol.INIT_BERNOULLI)
    init = [a.copy() for a in case.arrays()]
    bufs = [torch.from_numpy(a.astype(np.uint8)).to("cuda") for a in init]
    by_ptr = {b.data_ptr(): b for b in bufs}
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(NT):
        kgb200.sweep(kgb200.problem("gameoflife", kgb200.KG_U8, shape, [], ptrs))
        ptrs = kgb200.rotate("gameoflife", ptrs)
        case.run(1)                     # one sweep and the reference's swap
        torch.cuda.synchronize()
        got = [by_ptr[p].cpu().numpy() for p in ptrs]
        for g, w in zip(got, case.arrays()):
            assert np.array_equal(g, (w > 0.5).astype(np.uint8))


@pytest.mark.parametrize("name", ["tricubic", "tricubic2"])
def test_full_size_tricubic_unit_offsets(name):
    """Offsets a, b, c drawn in [0,1) (the full-suite workload's tricubic
    inputs): the plan path (weights once) equals the strict oracle bit for
    bit."""
    case = ol.Case(name, SHAPE3, variant=ol.INIT_UNIT_OFFSETS)
    init = [a.copy() for a in case.arrays()]
    want = oracle_after(case)
    got = gpu_plan(name, kgb200.KG_F64, case.shape, case.coef, init)
    for q, (g, w) in enumerate(zip(got, want)):
        assert same_bits(g, w), "%s slot %d differs" % (name, q)
