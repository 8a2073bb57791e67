"""The bounded waits of the TMA engines (tiled and vector) and of the
tensor-core matmul: the give-up path, run without a fault.

A compute warp that waits longer than the wait limit for a step's tile copies
raises the CTA's abort flag and the device error flag and returns; the
producer stops issuing and waits for the copies it issued before the CTA
exits, and kg_engine_status reports KG_ETIMEOUT.  With the limit set to 0 a
warp gives up unless its copies have already landed when it first looks,
which the first step of a run never finds (the copies were issued a few
cycles earlier), so every CTA takes the path: an ordinary, in-bounds sweep
whose waits run out.  Afterwards the default limit gives complete sweeps
again, bit for bit the oracle's.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

KG_ETIMEOUT = 4


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())
    yield
    kgb200.load().kg_set_tma_wait_limit(-1)


def _sweep(name, dtype, shape, coef, bufs, engine="tma"):
    p = kgb200.problem(name, dtype, shape, coef, [b.data_ptr() for b in bufs], engine=engine)
    kgb200.sweep(p)


@pytest.mark.parametrize("name,dtype,shape,engine", [
    ("laplacian", kgb200.KG_F32, (64, 32, 40), "tma"),
    ("wave13pt", kgb200.KG_F64, (48, 24, 30), "tma"),
    ("gaussblur", kgb200.KG_F32, (128, 200), "tma"),
    ("laplacian", kgb200.KG_F32, (128, 32, 40), "tmavec"),
    ("wave13pt", kgb200.KG_BF16, (128, 24, 30), "tmavec"),
    ("gaussblur", kgb200.KG_F32, (128, 200), "tmavec"),
])
def test_wait_limit_zero_reports_timeout_then_recovers(name, dtype, shape, engine):
    lib = kgb200.load()
    tdt = {kgb200.KG_F64: torch.float64, kgb200.KG_F32: torch.float32, kgb200.KG_BF16: torch.bfloat16}[dtype]
    case = ol.Case(name, shape)
    bufs = [torch.from_numpy(a).to("cuda").to(tdt) for a in case.arrays()]
    kgb200.check(lib.kg_engine_status(None))       # clear any earlier record

    kgb200.check(lib.kg_set_tma_wait_limit(0))
    try:
        _sweep(name, dtype, case.shape, case.coef, bufs, engine)
        torch.cuda.synchronize()                    # the context stays usable
        assert lib.kg_engine_status(None) == KG_ETIMEOUT
        assert b"gave up" in lib.kg_last_error()
        assert lib.kg_engine_status(None) == 0      # the record is cleared
    finally:
        kgb200.check(lib.kg_set_tma_wait_limit(-1))

    # default limit: a complete sweep from fresh inputs, checked against the oracle
    bufs = [torch.from_numpy(a).to("cuda").to(tdt) for a in case.arrays()]
    _sweep(name, dtype, case.shape, case.coef, bufs, engine)
    torch.cuda.synchronize()
    kgb200.check(lib.kg_engine_status(None))
    if dtype == kgb200.KG_F64:
        case.sweep()
        for b, w in zip(bufs, case.arrays()):
            assert np.array_equal(b.cpu().numpy().view(np.uint64), w.view(np.uint64))
    else:
        ref = [torch.from_numpy(a).to("cuda").to(tdt) for a in case.arrays()]
        _sweep_direct = kgb200.problem(name, dtype, case.shape, case.coef, [b.data_ptr() for b in ref],
                                       engine="direct")
        kgb200.sweep(_sweep_direct)
        torch.cuda.synchronize()
        for b, r in zip(bufs, ref):
            assert torch.equal(b, r)


def test_matmul_tc_wait_limit_zero_reports_timeout_then_recovers():
    """The tensor-core matmul's MMA thread waits for its stages with the same
    limit: at 0 it gives up, the producer drains its copies, the epilogue adds
    nothing, the tensor memory is released (the next launch allocates it
    again), and kg_engine_status reports KG_ETIMEOUT."""
    lib = kgb200.load()
    nx, ny, ns = 256, 512, 256
    rng = np.random.default_rng(11)
    A = torch.from_numpy(rng.uniform(-1, 1, nx * ny).astype(np.float32)).cuda()
    B = torch.from_numpy(rng.uniform(-1, 1, ny * ns).astype(np.float32)).cuda()
    C = torch.zeros(nx * ns, dtype=torch.float32, device="cuda")
    kgb200.check(lib.kg_engine_status(None))
    kgb200.check(lib.kg_set_tma_wait_limit(0))
    try:
        kgb200.check(lib.kg_matmul_tc(nx, ny, ns, A.data_ptr(), B.data_ptr(), C.data_ptr(), None))
        torch.cuda.synchronize()
        assert lib.kg_engine_status(None) == KG_ETIMEOUT
    finally:
        kgb200.check(lib.kg_set_tma_wait_limit(-1))
    C.zero_()
    kgb200.check(lib.kg_matmul_tc(nx, ny, ns, A.data_ptr(), B.data_ptr(), C.data_ptr(), None))
    torch.cuda.synchronize()
    kgb200.check(lib.kg_engine_status(None))
    ref = B.double().cpu().numpy().reshape(ns, ny) @ A.double().cpu().numpy().reshape(ny, nx)
    assert np.max(np.abs(C.double().cpu().numpy().reshape(ns, nx) - ref)) <= 1e-5 * np.max(np.abs(ref))
