"""The TMA engine's bounded waits: the give-up path, run without a fault.

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


def _sweep(name, dtype, shape, coef, bufs):
    p = kgb200.problem(name, dtype, shape, coef, [b.data_ptr() for b in bufs], engine="tma")
    kgb200.sweep(p)


@pytest.mark.parametrize("name,dtype,shape", [
    ("laplacian", kgb200.KG_F32, (64, 32, 40)),
    ("wave13pt", kgb200.KG_F64, (48, 24, 30)),
    ("gaussblur", kgb200.KG_F32, (128, 200)),
])
def test_wait_limit_zero_reports_timeout_then_recovers(name, dtype, shape):
    lib = kgb200.load()
    tdt = torch.float64 if dtype == kgb200.KG_F64 else torch.float32
    case = ol.Case(name, shape)
    bufs = [torch.from_numpy(a).to("cuda").to(tdt) for a in case.arrays()]
    kgb200.check(lib.kg_engine_status(None))       # clear any earlier record

    kgb200.check(lib.kg_set_tma_wait_limit(0))
    try:
        _sweep(name, dtype, case.shape, case.coef, bufs)
        torch.cuda.synchronize()                    # the context stays usable
        assert lib.kg_engine_status(None) == KG_ETIMEOUT
        assert b"gave up" in lib.kg_last_error()
        assert lib.kg_engine_status(None) == 0      # the record is cleared
    finally:
        kgb200.check(lib.kg_set_tma_wait_limit(-1))

    # default limit: a complete sweep from fresh inputs, checked against the oracle
    bufs = [torch.from_numpy(a).to("cuda").to(tdt) for a in case.arrays()]
    _sweep(name, dtype, case.shape, case.coef, bufs)
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
