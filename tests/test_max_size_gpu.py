"""Sizes at the limits, on the GPU through the C ABI.

* Arrays beyond 2^31 and 2^32 points (64-bit indexing in every engine): a
  sweep's output at a point depends only on its neighbours, so the last
  planes (rows, for 2D stencils) of a full-size sweep must equal the same
  sweep of a small array cut from the last planes of the inputs.  That small
  sweep is checked against the oracle (bit for bit for KG_F64 and byte
  cells), and the full-size one against it bit for bit for every type.
  The window's first planes are its rim (left unchanged by the small sweep)
  and are not compared.
* Tile grids beyond the launch limit of 65535 along y and z, checked whole
  against the oracle.

The full-size cases hold at most 70 GB of device memory each and free it
before the next one.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

W = 6      # planes (rows) in the window
SKIP = 3   # the window's rim planes at its start (every stencil reaches <= 2)


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def coef_of(name):
    return ol.Case(name, (5, 5) if name in kgb200.IS2D else (5, 5, 5)).coef


def device_inputs(name, n, tdt, gen):
    """Uniform [-1, 1) arrays (tricubic offsets in [0, 1)) made on the device."""
    narr = kgb200.load().kg_stencil_narrays(kgb200.STENCIL_ID[name])
    out = []
    for q in range(narr):
        if tdt == torch.uint8:
            out.append((torch.rand(n, device="cuda", generator=gen) < 0.3).to(torch.uint8))
            continue
        a = torch.rand(n, dtype=torch.float32 if tdt != torch.float64 else torch.float64,
                       device="cuda", generator=gen)
        if not (name.startswith("tricubic") and q >= 2):
            a.mul_(2).sub_(1)
        out.append(a.to(tdt))
    return out


def window_of(bufs, plane, planes):
    """The last `planes` planes (plane = points per plane) of every array."""
    return [b[b.numel() - plane * planes:].clone() for b in bufs]


def run_sweep(name, dtype, shape, bufs, engine):
    kgb200.sweep(kgb200.problem(name, dtype, shape, coef_of(name), [b.data_ptr() for b in bufs], engine))
    kgb200.engine_status()
    torch.cuda.synchronize()


FAR = [
    # (stencil, dtype, engine, shape); points > 2^32 unless noted
    ("laplacian", kgb200.KG_F64, kgb200.KG_ENGINE_DIRECT, (2048, 2048, 1025)),
    ("laplacian", kgb200.KG_F32, kgb200.KG_ENGINE_TMA, (2048, 2048, 1025)),
    ("wave13pt", kgb200.KG_F64_FF, kgb200.KG_ENGINE_STAGED, (1024, 1024, 2049)),      # > 2^31
    ("uxx1", kgb200.KG_F32, kgb200.KG_ENGINE_TMA, (1024, 1024, 2049)),               # > 2^31
    ("tricubic", kgb200.KG_F32, kgb200.KG_ENGINE_DIRECT, (1024, 1024, 2049)),        # > 2^31
    ("gaussblur", kgb200.KG_F64, kgb200.KG_ENGINE_AUTO, (65536, 65600)),
    ("gameoflife", kgb200.KG_U8, kgb200.KG_ENGINE_AUTO, (65536, 65600)),
]
TDT = {kgb200.KG_F64: torch.float64, kgb200.KG_F64_FF: torch.float64, kgb200.KG_F32: torch.float32,
       kgb200.KG_U8: torch.uint8}


@pytest.mark.parametrize("name,dtype,engine,shape", FAR,
                         ids=["%s-%d-%s" % (c[0], c[1], "x".join(map(str, c[3]))) for c in FAR])
def test_far_end_of_large_arrays(name, dtype, engine, shape):
    is2d = len(shape) == 2
    plane = shape[0] if is2d else shape[0] * shape[1]
    n = plane * shape[-1]
    assert n > 2 ** 31
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    bufs = device_inputs(name, n, TDT[dtype], gen)
    before = window_of(bufs, plane, W)
    try:
        run_sweep(name, dtype, shape, bufs, engine)
        after = window_of(bufs, plane, W)
    finally:
        del bufs
        torch.cuda.empty_cache()
    wshape = (shape[0], W) if is2d else (shape[0], shape[1], W)
    small = [b.clone() for b in before]
    run_sweep(name, dtype, wshape, small, engine)
    for q, (a, s) in enumerate(zip(after, small)):
        a = a[plane * SKIP:].cpu().numpy()
        s = s[plane * SKIP:].cpu().numpy()
        assert np.array_equal(a.view(np.uint8), s.view(np.uint8)), "array %d differs from the small sweep" % q
    # the small sweep against the oracle
    if dtype == kgb200.KG_F64:
        case = ol.Case.from_arrays(name, wshape, coef_of(name), [b.cpu().numpy() for b in before])
        case.sweep()
        for q, (s, o) in enumerate(zip(small, case.buffers)):
            assert np.array_equal(s[plane * SKIP:].cpu().numpy().view(np.uint64),
                                  o[plane * SKIP:].view(np.uint64)), "array %d differs from the oracle" % q
    elif dtype == kgb200.KG_U8:
        u0, u1 = (b.cpu().numpy() for b in before)
        want = ol.conway_u8(u0, u1, shape[0], W)
        assert np.array_equal(small[1][plane * SKIP:].cpu().numpy(), want[plane * SKIP:])


TALL = [
    # (stencil, dtype, engine, shape): tiles beyond 65535 along y (or z)
    ("laplacian", kgb200.KG_F64_FF, kgb200.KG_ENGINE_STAGED, (5, 600000, 4)),
    ("divergence", kgb200.KG_F64_FF, kgb200.KG_ENGINE_AUTO, (40, 540000, 3)),
    ("laplacian", kgb200.KG_F64, kgb200.KG_ENGINE_DIRECT, (5, 600000, 4)),
    ("gradient", kgb200.KG_F64, kgb200.KG_ENGINE_DIRECT, (5, 3, 600000)),
    ("lapgsrb", kgb200.KG_F64, kgb200.KG_ENGINE_AUTO, (4, 4, 1100000)),
    ("lapgsrb", kgb200.KG_F32, kgb200.KG_ENGINE_TMA, (8, 1100000, 3)),
    ("jacobi", kgb200.KG_F64_FF, kgb200.KG_ENGINE_STAGED, (7, 2200000)),
    ("gameoflife", kgb200.KG_F64, kgb200.KG_ENGINE_AUTO, (3, 2200000)),
]


@pytest.mark.parametrize("name,dtype,engine,shape", TALL,
                         ids=["%s-%d-%d-%s" % (c[0], c[1], c[2], "x".join(map(str, c[3]))) for c in TALL])
def test_grids_beyond_launch_limits(name, dtype, engine, shape):
    case = ol.Case(name, shape)
    arrays = [a.copy() for a in case.arrays()]
    tdt = TDT[dtype]
    bufs = [torch.from_numpy(a).cuda().to(tdt) for a in arrays]
    run_sweep(name, dtype, shape, bufs, engine)
    case.sweep()
    for q, (g, w) in enumerate(zip(bufs, case.arrays())):
        g = g.double().cpu().numpy()
        if dtype == kgb200.KG_F64:
            assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), "array %d differs" % q
        else:
            # float-float ~1e-14 of FP64; FP32 storage 2^-24 per value
            tol = 1e-12 if dtype == kgb200.KG_F64_FF else 2e-6
            m = float(np.max(np.abs(w)))
            assert float(np.max(np.abs(g - w))) <= tol * m, "array %d beyond %g" % (q, tol)
