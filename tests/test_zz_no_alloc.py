"""kg_checksum_noalloc: the checksum for callers that cannot allocate.

Some callers of this library may not allocate device memory once they run:
a host framework that owns every byte of device memory through its own
arena, or a latency-critical loop that cannot accept the synchronisation a
cudaMalloc/cudaFree may cause.  For them kg_checksum_noalloc keeps its
partial sums in a fixed device array compiled into the library instead of
taking scratch from the stream-ordered pool as kg_checksum does.

The two entry points run the same two-level tree, so their results must be
equal bit for bit.  The no-allocation promise is checked on the device's
current stream-ordered pool: its high-water mark of used memory, reset before
the call, must stay where it was (kg_checksum, which does take its scratch
from that pool, moves it: the check is shown to see an allocation).

This file is collected last (the name sorts after the other test files), so
a run that stops at the first failure has run everything else first.  It must
pass alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

# cudaMemPoolAttr values (driver_types.h)
USED_MEM_CURRENT, USED_MEM_HIGH = 0x7, 0x8


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def _call(fn, dtype, arrays, n, out):
    ptrs = (ctypes.c_void_p * len(arrays))(*[a.data_ptr() for a in arrays])
    kgb200.check(fn(dtype, n, len(arrays), ptrs, out.data_ptr(), None))


def _sum_both(dtype, arrays, n):
    lib = kgb200.load()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    _call(lib.kg_checksum, dtype, arrays, n, out)
    _call(lib.kg_checksum_noalloc, dtype, arrays, n, out[1:])
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _arrays(rng, dtype, n, narr):
    if dtype == kgb200.KG_U8:
        return [torch.from_numpy(rng.integers(0, 2, n, dtype=np.uint8)).cuda() for _ in range(narr)]
    tdt = {kgb200.KG_F64: torch.float64, kgb200.KG_F32: torch.float32,
           kgb200.KG_BF16: torch.bfloat16, kgb200.KG_F16: torch.float16}[dtype]
    return [torch.from_numpy(rng.uniform(-1, 1, n)).to(tdt).cuda() for _ in range(narr)]


@pytest.mark.parametrize("dtype", [kgb200.KG_F64, kgb200.KG_F32, kgb200.KG_BF16, kgb200.KG_F16, kgb200.KG_U8])
def test_noalloc_matches_checksum_twice(dtype):
    """Two calls in a row, different sizes, array counts and data: each equals
    kg_checksum bit for bit (the second call sees the first call's partials
    left in the array)."""
    rng = np.random.default_rng(11 + dtype)
    for n, narr in ((5_000_003, 3), (777_777, 6), (1, 1)):
        xs = _arrays(rng, dtype, n, narr)
        ref, got = _sum_both(dtype, xs, n)
        assert np.float64(got).view(np.uint64) == np.float64(ref).view(np.uint64), (n, narr, got, ref)


class _Cudart:
    """The CUDA runtime the library is linked against (already loaded)."""

    def __init__(self):
        self.lib = ctypes.CDLL("libcudart.so.13")

    def pool(self):
        dev = ctypes.c_int()
        assert self.lib.cudaGetDevice(ctypes.byref(dev)) == 0
        pool = ctypes.c_void_p()
        assert self.lib.cudaDeviceGetMemPool(ctypes.byref(pool), dev.value) == 0
        return pool

    def get(self, pool, attr):
        v = ctypes.c_uint64()
        assert self.lib.cudaMemPoolGetAttribute(pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self, pool):
        zero = ctypes.c_uint64(0)   # resets the high-water mark to the current use
        assert self.lib.cudaMemPoolSetAttribute(pool, USED_MEM_HIGH, ctypes.byref(zero)) == 0


def test_noalloc_takes_nothing_from_the_pool():
    lib = kgb200.load()
    rt = _Cudart()
    rng = np.random.default_rng(5)
    n = 3_000_001
    xs = _arrays(rng, kgb200.KG_F64, n, 2)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # one call first: module loading on first use is not part of the promise
    _call(lib.kg_checksum_noalloc, kgb200.KG_F64, xs, n, out)
    torch.cuda.synchronize()
    pool = rt.pool()

    def high_after(fn):
        torch.cuda.synchronize()
        rt.reset_high(pool)
        base = rt.get(pool, USED_MEM_CURRENT)
        _call(fn, kgb200.KG_F64, xs, n, out)
        torch.cuda.synchronize()
        return max(rt.get(pool, USED_MEM_HIGH) - base, 0)

    assert high_after(lib.kg_checksum_noalloc) == 0
    assert high_after(lib.kg_checksum) > 0      # the check sees kg_checksum's scratch
    assert high_after(lib.kg_checksum_noalloc) == 0


def test_noalloc_rejects_sizes_beyond_the_maximum():
    lib = kgb200.load()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ptrs = (ctypes.c_void_p * 1)(x.data_ptr())
    too_many = (1 << 33) + 1
    rc = lib.kg_checksum_noalloc(kgb200.KG_F64, too_many, 1, ptrs, out.data_ptr(), None)
    assert rc == 1
    assert b"exceeds the maximum" in lib.kg_last_error()
