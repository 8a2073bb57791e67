"""kg_checksum_noalloc: the checksum for callers that cannot allocate.

Some callers of this library may not allocate device memory once they run:
a host framework that owns every byte of device memory through its own
arena, or a latency-critical loop that cannot accept the synchronisation a
cudaMalloc/cudaFree may cause.  For them kg_checksum_noalloc keeps its
partial sums in a fixed device array compiled into the library instead of
taking scratch from the stream-ordered pool as kg_checksum does.

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

# The tolerance the checksum tests use: relative to the sum of magnitudes.
REL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


def _sum_both(dtype, arrays, n):
    lib = kgb200.load()
    ptrs = (ctypes.c_void_p * len(arrays))(*[a.data_ptr() for a in arrays])
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    kgb200.check(lib.kg_checksum(dtype, n, len(arrays), ptrs, out.data_ptr(), None))
    kgb200.check(lib.kg_checksum_noalloc(dtype, n, len(arrays), ptrs, out[1:].data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("dtype,tdt", [(kgb200.KG_F64, torch.float64), (kgb200.KG_F32, torch.float32)])
def test_noalloc_matches_checksum_twice(dtype, tdt):
    """Two calls in a row, different sizes and data: each equals kg_checksum
    (the second call sees the first call's partials left in the array)."""
    rng = np.random.default_rng(11)
    for n, narr in ((5_000_003, 3), (777_777, 2)):
        xs = [torch.from_numpy(rng.uniform(-1, 1, n)).to(tdt).cuda() for _ in range(narr)]
        ref, got = _sum_both(dtype, xs, n)
        mag = float(sum(x.double().abs().sum().item() for x in xs))
        assert abs(got - ref) <= REL * mag


def test_noalloc_rejects_sizes_beyond_the_maximum():
    lib = kgb200.load()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ptrs = (ctypes.c_void_p * 1)(x.data_ptr())
    too_many = (1 << 33) + 1
    rc = lib.kg_checksum_noalloc(kgb200.KG_F64, too_many, 1, ptrs, out.data_ptr(), None)
    assert rc == 1
    assert b"exceeds the maximum" in lib.kg_last_error()
