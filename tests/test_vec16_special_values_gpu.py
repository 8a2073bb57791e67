"""16-bit storage on the vector TMA engine with special values.

With BF16 or FP16 storage the vector engine adds stored neighbours to FP32
sums by the mixed-precision add, which takes the 16-bit operand from its half
of a 32-bit word, where the direct engine widens every value first.  Both are
the IEEE sum of the same FP32 values, so their outputs must agree bit for bit
also on subnormal, zero, infinite and NaN inputs (a NaN leaves as the storage
type's canonical NaN either way).  Random finite values are covered by
test_engines_gpu.py; here a share of every input is replaced by special
values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    kgb200.check(kgb200.load().kg_device_check())


SPECIAL = {
    # bit patterns: +-0, +-inf, quiet NaN with a payload, the smallest and the
    # largest subnormal, the largest finite
    kgb200.KG_BF16: [0x0000, 0x8000, 0x7F80, 0xFF80, 0x7FC1, 0x0001, 0x807F, 0x7F7F],
    kgb200.KG_F16: [0x0000, 0x8000, 0x7C00, 0xFC00, 0x7E01, 0x0001, 0x83FF, 0x7BFF],
}
TDT = {kgb200.KG_BF16: torch.bfloat16, kgb200.KG_F16: torch.float16}
CASES = [("laplacian", (136, 20, 17)), ("divergence", (136, 20, 17)), ("wave13pt", (136, 20, 17)),
         ("uxx1", (136, 20, 17)), ("lapgsrb", (136, 20, 17)), ("gaussblur", (264, 77)), ("gameoflife", (264, 77))]


def _inputs(name, dtype, shape, seed):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    narr = kgb200.load().kg_stencil_narrays(kgb200.STENCIL_ID[name])
    arrays = []
    for q in range(narr):
        v = torch.from_numpy(rng.uniform(-1, 1, n).astype(np.float32)).to(TDT[dtype])
        bits = v.view(torch.int16).numpy().copy()
        pick = rng.random(n) < 0.08
        bits[pick] = np.array(SPECIAL[dtype], dtype=np.uint16)[rng.integers(0, len(SPECIAL[dtype]), pick.sum())].view(np.int16)
        arrays.append(torch.from_numpy(bits).view(TDT[dtype]))
    return arrays


@pytest.mark.parametrize("dtype", [kgb200.KG_BF16, kgb200.KG_F16], ids=["bf16", "f16"])
@pytest.mark.parametrize("name,shape", CASES, ids=[c[0] for c in CASES])
def test_vector_engine_equals_direct_on_special_values(name, shape, dtype):
    host = _inputs(name, dtype, shape, seed=len(name) + dtype)
    coef = [0.3, 0.1, 0.05, 0.02, 0.01, 0.005]
    out = {}
    for engine in ("tmavec", "direct"):
        bufs = [a.cuda() for a in host]
        ptrs = [b.data_ptr() for b in bufs]
        kgb200.sweep(kgb200.problem(name, dtype, shape, coef, ptrs, engine=engine))
        torch.cuda.synchronize()
        kgb200.engine_status()
        out[engine] = [b.view(torch.int16).cpu().numpy() for b in bufs]
    for q, (a, b) in enumerate(zip(out["tmavec"], out["direct"])):
        assert np.array_equal(a, b), "%s array %d: %d of %d elements differ" % (name, q, int((a != b).sum()), a.size)
