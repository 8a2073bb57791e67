"""The strict sweeps' FP64 arithmetic on the integer pipes, bit for bit.

KG_F64 sweeps form coefficient products (se_mul), tricubic's products and
uxx1's and gameoflife's divisions (se_div) from integer and FP32 operations
instead of the FP64 unit; kg_exact_arith exposes them element-wise.  They
must equal IEEE round-to-nearest-even arithmetic (numpy on the host, and the
FP64 unit on the device) on every operand: random values over the whole
exponent range, mantissa patterns that stress rounding and carries, exact
results, and zeros, subnormals, infinities and NaNs (NaNs compare as NaN).
The sweeps themselves are then run on inputs holding such values and
compared with the oracle.
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


SPECIAL = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 2.225073858507201e-308,
                    1.7976931348623157e308, -1.7976931348623157e308, np.inf, -np.inf, np.nan,
                    1.0, -1.0, 2.0, 0.5, 3.0, 1.0 + 2.0 ** -52, 1.0 - 2.0 ** -53, 2.0 ** 1023, 2.0 ** -1022,
                    1e300, 1e-300, 0.1, 1.0 / 3.0])


def operands(n, seed):
    rng = np.random.default_rng(seed)
    mant = rng.integers(0, 2 ** 52, size=(2, n), dtype=np.uint64)
    kind = rng.integers(0, 12, size=n)
    # mantissa patterns: equal, adjacent, all ones, zero
    mant[1] = np.where(kind == 1, mant[0], mant[1])
    mant[1] = np.where(kind == 2, (mant[0] + np.uint64(1)) & np.uint64(2 ** 52 - 1), mant[1])
    mant[0] = np.where(kind == 3, np.uint64(2 ** 52 - 1), mant[0])
    mant[1] = np.where(kind == 4, np.uint64(0), mant[1])
    wide = kind >= 9                                  # the whole exponent range
    exp = np.where(wide, rng.integers(1, 2047, size=(2, n)), 1023 + rng.integers(-60, 61, size=(2, n)))
    sign = rng.integers(0, 2, size=(2, n)).astype(np.uint64) << np.uint64(63)
    x = (sign | (exp.astype(np.uint64) << np.uint64(52)) | mant).view(np.float64)
    a, b = x[0].copy(), x[1].copy()
    # near cancellation, far-apart exponents, exact quotients
    b = np.where(kind == 5, -a * (1.0 + 2.0 ** -52 * rng.integers(0, 4, size=n)), b)
    b = np.where(kind == 6, a * 2.0 ** -53, b)
    with np.errstate(over="ignore", invalid="ignore"):
        a = np.where(kind == 7, b * rng.integers(1, 1000, size=n).astype(np.float64), a)
    b = np.where(kind == 8, a * (1.0 + 2.0 ** -52 * rng.integers(0, 5, size=n)), b)
    # every pair of special values
    s = np.array(np.meshgrid(SPECIAL, SPECIAL)).reshape(2, -1)
    return np.concatenate([a, s[0]]), np.concatenate([b, s[1]])


def same(x, y):
    return (x.view(np.uint64) == y.view(np.uint64)) | (np.isnan(x) & np.isnan(y))


OPS = [("add", kgb200.KG_ARITH_ADD, kgb200.KG_ARITH_NATIVE_ADD, np.add),
       ("mul", kgb200.KG_ARITH_MUL, kgb200.KG_ARITH_NATIVE_MUL, np.multiply),
       ("div", kgb200.KG_ARITH_DIV, kgb200.KG_ARITH_NATIVE_DIV, np.divide)]


@pytest.mark.parametrize("name,op,native,ref", OPS, ids=[o[0] for o in OPS])
@pytest.mark.parametrize("seed", [1, 2])
def test_integer_pipe_arithmetic_is_ieee(name, op, native, ref, seed):
    a, b = operands(1 << 22, seed)
    lib = kgb200.load()
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out, nat = torch.empty_like(da), torch.empty_like(da)
    kgb200.check(lib.kg_exact_arith(op, a.size, da.data_ptr(), db.data_ptr(), out.data_ptr(), None))
    kgb200.check(lib.kg_exact_arith(native, a.size, da.data_ptr(), db.data_ptr(), nat.data_ptr(), None))
    got, fpu = out.cpu().numpy(), nat.cpu().numpy()
    with np.errstate(all="ignore"):
        want = ref(a, b)
    bad = ~same(got, want)
    assert not bad.any(), "%s: %d of %d differ, e.g. %r (op) %r = %r, IEEE %r" % (
        name, int(bad.sum()), a.size, a[bad][0], b[bad][0], got[bad][0], want[bad][0])
    assert same(got, fpu).all()


def test_exact_arith_argument_errors():
    lib = kgb200.load()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert lib.kg_exact_arith(9, 4, x.data_ptr(), x.data_ptr(), x.data_ptr(), None) == 1
    assert lib.kg_exact_arith(0, 4, None, x.data_ptr(), x.data_ptr(), None) == 1
    assert lib.kg_exact_arith(0, 0, None, None, None, None) == 0


@pytest.mark.parametrize("name", ["laplacian", "uxx1", "tricubic", "gameoflife", "gaussblur", "divergence"])
def test_sweeps_on_special_values(name):
    """KG_F64 sweeps of inputs sprinkled with zeros, subnormals, huge values,
    infinities and NaNs equal the strict oracle (NaN as NaN)."""
    shape = (129, 300) if name in kgb200.IS2D else (33, 17, 9)
    case = ol.Case(name, shape)
    rng = np.random.default_rng(5)
    arrays = [a.copy() for a in case.arrays()]
    for a in arrays:
        idx = rng.integers(0, a.size, size=a.size // 20)
        a[idx] = rng.choice(SPECIAL, size=idx.size)
        big = rng.integers(0, a.size, size=a.size // 20)
        a[big] *= rng.choice([1e300, 1e-300, 2.0 ** 1000, 2.0 ** -1060], size=big.size)
    case = ol.Case.from_arrays(name, shape, case.coef, arrays)
    bufs = [torch.from_numpy(a.copy()).cuda() for a in arrays]
    kgb200.sweep(kgb200.problem(name, kgb200.KG_F64, shape, case.coef, [b.data_ptr() for b in bufs]))
    torch.cuda.synchronize()
    with np.errstate(all="ignore"):
        case.sweep()
    for q, (g, w) in enumerate(zip(bufs, case.buffers)):
        g = g.cpu().numpy()
        bad = ~same(g, w)
        assert not bad.any(), "array %d: %d points differ" % (q, int(bad.sum()))
