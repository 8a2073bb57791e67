"""The digit-recurrence division of the strict sweeps, restated in numpy.

se_div (kernelgen-perf-tests_gb300/csrc/kg_num.cuh) divides doubles exactly
on the integer and FP32 pipes: three signed quotient digits (20, 20, 13 bits)
estimated in FP32 from the running remainder times an approximate reciprocal
of the divisor, remainders updated exactly modulo 2^64, one correction of the
last digit, then round to nearest even from the 54-bit floor and its
remainder.  This restatement runs the same steps with numpy's IEEE FP32 and
wrapping uint64 arithmetic, with the reciprocal pushed to both ends of the
error bound the method assumes (2^-22 relative), and must equal IEEE double
division bit for bit.  (The GPU implementation itself is checked against IEEE
division in test_exact_arith_gpu.py.)
"""
import numpy as np
import pytest

MAGIC_BITS = np.uint32(0x4B400000)          # 1.5 * 2^23
MAGIC = np.float32(12582912.0)


def i2f(t):
    """int32 (|t| < 2^22) -> float32 through the 1.5 * 2^23 bit pattern."""
    return (MAGIC_BITS.astype(np.int64) + t.astype(np.int64)).astype(np.uint32).view(np.float32) - MAGIC


def f2i_rn(x):
    """float32 (|x| < 2^22) -> nearest int through the same pattern."""
    return (x + MAGIC).view(np.uint32).astype(np.int64) - int(MAGIC_BITS)


def digit_division(a, b, rcp_scale):
    A, B = a.view(np.uint64), b.view(np.uint64)
    ea = ((A >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    eb = ((B >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    frac, hidden = np.uint64(0xFFFFFFFFFFFFF), np.uint64(1 << 52)
    ma, mb = (A & frac) | hidden, (B & frac) | hidden
    sh = (ma < mb).astype(np.uint64)
    N = ma << sh
    E = ea - eb - sh.astype(np.int64) + 1023
    # rb ~ 2^52 / mb from mb's leading 24 bits
    fb = (np.uint64(0x3F800000) | ((mb >> np.uint64(29)) & np.uint64(0x7FFFFF))).astype(np.uint32).view(np.float32)
    rb = (np.float32(1.0) / fb) * np.float32(rcp_scale)
    with np.errstate(over="ignore"):
        d1 = f2i_rn(i2f((N >> np.uint64(32)).astype(np.int64)) * rb)
        R1 = (N << np.uint64(20)) - d1.astype(np.uint64) * mb
        d2 = f2i_rn(i2f(R1.view(np.int64) >> 33) * (np.float32(2.0) * rb))
        R2 = (R1 << np.uint64(20)) - d2.astype(np.uint64) * mb
        d3 = f2i_rn(i2f(R2.view(np.int64) >> 33) * (np.float32(0.015625) * rb))
        R3 = (R2 << np.uint64(13)) - d3.astype(np.uint64) * mb
    neg = (R3.view(np.int64) < 0).astype(np.uint64)
    Q = (d1.astype(np.uint64) << np.uint64(33)) + (d2.astype(np.uint64) << np.uint64(13)) + d3.astype(np.uint64) - neg
    R = R3 + np.where(neg == 1, mb, np.uint64(0))
    assert np.all(R < mb), "remainder out of [0, mb)"
    mant0 = Q >> np.uint64(1)
    up = (Q & np.uint64(1)) & ((R != 0).astype(np.uint64) | (mant0 & np.uint64(1)))
    mant = mant0 + up
    sign = (A ^ B) & np.uint64(1 << 63)
    ok = (ea >= 1) & (ea <= 2046) & (eb >= 1) & (eb <= 2046) & (E >= 1) & (E <= 2045)
    bits = sign | (((E - 1).astype(np.uint64) << np.uint64(52)) + mant)
    return bits.view(np.float64), ok


def operands(n, seed):
    rng = np.random.default_rng(seed)
    m = rng.integers(0, 2 ** 52, size=(2, n), dtype=np.uint64)
    kind = rng.integers(0, 8, size=n)
    m[1] = np.where(kind == 1, m[0], m[1])                                         # equal mantissas
    m[1] = np.where(kind == 2, (m[0] + np.uint64(1)) & np.uint64(2 ** 52 - 1), m[1])
    m[0] = np.where(kind == 3, np.uint64(2 ** 52 - 1), m[0])
    m[1] = np.where(kind == 4, np.uint64(0), m[1])                                  # power-of-two divisor
    e = 1023 + rng.integers(-100, 101, size=(2, n))
    x = ((e.astype(np.uint64) << np.uint64(52)) | m).view(np.float64)
    a, b = x[0].copy(), x[1].copy()
    a = np.where(kind == 5, b * rng.integers(1, 4096, size=n), a)                   # exact quotients
    return a, b


@pytest.mark.parametrize("rcp_scale", [1.0, 1 + 2.0 ** -22, 1 - 2.0 ** -22, 1 + 2.0 ** -23])
def test_digit_division_is_ieee(rcp_scale):
    a, b = operands(400_000, 7)
    got, ok = digit_division(a, b, rcp_scale)
    want = a / b
    assert ok.mean() > 0.99
    bad = ok & (got.view(np.uint64) != want.view(np.uint64))
    assert not bad.any(), (a[bad][:3], b[bad][:3], got[bad][:3], want[bad][:3])


def test_digit_division_small_integers():
    i, j = np.meshgrid(np.arange(1, 700, dtype=np.float64), np.arange(1, 700, dtype=np.float64))
    a, b = i.ravel(), j.ravel()
    got, ok = digit_division(a, b, 1.0)
    assert ok.all()
    assert np.array_equal(got.view(np.uint64), (a / b).view(np.uint64))
