"""The exact integer-pipe addition and multiplication of the strict sweeps,
restated in numpy.

se_add and se_mul (kernelgen-perf-tests_gb300/csrc/kg_num.cuh) add and
multiply normal doubles with 32/64-bit integer arithmetic: operands swapped
by magnitude (compared as 32-bit words), mantissas with the hidden bit at bit
62, the smaller one aligned with its lost bits kept as a sticky bit, the same-
sign sum and the opposite-sign difference (normalised by its leading zeros)
both formed, round to nearest even from the guard and sticky bits; products
from four 32 x 32 -> 64-bit partial products.  This restatement runs the same
steps on numpy's wrapping uint64 and must equal IEEE arithmetic bit for bit
wherever the fast path applies (the rest goes to the FP64 unit).  The GPU
implementations are checked against IEEE in test_exact_arith_gpu.py.
"""
import numpy as np

U = np.uint64


def clz64(x):
    """Leading zeros of uint64 values (64 for zero)."""
    n = np.zeros(x.shape, dtype=np.int64)
    y = x.copy()
    for s in (32, 16, 8, 4, 2, 1):
        small = y < (U(1) << U(64 - s))
        n += np.where(small, s, 0)
        y = np.where(small, y << U(s), y)
    return np.where(x == 0, 64, n)


def add_restated(a, b):
    A, B = a.view(U), b.view(U)
    ah, bh = (A >> U(32)) & U(0x7FFFFFFF), (B >> U(32)) & U(0x7FFFFFFF)
    al, bl = A & U(0xFFFFFFFF), B & U(0xFFFFFFFF)
    sw = (ah < bh) | ((ah == bh) & (al < bl))
    X, Y = np.where(sw, B, A), np.where(sw, A, B)
    ex = ((X >> U(52)) & U(0x7FF)).astype(np.int64)
    ey = ((Y >> U(52)) & U(0x7FF)).astype(np.int64)
    ok_in = (ex >= 1) & (ex <= 2046) & (ey >= 1) & (ey <= 2046)
    dd = ex - ey
    frac, hid = U(0xFFFFFFFFFFFFF), U(1 << 52)
    Mx = ((X & frac) | hid) << U(10)
    My0 = ((Y & frac) | hid) << U(10)
    ds = np.minimum(dd, 63).astype(U)
    My = My0 >> ds
    lost = np.where(ds == 0, U(0), My0 << ((U(64) - ds) & U(63)))
    stk_in = np.where(ds == 0, U(0), (lost != 0).astype(U))
    sub = ((X ^ Y) >> U(63)) != 0
    Sa = Mx + My
    ca = (Sa >> U(63))
    Sa_n = (Sa >> ca) | (Sa & ca)
    Ss = Mx - My - stk_in
    lz = np.where(Ss != 0, clz64(Ss) - 1, 0)
    S = np.where(sub, Ss << np.maximum(lz, 0).astype(U), Sa_n)
    E = ex + np.where(sub, -lz, ca.astype(np.int64))
    mant0 = S >> U(10)
    rnd = (S >> U(9)) & U(1)
    stk = stk_in | ((S & U(0x1FF)) != 0).astype(U)
    mant = mant0 + (rnd & (stk | (mant0 & U(1))))
    ok = ok_in & (dd <= 60) & ~(sub & (Ss == 0) & (stk_in == 0)) & (E >= 1) & (E <= 2045)
    bits = (X & U(1 << 63)) | (((E - 1).astype(U) << U(52)) + mant)
    return bits.view(np.float64), ok


def mul_restated(a, b):
    A, B = a.view(U), b.view(U)
    ahw, bhw = A >> U(32), B >> U(32)
    ea = ((ahw >> U(20)) & U(0x7FF)).astype(np.int64)
    eb = ((bhw >> U(20)) & U(0x7FF)).astype(np.int64)
    ah, bh = (ahw & U(0xFFFFF)) | U(0x100000), (bhw & U(0xFFFFF)) | U(0x100000)
    al, bl = A & U(0xFFFFFFFF), B & U(0xFFFFFFFF)
    p0, p1, p2, p3 = al * bl, ah * bl, al * bh, ah * bh
    mid = p1 + p2 + (p0 >> U(32))
    hi = (p3 << U(22)) + (mid >> U(10))
    low_nz = ((mid & U(0x3FF)) | (p0 & U(0xFFFFFFFF))) != 0
    top = hi >> U(63)
    sh = U(10) + top
    mant = hi >> sh
    rnd = (hi >> (sh - U(1))) & U(1)
    stk = low_nz | ((hi & ((U(1) << (sh - U(1))) - U(1))) != 0)
    mant = mant + (rnd & (stk.astype(U) | (mant & U(1))))
    E = ea + eb - 1023 + top.astype(np.int64)
    ok = (ea >= 1) & (ea <= 2046) & (eb >= 1) & (eb <= 2046) & (E >= 1) & (E <= 2045)
    bits = ((A ^ B) & U(1 << 63)) | (((E - 1).astype(U) << U(52)) + mant)
    return bits.view(np.float64), ok


def operands(n, seed):
    rng = np.random.default_rng(seed)
    m = rng.integers(0, 2 ** 52, size=(2, n), dtype=U)
    kind = rng.integers(0, 10, size=n)
    m[1] = np.where(kind == 1, m[0], m[1])
    m[1] = np.where(kind == 2, (m[0] + U(1)) & U(2 ** 52 - 1), m[1])
    m[0] = np.where(kind == 3, U(2 ** 52 - 1), m[0])
    m[1] = np.where(kind == 4, U(0), m[1])
    e = 1023 + rng.integers(-30, 31, size=(2, n))
    e[1] = np.where(kind == 5, e[0], e[1])                   # equal exponents: cancellation
    e[1] = np.where(kind == 6, e[0] - 1, e[1])
    s = rng.integers(0, 2, size=(2, n)).astype(U) << U(63)
    x = (s | (e.astype(U) << U(52)) | m).view(np.float64)
    return x[0].copy(), x[1].copy()


def same_bits(x, y):
    return x.view(U) == y.view(U)


def test_add_restated_is_ieee():
    a, b = operands(1_000_000, 11)
    with np.errstate(over="ignore"):
        got, ok = add_restated(a, b)
    want = a + b
    assert ok.mean() > 0.9
    bad = ok & ~same_bits(got, want)
    assert not bad.any(), (a[bad][:3], b[bad][:3])


def test_add_restated_near_cancellation():
    a, _ = operands(200_000, 12)
    rng = np.random.default_rng(13)
    b = -a * (1.0 + 2.0 ** -52 * rng.integers(-3, 4, size=a.size))
    got, ok = add_restated(a, b)
    bad = ok & ~same_bits(got, a + b)
    assert not bad.any()


def test_mul_restated_is_ieee():
    a, b = operands(1_000_000, 14)
    with np.errstate(over="ignore"):
        got, ok = mul_restated(a, b)
    want = a * b
    assert ok.mean() > 0.9
    bad = ok & ~same_bits(got, want)
    assert not bad.any(), (a[bad][:3], b[bad][:3])
