"""The algebra of the KG_F64_MIX forms (kernelgen-perf-tests_gb300/csrc/kg_mix.cu),
checked in numpy.

wave13pt's update (wave13pt/wave13pt.c:640-651)
    w2 = m0 w1 - w0 + m1 (six neighbours at distance 1) + m2 (six at distance 2)
is evaluated as (m0 + 6 m1 + 6 m2) c - w0 + m1 D1 + m2 D2 with c = w1[i] and D1, D2
the sums of the neighbour differences from c; uxx1's density sum
((d0 + d1) + d2) + d3 as (d0 + d1) + (d2 + d3), the second pair being the
previous plane's first.  Both are the same values in exact arithmetic: in FP64
they agree to rounding, and with the differences rounded to FP32 (as the
kernel forms them) the error stays at FP32's relative error of the small part.
"""
import numpy as np


def shifted(a, d, axis):
    return np.roll(a, -d, axis=axis)


def interior(a, r):
    return a[r:-r, r:-r, r:-r]


def wave_reference(w0, w1, m0, m1, m2):
    s1 = sum(shifted(w1, d, ax) for ax in (2, 1, 0) for d in (1, -1))
    s2 = sum(shifted(w1, d, ax) for ax in (2, 1, 0) for d in (2, -2))
    return m0 * w1 - w0 + m1 * s1 + m2 * s2


def wave_rewritten(w0, w1, m0, m1, m2, diff_dtype=np.float64):
    c = w1
    d1 = sum((shifted(w1, d, ax) - c).astype(diff_dtype) for ax in (2, 1, 0) for d in (1, -1))
    d2 = sum((shifted(w1, d, ax) - c).astype(diff_dtype) for ax in (2, 1, 0) for d in (2, -2))
    inc = (diff_dtype(m1) * d1 + diff_dtype(m2) * d2).astype(np.float64)
    return (m0 + 6 * m1 + 6 * m2) * c - w0 + inc


def pulse(n, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    r2 = (x - n / 2) ** 2 + (y - n / 2) ** 2 + (z - n / 2) ** 2
    return np.exp(-r2 / (2 * 4.0 ** 2)) + 1e-3 * rng.uniform(-1, 1, size=r2.shape)


def test_wave13pt_rewrite_is_the_same_update():
    rng = np.random.default_rng(1)
    w0, w1 = rng.uniform(-1, 1, size=(2, 24, 20, 28))
    m0, m1, m2 = rng.uniform(-1, 1, size=3)
    ref = interior(wave_reference(w0, w1, m0, m1, m2), 2)
    new = interior(wave_rewritten(w0, w1, m0, m1, m2), 2)
    assert np.max(np.abs(new - ref)) <= 1e-14 * np.max(np.abs(ref))


def test_wave13pt_fp32_differences_keep_the_state_precise():
    """On a smooth field (the precision workload's pulse) the FP32 part is small,
    so one step stays within ~1e-9 of FP64, far below FP32 storage's rounding."""
    w1 = pulse(32, 2)
    w0 = pulse(32, 3)
    c = 0.4
    m0, m1, m2 = 2 - 7.5 * c * c, 4 * c * c / 3, -c * c / 12
    ref = interior(wave_reference(w0, w1, m0, m1, m2), 2)
    mixed = interior(wave_rewritten(w0, w1, m0, m1, m2, np.float32), 2)
    f32 = interior(wave_reference(w0.astype(np.float32), w1.astype(np.float32), np.float32(m0), np.float32(m1),
                                  np.float32(m2)).astype(np.float64), 2)
    err_mixed = np.max(np.abs(mixed - ref)) / np.max(np.abs(ref))
    err_f32 = np.max(np.abs(f32 - ref)) / np.max(np.abs(ref))
    assert err_mixed < 1e-8 and err_mixed < err_f32 / 10, (err_mixed, err_f32)


def test_uxx1_density_pairs_are_the_same_sum():
    rng = np.random.default_rng(4)
    d = rng.uniform(0.5, 1.5, size=(4, 100000))
    ref = ((d[0] + d[1]) + d[2]) + d[3]
    new = (d[0] + d[1]) + (d[2] + d[3])
    assert np.max(np.abs(new - ref) / np.abs(ref)) <= 4 * 2.0 ** -53
