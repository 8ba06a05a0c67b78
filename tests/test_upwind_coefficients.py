"""The upwind-trace stage variant forms the face flux from the bitwise or
of the two upwind coefficients P = (c + |c|) / 2 and M = (c - |c|) / 2 of a
face point (stage_gauss.cuh, `or_bits`): with flux_alpha 1 one of them is
+0.0 in IEEE arithmetic, so the or is exactly the nonzero one, c itself.
The geometry builder forms them as 0.5 * (c +- alpha * |c|) in binary64
(geometry.cpp); the binary32 copies are the roundings of those."""
import numpy as np


def _coefficients(c, alpha=1.0):
    c = np.asarray(c, dtype=np.float64)
    return 0.5 * (c + alpha * np.abs(c)), 0.5 * (c - alpha * np.abs(c))


def _or_bits(a, b, itype):
    return (a.view(itype) | b.view(itype)).view(a.dtype)


def test_one_coefficient_is_positive_zero():
    rng = np.random.default_rng(7)
    c = np.concatenate([rng.standard_normal(100000) * 10.0 ** rng.integers(-30, 30, 100000),
                        [1e-310, -1e-310, 5e-324, -5e-324, 1e300, -1e300]])
    p, m = _coefficients(c)
    zero_p, zero_m = p == 0.0, m == 0.0
    assert np.all(zero_p | zero_m)
    # the zero one is +0.0 (no sign bit)
    assert not np.any(np.signbit(p[zero_p])) and not np.any(np.signbit(m[zero_m]))
    for dtype, itype in ((np.float64, np.int64), (np.float32, np.int32)):
        with np.errstate(over="ignore"):  # binary32 roundings of |c| > 3.4e38 are infinite
            pp, mm, cc = p.astype(dtype), m.astype(dtype), c.astype(dtype)
        merged = _or_bits(pp, mm, itype)
        assert np.array_equal(merged, np.where(c > 0, pp, mm))
        assert np.array_equal(merged, cc)


def test_zero_normal_speed_gives_no_upwind_side():
    p, m = _coefficients([0.0, -0.0])
    # both coefficients vanish: the face point reads no trace and its flux is zero
    assert np.all(p == 0.0) and np.all(m == 0.0)
