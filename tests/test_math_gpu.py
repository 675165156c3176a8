"""The trace's arithmetic helpers on the GPU against their stated bounds
(mx_math_check in include/marx_gb300.h): the Newton-Raphson reciprocal,
the double-float sin(pi y)/cos(pi y), the integer-pipe double-to-float
conversions, the float-rounded sine of the dither offsets and the
double-float Fresnel reflectivity.  The exact values come from Python's
rational arithmetic and numpy's long double."""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(fn, x):
    import torch
    from marx_gb300._native import load_library
    L = load_library()
    L.mx_math_check.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_size_t]
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    n = x.size // 3 if fn == 5 else x.size
    yd = torch.empty(n * {1: 2, 5: 4}.get(fn, 1), dtype=torch.float64, device="cuda")
    assert L.mx_math_check(fn, xd.data_ptr(), yd.data_ptr(), n) == 0
    return yd.cpu().numpy()


def _magnitudes(rng, n):
    m = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-140, 140, n).astype(np.float64))
    return m * rng.choice([-1.0, 1.0], n)


def test_reciprocal_within_one_ulp(cuda):
    rng = np.random.default_rng(11)
    edges = np.array([2.0 ** -125, 2.0 ** 125 * (1 - 2 ** -53), 2.0 ** 125, 2.0 ** -126, 1.0, -1.0, 3.0, 0.1,
                      1.0 + 2 ** -52, 2.0 - 2 ** -52, 5e-324, 1e308, -7.5e-200])
    x = np.concatenate([edges, _magnitudes(rng, 4000), rng.uniform(-1e4, 1e4, 2000)])
    y = _run(0, x)
    for xi, yi in zip(x, y):
        if not np.isfinite(yi):
            assert abs(xi) < 2.0 ** -1022, (xi, yi)    # 1 / a subnormal overflows, as the division does
            continue
        exact = 1 / Fraction(float(xi))
        assert abs(Fraction(float(yi)) - exact) <= Fraction(float(np.spacing(abs(float(exact))))), (xi, yi)
    # outside the fast range the division decides: the correctly rounded quotient
    out = np.abs(x) >= 2.0 ** 125
    assert np.array_equal(y[out], 1.0 / x[out])
    for v in (0.0, -0.0, np.inf, -np.inf):
        r = _run(0, np.array([v]))[0]
        with np.errstate(divide="ignore"):
            q = np.float64(1.0) / np.float64(v)
        assert r == q and np.signbit(r) == np.signbit(q)
    assert np.isnan(_run(0, np.array([np.nan]))[0])


def test_sincospi_within_two_to_minus_44(cuda):
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.uniform(-4.0, 4.0, 20000), np.arange(-16, 17) / 8.0, rng.uniform(-1e-8, 1e-8, 100)])
    y = _run(1, x).reshape(-1, 2)
    pi = np.longdouble("3.14159265358979323846264338327950288")
    arg = pi * x.astype(np.longdouble)
    ds = np.abs(y[:, 0].astype(np.longdouble) - np.sin(arg))
    dc = np.abs(y[:, 1].astype(np.longdouble) - np.cos(arg))
    assert float(max(ds.max(), dc.max())) <= 2.0 ** -44
    # exact at multiples of a quarter turn where the value is 0 or +-1
    k = np.arange(-16, 17)
    yk = _run(1, k / 2.0).reshape(-1, 2)
    assert np.array_equal(np.abs(yk[:, 0]) + np.abs(yk[:, 1]), np.ones(k.size))


def test_double_to_float_conversions_on_the_integer_pipe(cuda):
    rng = np.random.default_rng(13)
    x = np.concatenate([_magnitudes(rng, 20000), rng.uniform(-1e3, 1e3, 5000)])
    # ties: halfway between neighbouring floats, both parities
    f = rng.uniform(1, 2, 200).astype(np.float32)
    x = np.concatenate([x, (f.astype(np.float64) + np.nextafter(f, np.float32(3)).astype(np.float64)) / 2,
                        [2.0 ** -126, 2.0 ** -127, 2.0 ** 127, 2.0 ** 128, 3.5e38, 1e-46, 0.0, -0.0]])
    with np.errstate(over="ignore"):
        want = x.astype(np.float32).astype(np.float64)
    got = _run(2, x)
    assert np.array_equal(got, want) and np.array_equal(np.signbit(got), np.signbit(want))
    # truncation toward zero: within one float ulp below |x|, never above
    t = _run(4, x)
    normal = (np.abs(x) >= 2.0 ** -126) & (np.abs(x) < 2.0 ** 127)
    a, b = np.abs(t[normal]), np.abs(x[normal])
    assert np.all(a <= b) and np.all(b - a < np.spacing(a.astype(np.float32)).astype(np.float64))


def test_sine_rounds_to_the_float_of_the_double_sine(cuda):
    rng = np.random.default_rng(14)
    x = np.concatenate([rng.uniform(-10.0, 10.0, 50000), rng.uniform(-1e-5, 1e-5, 5000),
                        rng.uniform(-3e5, 3e5, 500)])
    got = _run(3, x).astype(np.float32)
    want = np.sin(x.astype(np.longdouble)).astype(np.float32)
    bad = np.flatnonzero(got != want)
    # a value within a few double ulps of a float rounding boundary may go
    # either way between two libraries' double sines; nothing else may differ
    assert bad.size <= 2, bad[:10]
    for i in bad:
        assert abs(int(got[i].view(np.int32)) - int(want[i].view(np.int32))) == 1


def _fresnel_parts(c, b, d):
    """reflectivity_parts (Fresnel numerator and denominator) evaluated
    in numpy's long double."""
    one = np.longdouble(1)
    nr, ni = one - d, b
    sr, si = nr * nr - ni * ni, 2 * nr * ni
    # n^2 - sin^2 without cancelling two numbers near 1
    wr, wi = c * c - (d * (2 - d) + b * b), si
    r = np.sqrt(wr * wr + wi * wi)
    h = (r + np.abs(wr)) / 2
    inv = one / np.sqrt(h)
    pos = wr >= 0
    rr = np.where(pos, h * inv, wi * inv / 2)
    ri = np.where(pos, wi * inv / 2, h * inv)
    a1, b1 = (c - rr) ** 2 + ri ** 2, (c + rr) ** 2 + ri ** 2
    pr, pi = c * sr, c * si
    a2, b2 = (pr - rr) ** 2 + (pi - ri) ** 2, (pr + rr) ** 2 + (pi + ri) ** 2
    return (a1 * b2 + a2 * b1) / 2, b1 * b2


def test_double_float_reflectivity(cuda):
    """The Fresnel numerator and denominator in double-float (the
    reflectivity test's screen, the weighted rays' weights) against the
    same algebra in long double and against the double-precision
    evaluation: grazing angles of 0.05-3 degrees (a quarter within 10% of
    the critical angle) and log-uniform beta 1e-9..1e-2, delta 1e-7..1e-2.
    The double-float values are within 2^-30 of the long-double ones (the
    numerator of a reflectivity near 1e-7, far above the critical angle,
    cancels in cos - root as it does in double precision; typically they
    are within 2^-42); the double-precision ones lose up to about 2^-28 near
    the critical angle at the smallest delta (n^2 - sin^2 cancels there).
    The two stay within 2^-26 of each other, four times inside the 2^-24
    band in which the reflectivity test leaves its decision to the double
    values."""
    rng = np.random.default_rng(15)
    n = 200000
    cos = np.sin(np.radians(rng.uniform(0.05, 3.0, n)))
    beta = np.exp(rng.uniform(np.log(1e-9), np.log(1e-2), n)).astype(np.float32).astype(np.float64)
    delta = np.exp(rng.uniform(np.log(1e-7), np.log(1e-2), n)).astype(np.float32).astype(np.float64)
    m = n // 4
    cos[:m] = np.sqrt(delta[:m] * (2 - delta[:m]) + beta[:m] ** 2) * rng.uniform(0.9, 1.1, m)
    x = np.stack([cos, beta, delta], axis=1).ravel()
    y = _run(5, x).reshape(n, 4)
    num_df, den_df, num, den = y.T
    assert np.all(den > 0) and np.all(num > 0)
    en, ed = _fresnel_parts(cos.astype(np.longdouble), beta.astype(np.longdouble), delta.astype(np.longdouble))

    def rel(a, b):
        return np.abs(a.astype(np.longdouble) - b) / b

    e = np.maximum(rel(num_df, en), rel(den_df, ed))
    assert float(e.max()) <= 2.0 ** -30 and float(np.median(e)) <= 2.0 ** -42
    assert float(max(rel(num_df, num.astype(np.longdouble)).max(), rel(den_df, den.astype(np.longdouble)).max())) <= 2.0 ** -26


def test_integer_pipe_truncations_and_fast_root(cuda):
    """(double) (unsigned) x and (unsigned) (4 x) built from the bits of x,
    exactly the casts; sqrt from the reciprocal square root within two
    ulps of the correctly rounded root."""
    rng = np.random.default_rng(16)
    x = np.concatenate([rng.uniform(0, 4.29e9, 20000), rng.uniform(0, 2, 5000), np.arange(0, 70) / 3.0,
                        [0.0, 0.999999, 1.0, 2.0 ** 31, 2.0 ** 32 - 1.0, 4294967295.5, 1e-300]])
    assert np.array_equal(_run(6, x), np.floor(x))
    u = np.concatenate([rng.uniform(0, 1, 20000), [0.0, 0.25, 0.5, 0.75, np.nextafter(0.25, 0), np.nextafter(1.0, 0),
                                                   1e-300, 5e-324]])
    assert np.array_equal(_run(8, u), np.floor(4 * u))
    r = np.concatenate([np.exp(rng.uniform(-700, 700, 20000)), rng.uniform(0, 1e6, 5000)])
    got = _run(7, r)
    want = np.sqrt(r)
    assert np.all(np.abs(got - want) <= 2 * np.spacing(want))
    edge = np.array([0.0, -0.0, np.inf, 5e-324, 1e-310])
    assert np.array_equal(_run(7, edge), np.sqrt(edge))
