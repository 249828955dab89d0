"""Accuracy of the table-driven FP64 exp and log of the hot path (P. T. P. Tang's
methods, csrc/fp64_math.cuh) against CUDA's exp/log on the same GPU and against
numpy (glibc), over the argument ranges the rheology reaches and the special values."""
import numpy as np
import pytest

import mdz_rheo as R

pytestmark = pytest.mark.gpu


def ulps(a, b):
    """|a - b| in units of the last place of b (float64)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    sp = np.spacing(np.abs(b))
    return np.where(a == b, 0.0, np.abs(a - b) / sp)


def test_exp_accuracy():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-700, 700, 400_000), rng.uniform(-1, 1, 200_000),
                        rng.uniform(-1e-8, 1e-8, 50_000), np.linspace(-745, 709.7, 10_001),
                        [0.0, -0.0, 1e-300, -1e-300, 700.0, -700.0, 709.78, -745.2, 710.0, -746.0,
                         np.inf, -np.inf, np.nan]])
    fe, ce, _, _ = R.math_selftest(x)
    # the table path serves |x| < 700; everything else is CUDA's exp itself
    fast = np.isfinite(x) & (np.abs(x) < 700.0)
    u_cuda = ulps(fe[fast], ce[fast])
    u_np = ulps(fe[fast], np.exp(x[fast]))
    print("exp: max ulp vs CUDA", u_cuda.max(), "vs numpy", u_np.max(), "mean", u_np.mean())
    assert u_cuda.max() <= 2.0 and u_np.max() <= 2.0
    assert np.array_equal(fe[~fast], ce[~fast], equal_nan=True)


def test_log_accuracy():
    rng = np.random.default_rng(1)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 400_000), rng.uniform(0.5, 2.0, 200_000),
                        1.0 + rng.uniform(-1e-6, 1e-6, 50_000),
                        [1.0, 2.0, 0.5, 0.75, 1.5, 1e-310, 5e-324, 0.0, -0.0, -1.0, np.inf, np.nan,
                         np.finfo(np.float64).max, np.finfo(np.float64).tiny]])
    _, _, fl, cl = R.math_selftest(x)
    fin = np.isfinite(cl) & (cl != 0.0)
    # absolute error near log(1) = 0, relative elsewhere
    den = np.maximum(np.abs(cl[fin]), 1.0)
    err_cuda = np.abs(fl[fin] - cl[fin]) / (np.spacing(den))
    err_np = np.abs(fl[fin] - np.log(x[fin])) / (np.spacing(den))
    print("log: max error (ulps of max(|log|,1)) vs CUDA", err_cuda.max(), "vs numpy", err_np.max())
    assert err_cuda.max() <= 2.0 and err_np.max() <= 2.0
    assert fl[np.where(x == 1.0)[0][0]] == 0.0
    special = ~fin
    assert np.array_equal(fl[special], cl[special], equal_nan=True)


def _near_midpoints(rng, b, n):
    """Numerators whose quotient by b lies as close as binary64 allows to a midpoint
    between two doubles (the hardest cases for rounding), and their neighbours."""
    from fractions import Fraction
    q = rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-30, 30, n)
    out = []
    for v in q:
        mid = Fraction(float(v)) + Fraction(float(np.spacing(v))) / 2
        a = float(Fraction(b) * mid)
        out += [a, np.nextafter(a, np.inf), np.nextafter(a, -np.inf)]
    return np.array(out)


@pytest.mark.parametrize("b", [1e5 / 2049, 1e5 / 4097, 0.1, 1.0 / 3.0, 3.0, 7.0, 1.0, 0.5, 1024.0,
                               1.9999999999999998, 1.0000000000000002, 48.80429477794046, 2.0 ** -399,
                               2.0 ** 399, -6.25e-3, 1e-200])
def test_known_divisor_division_is_exact(b):
    """The division by a mesh spacing (csrc/fp64_div.cuh) against CUDA's division and
    numpy's: bit for bit on random numerators of every scale, near-midpoint quotients and
    the special values (which take CUDA's division itself)."""
    rng = np.random.default_rng(int(abs(b) * 1e6) % 2 ** 32)
    a = np.concatenate([rng.standard_normal(1_000_000) * 10.0 ** rng.uniform(-300, 300, 1_000_000),
                        rng.uniform(-1.0, 1.0, 200_000) * 1e-12,
                        _near_midpoints(rng, b, 5_000),
                        [0.0, -0.0, 5e-324, -5e-324, 2.0 ** -500, 2.0 ** 500, 2.0 ** -501, 2.0 ** 501,
                         1.7976931348623157e308, np.inf, -np.inf, np.nan]])
    fast, plain = R.div_selftest(a, b)
    with np.errstate(all="ignore"):
        host = a / b
    assert np.array_equal(fast.view(np.uint64)[~np.isnan(a)], plain.view(np.uint64)[~np.isnan(a)])
    assert np.array_equal(fast.view(np.uint64)[~np.isnan(a)], host.view(np.uint64)[~np.isnan(a)])
    assert np.isnan(fast[np.isnan(a)]).all()


def test_integer_pipe_ceil_matches_cuda():
    """The cell-index ceil read from the bits of a double (csrc/fp64_bits.cuh) against
    CUDA's ceil: equal on every argument below 2^30 in magnitude -- integers, their
    neighbours one ulp away, halves, signed zeros, subnormals, random values of every
    scale -- and saturated to +-2^30 beyond (NaN to +2^30)."""
    rng = np.random.default_rng(5)
    ints = np.arange(-5000.0, 5000.0)
    q = np.concatenate([ints, np.nextafter(ints, np.inf), np.nextafter(ints, -np.inf), ints + 0.5,
                        rng.uniform(-3e4, 3e4, 1_000_000),
                        rng.standard_normal(200_000) * 10.0 ** rng.uniform(-320, 12, 200_000),
                        [0.0, -0.0, 5e-324, -5e-324, 0.9999999999999999, -0.9999999999999999,
                         2.0 ** 30 - 0.5, -(2.0 ** 30) + 0.5, 2.0 ** 30, -(2.0 ** 30), 2.0 ** 52 + 1.0,
                         1e300, -1e300, np.inf, -np.inf, np.nan]])
    fast, plain = R.ceil_selftest(q)
    small = np.abs(q) < 2.0 ** 30
    assert np.array_equal(fast[small].astype(np.float64), plain[small])
    assert np.array_equal(plain[small], np.ceil(q[small]))
    big = ~small & ~np.isnan(q)
    assert np.array_equal(fast[big], np.where(q[big] < 0, -(2 ** 30), 2 ** 30))
    assert (fast[np.isnan(q)] == 2 ** 30).all()


def test_output_quotient_within_two_ulp():
    """The quotient of the local solve's outputs (csrc/fp64_div.cuh `quotient`: two Newton
    steps on the hardware reciprocal estimate, then one product) against IEEE division:
    within 2 ulp of the correctly rounded quotient for operands of every scale and sign,
    and equal to it where the divisor lies outside [2^-1000, 2^1000] (zero, subnormal,
    huge, Inf, NaN: the IEEE division itself)."""
    rng = np.random.default_rng(17)
    n = 2_000_000
    r = rng.standard_normal(n) * 10.0 ** rng.uniform(-150, 150, n)
    den = rng.standard_normal(n) * 10.0 ** rng.uniform(-290, 290, n)
    # mantissas near 1 and near 2, and exact powers of two
    den[:1000] = 2.0 ** rng.integers(-900, 900, 1000)
    den[1000:2000] = np.nextafter(2.0, 0.0) * 2.0 ** rng.integers(-900, 900, 1000)
    den[2000:3000] = np.nextafter(1.0, 2.0) * 2.0 ** rng.integers(-900, 900, 1000)
    r[:3000] = 1.0
    with np.errstate(all="ignore"):
        exact = r / den
    got = R.quotient_selftest(r, den)
    ok = np.isfinite(exact) & (exact != 0) & (np.abs(exact) > 1e-290) & (np.abs(exact) < 1e290)
    ulps = np.abs(got[ok] - exact[ok]) / np.spacing(np.abs(exact[ok]))
    print("output quotient: worst", float(ulps.max()), "ulp; mean", float(ulps.mean()))
    assert ulps.max() <= 2.0
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.0 ** -1001, 2.0 ** 1001, 1.7976931348623157e308,
                        np.inf, -np.inf, np.nan])
    rs = np.full(special.size, 3.0)
    with np.errstate(all="ignore"):
        want = rs / special
    got = R.quotient_selftest(rs, special)
    assert np.array_equal(got, want, equal_nan=True)
