"""Double-float arithmetic of the local solve's start (dd_math.cuh) on the GPU.

The start of every FP64 local Newton ends with one Halley step whose residual is
evaluated in double-float (pairs of FP32 numbers, about 48 significant bits).  These
tests bound the conversion from double, exp and log against 40-digit decimal
arithmetic: the conversion keeps 47 bits, exp is within 2^-45 relative, log within
2^-46 of (|log s| + 1) absolute.
"""
from decimal import Decimal, getcontext

import numpy as np
import pytest

import mdz_rheo as R

pytestmark = pytest.mark.gpu

getcontext().prec = 40


def exact(pair):
    return Decimal(float(pair[0])) + Decimal(float(pair[1]))


def test_conversion_keeps_47_bits():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-10, 10, 4000), np.exp(rng.uniform(-150, 80, 4000)),
                        -np.exp(rng.uniform(-50, 50, 2000)), [1.0, -2.5, 3.5, 2.3, 0.1, 1e-20]])
    a, _, _ = R.dd_selftest(x)
    worst = 0.0
    for xi, p in zip(x, a):
        if abs(xi) < 2.0 ** -74:
            continue
        err = abs(exact(p) - Decimal(float(xi))) / abs(Decimal(float(xi)))
        worst = max(worst, float(err))
        assert abs(p[1]) <= abs(p[0]) * 2.0 ** -23
    assert worst <= 2.0 ** -47, worst


def test_exp_relative_error():
    rng = np.random.default_rng(2)
    # below about -60 the low word becomes subnormal and the relative accuracy degrades
    # (there exp(x) < 1e-26, nothing next to the O(1) terms of the residual)
    x = np.concatenate([rng.uniform(-60, 5, 6000), rng.uniform(-1e-3, 1e-3, 2000), rng.uniform(-8, 0, 6000),
                        [0.0, -0.0, 1.0, -1.0, 1e-30, np.log(2.0), -np.log(2.0) / 512]])
    a, e, _ = R.dd_selftest(x)
    worst = 0.0
    for p, q in zip(a, e):
        ref = exact(p).exp()          # exp of the double-float argument the kernel received
        err = abs(exact(q) - ref) / ref
        worst = max(worst, float(err))
    print("dd exp worst relative error", worst)
    assert worst <= 2.0 ** -45, worst
    # far below the range: 0; between -79 and -60 within 1e-40 absolute
    _, e, _ = R.dd_selftest(np.array([-90.0, -200.0]))
    assert np.all(e == 0.0)
    x = rng.uniform(-79, -60, 500)
    a, e, _ = R.dd_selftest(x)
    assert max(float(abs(exact(q) - exact(p).exp())) for p, q in zip(a, e)) < 1e-40


def test_log_absolute_error():
    rng = np.random.default_rng(3)
    s = np.concatenate([rng.uniform(0.2, 2.0, 8000), np.exp(rng.uniform(-80, 80, 4000)),
                        [1.0, 0.75, 1.5, 0.999999, 1.000001, 2.0, 0.25]]).astype(np.float32).astype(np.float64)
    _, _, l = R.dd_selftest(s)
    worst = 0.0
    for si, p in zip(s, l):
        ref = Decimal(float(si)).ln()
        err = abs(exact(p) - ref) / (abs(ref) + 1)
        worst = max(worst, float(err))
    print("dd log worst error / (|log| + 1)", worst)
    assert worst <= 2.0 ** -46, worst
