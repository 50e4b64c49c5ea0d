"""The double-double arithmetic behind the finite-difference gradient check,
against exact rational arithmetic (fractions.Fraction) on small cases."""
from fractions import Fraction as F

import numpy as np
import pytest

import pyoracle
from gcge_gb300 import problems as P


@pytest.fixture(scope="module")
def oracle():
    return pyoracle.Oracle()


def exact_vec(xh, xl):
    return [F(a) + F(b) for a, b in zip(xh, xl)]


def test_dd_rayleigh_residual_and_weighted_sums_are_exact_to_double_double(oracle):
    A, _ = P.varcoef2d(nc=12, seed=3, sigma=0.5)
    n = A.n
    rng = np.random.default_rng(5)
    xh = rng.standard_normal(n)
    xl = rng.standard_normal(n) * 1e-17 * np.abs(xh)
    w = rng.uniform(0.0, 1.0, n)
    x = exact_vec(xh, xl)
    Ax = [sum((F(A.val[j]) * x[A.col[j]] for j in range(A.rowptr[i], A.rowptr[i + 1])), F(0)) for i in range(n)]
    xax = sum((a * b for a, b in zip(x, Ax)), F(0))
    xx = sum((a * a for a in x), F(0))
    q = xax / xx
    hi, lo = oracle.dd_rayleigh(A, xh, xl)
    assert abs(F(hi) + F(lo) - q) <= abs(q) * F(2) ** -100
    r = oracle.dd_residual(A, xh, xl, (hi, lo))
    th = F(hi) + F(lo)
    for i in range(n):
        exact = Ax[i] - th * x[i]
        assert abs(F(r[i]) - exact) <= abs(exact) * F(2) ** -52 + F(2) ** -1000
    s = oracle.dd_weighted_sq(w, xh, xl)
    sw = sum((F(wi) * a * a for wi, a in zip(w, x)), F(0))
    assert abs(F(s[0]) + F(s[1]) - sw) <= sw * F(2) ** -100
    assert abs(F(s[2]) + F(s[3]) - xx) <= xx * F(2) ** -100
    d = rng.standard_normal(n) * 1e-9
    yh, yl = xh.copy(), xl.copy()
    oracle.dd_add_vec(yh, yl, d)
    for i in range(n):
        exact = x[i] + F(d[i])
        assert abs(F(yh[i]) + F(yl[i]) - exact) <= abs(exact) * F(2) ** -104
