"""FP64-accurate dense contractions on the bf16 tensor cores (error-free digit
splitting) against the FP64-pipe kernels and exact rational arithmetic."""
from fractions import Fraction

import numpy as np
import pytest

import gcge_gb300 as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def gram(ctx, V, W, sym=False, tc=True):
    ctx.tensor_emulation(tc)
    try:
        n, k1 = V.shape
        k2 = W.shape[1]
        v, w = ctx.multivec(n, k1, V), ctx.multivec(n, k2, W)
        a = G.multivec_inner_prod(v, w, (0, 0), (k1, k2), k1, sym=sym)
        return a.reshape(k2, k1).T
    finally:
        ctx.tensor_emulation(True)


def exact_dot(x, y):
    return float(sum((Fraction(a) * Fraction(b) for a, b in zip(x, y)), Fraction(0)))


@pytest.mark.parametrize("n,k1,k2", [(100003, 37, 21), (857375 // 8, 108, 50), (5000, 64, 64), (77, 3, 5)])
def test_tensor_gram_matches_fp64_pipe(ctx, n, k1, k2):
    rng = np.random.default_rng(n + k1)
    V = rng.standard_normal((n, k1))
    W = rng.standard_normal((n, k2))
    a_tc = gram(ctx, V, W, tc=True)
    a_64 = gram(ctx, V, W, tc=False)
    scale = np.outer(np.linalg.norm(V, axis=0), np.linalg.norm(W, axis=0))
    assert np.max(np.abs(a_tc - a_64) / scale) < 1e-14
    # a few entries against exact rational arithmetic: both within FP64 rounding
    for (i, j) in [(0, 0), (k1 - 1, k2 - 1), (k1 // 2, 0)]:
        if n > 20000:
            idx = np.arange(0, n, 7)[:3000]
            ex = exact_dot(V[idx, i], W[idx, j])
            sub = gram(ctx, V[idx][:, [i]], W[idx][:, [j]], tc=True)[0, 0]
            assert abs(sub - ex) <= 1e-15 * np.linalg.norm(V[idx, i]) * np.linalg.norm(W[idx, j])
        else:
            ex = exact_dot(V[:, i], W[:, j])
            assert abs(a_tc[i, j] - ex) <= 1e-15 * scale[i, j]


def test_tensor_gram_exact_on_integers(ctx):
    """Small integers have short expansions: the digit products are exact and so is the sum."""
    rng = np.random.default_rng(3)
    n = 40000
    V = rng.integers(-1000, 1000, size=(n, 9)).astype(np.float64)
    W = rng.integers(-1000, 1000, size=(n, 7)).astype(np.float64)
    assert np.array_equal(gram(ctx, V, W, tc=True), V.T @ W)


def test_tensor_gram_wide_dynamic_range(ctx):
    """Entries spanning 2^-40 .. 1 inside a column: error bounded by the column scale."""
    rng = np.random.default_rng(4)
    n = 30000
    V = rng.standard_normal((n, 6)) * np.exp2(-40 * rng.random((n, 6)))
    W = rng.standard_normal((n, 5)) * np.exp2(-40 * rng.random((n, 5)))
    a_tc = gram(ctx, V, W, tc=True)
    for i in range(6):
        for j in range(5):
            ex = exact_dot(V[:, i], W[:, j])
            bound = n * 2.0 ** -55 * np.max(np.abs(V[:, i])) * np.max(np.abs(W[:, j])) + 4e-16 * np.abs(V[:, i]) @ np.abs(W[:, j])
            assert abs(a_tc[i, j] - ex) <= bound


def test_tensor_gram_symmetric(ctx):
    rng = np.random.default_rng(5)
    V = rng.standard_normal((50000, 70))
    a = gram(ctx, V, V, sym=True, tc=True)
    assert np.array_equal(a, a.T)
    ref = V.T @ V
    assert np.max(np.abs(a - ref)) / np.max(np.abs(ref)) < 1e-14


def lincomb(ctx, X, C, tc=True):
    ctx.tensor_emulation(tc)
    try:
        n, k1 = X.shape
        k2 = C.shape[1]
        x, y = ctx.multivec(n, k1, X), ctx.multivec(n, k2 + 1, np.full((n, k2 + 1), 3.0))
        G.multivec_linear_comb(x, y, (0, 1), (k1, 1 + k2), np.asfortranarray(C).ravel(order="F"), k1)
        out = y.download()
        assert np.all(out[:, 0] == 3.0)           # the column outside the range is untouched
        return out[:, 1:]
    finally:
        ctx.tensor_emulation(True)


def oz_lincomb_bound(X, C):
    """Elementwise error guarantee of the split product: with g_i the exponent of
    row i of C, Xt = X 2^g and Ct = 2^-g C are split against their row and column
    maxima (rounding below 2^-53 of the maximum each) and the dropped digit
    levels add less than 2^-54 of maxX*maxC per term."""
    g = np.frexp(np.max(np.abs(C), axis=1))[1].astype(np.float64)
    Xt, Ct = X * np.exp2(g), C * np.exp2(-g)[:, None]
    mx, mc = np.max(np.abs(Xt), axis=1), np.max(np.abs(Ct), axis=0)
    k1 = X.shape[1]
    return 2.0 ** -53 * (mx[:, None] * np.sum(np.abs(Ct), axis=0)[None, :] +
                         np.sum(np.abs(Xt), axis=1)[:, None] * mc[None, :]) + \
        2.0 ** -54 * k1 * mx[:, None] * mc[None, :]


@pytest.mark.parametrize("n,k1,k2", [(1000, 37, 21), (100003, 178, 50), (5000, 64, 64), (20000, 100, 130),
                                     (77, 3, 5), (300, 1, 1), (4099, 129, 17)])
def test_tensor_lincomb_matches_fp64_pipe(ctx, n, k1, k2):
    rng = np.random.default_rng(n * 7 + k1)
    X = rng.standard_normal((n, k1)) * np.exp2(rng.integers(-8, 8, size=(n, 1)))
    C = rng.standard_normal((k1, k2))
    y_tc = lincomb(ctx, X, C, tc=True)
    y_64 = lincomb(ctx, X, C, tc=False)
    scale = np.abs(X) @ np.abs(C)
    assert np.max(np.abs(y_tc - y_64) / scale) < 1e-14
    bound = oz_lincomb_bound(X, C)
    for r in (0, n // 2, n - 1):
        for j in (0, k2 - 1):
            ex = exact_dot(X[r], C[:, j])
            assert abs(y_tc[r, j] - ex) <= 2.0 ** -52 * abs(ex) + bound[r, j]


def test_tensor_lincomb_exact_on_integers(ctx):
    rng = np.random.default_rng(8)
    X = rng.integers(-1000, 1000, size=(3000, 140)).astype(np.float64)
    C = rng.integers(-1000, 1000, size=(140, 40)).astype(np.float64)
    assert np.array_equal(lincomb(ctx, X, C), X @ C)


def test_tensor_lincomb_wide_dynamic_range(ctx):
    """Row entries spanning 2^-40 .. 1: errors bounded by the row and column scales."""
    rng = np.random.default_rng(9)
    X = rng.standard_normal((2000, 45)) * np.exp2(-40 * rng.random((2000, 45)))
    C = rng.standard_normal((45, 9)) * np.exp2(-30 * rng.random((45, 9)))
    y = lincomb(ctx, X, C)
    for r in range(0, 2000, 97):
        for j in range(9):
            ex = exact_dot(X[r], C[:, j])
            bound = 45 * 2.0 ** -53 * np.max(np.abs(X[r])) * np.max(np.abs(C[:, j])) + 2.0 ** -52 * abs(ex)
            assert abs(y[r, j] - ex) <= bound


def test_tensor_lincomb_zero_rows_and_columns(ctx):
    rng = np.random.default_rng(10)
    X = rng.standard_normal((700, 20))
    X[5] = 0.0
    X[:, 3] = 0.0
    C = rng.standard_normal((20, 6))
    C[:, 2] = 0.0
    y = lincomb(ctx, X, C)
    assert np.all(y[5] == 0.0) and np.all(y[:, 2] == 0.0)
    np.testing.assert_allclose(y, X @ C, rtol=0, atol=1e-13 * np.max(np.abs(X) @ np.abs(C)))


def test_tensor_lincomb_compensating_scales(ctx):
    """Columns of X spanning 2^-30 .. 1 with C scaling them back up (the W R^-1 of a
    Cholesky QR after projection): the inner dimension is equilibrated, so errors
    stay at FP64 level normwise and within the split's guarantee elementwise."""
    rng = np.random.default_rng(11)
    n, k1, k2 = 5000, 40, 40
    colscale = np.exp2(-30 * rng.random(k1))
    X = rng.standard_normal((n, k1)) * colscale
    C = np.triu(rng.standard_normal((k1, k2))) / colscale[:, None]
    y_tc = lincomb(ctx, X, C, tc=True)
    y_64 = lincomb(ctx, X, C, tc=False)
    scale = np.abs(X) @ np.abs(C)
    col_err = np.linalg.norm(y_tc - y_64, axis=0) / np.linalg.norm(scale, axis=0)
    assert np.max(col_err) < 1e-14
    bound = oz_lincomb_bound(X, C)
    for r in (0, 1234, n - 1):
        for j in (0, 17, k2 - 1):
            ex = exact_dot(X[r], C[:, j])
            assert abs(y_tc[r, j] - ex) <= 2.0 ** -52 * abs(ex) + bound[r, j]


@pytest.mark.parametrize("pattern", ["same_sign", "cancelling"])
def test_tensor_gram_at_full_size_against_exact(ctx, pattern):
    """Adversarial Gram at the 160^3 size (n = 4,096,000) with an exact answer.
    Constant columns make every row drop the same digit pairs, so the dropped mass
    adds up coherently over all n rows (the worst case of the splitting): V[:, i] =
    c_i, W[:, j] = d_j on every row (same sign) or d_j on even rows and -d'_j =
    -fl(d_j (1 + 2^-20)) on odd rows (a 2^20-fold cancellation). The entries carry
    full 53-bit significands, so every digit level is populated. Bound: one final
    rounding plus n 2^-57.4 2^(e+f) for the dropped pairs (levels >= 8)."""
    n, k1, k2 = 4096000, 128, 64
    rng = np.random.default_rng(41)
    c = rng.uniform(0.5, 1.0, k1) * 2.0 ** rng.integers(-3, 4, k1)
    d = rng.uniform(0.5, 1.0, k2) * 2.0 ** rng.integers(-3, 4, k2)
    V = np.broadcast_to(c, (n, k1))
    if pattern == "same_sign":
        W = np.broadcast_to(d, (n, k2))
        exact = [[Fraction(n) * Fraction(ci) * Fraction(dj) for dj in d] for ci in c]
    else:
        dp = d * (1.0 + 2.0 ** -20)
        W = np.empty((n, k2))
        W[0::2] = d
        W[1::2] = -dp
        exact = [[Fraction(n // 2) * Fraction(ci) * (Fraction(dj) - Fraction(dpj)) for dj, dpj in zip(d, dp)]
                 for ci in c]
    got = gram(ctx, np.ascontiguousarray(V), W)
    e = np.frexp(c)[1]                                   # column scales: |x| < 2^e
    f = np.frexp(np.max(np.abs(W[:2]), axis=0))[1]
    worst = 0.0
    for i in range(k1):
        for j in range(k2):
            ex = exact[i][j]
            err = float(abs(Fraction(got[i, j]) - ex))
            bound = float(abs(ex)) * 2.0 ** -52 + n * 2.0 ** (-57.4 + e[i] + f[j])
            assert err <= bound, (pattern, i, j, err, bound)
            worst = max(worst, err / float(abs(ex)))
    # far inside the FP64 summation error of the same Gram (same sign: ~n eps / nsplit relative)
    assert worst < (1e-15 if pattern == "same_sign" else 1e-10), worst
