"""FP32-pair sparse products (GCGE_GPU_SetPairSpMM, the outer products of a
precision-2 solve) through the C ABI.

Accuracy is checked against the product accumulated in numpy's longdouble
(64-bit significand on x86, 113 on aarch64): every entry within 2^-40 of
sum_j |a_ij x_j| and the whole block within 1e-13 of || |A| |X| ||_F (the pair
form carries a 48-bit significand; FP64 gives ~1e-16). Values the pair range does
not cover (|x| >= 2^100, non-finite x, a matrix whose largest entry is beyond
2^700) must give exactly the FP64 product, which the kernel then computes.
"""
import numpy as np
import pytest

import gcge_gb300 as G
from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.pair_spmm(False)
    c.close()


def exact_product(A, X):
    """(A X in longdouble, |A| |X|) for a CSR matrix."""
    lens = np.diff(A.rowptr)
    nz = lens > 0
    starts = A.rowptr[:-1][nz]
    prod = A.val.astype(np.longdouble)[:, None] * X[A.col].astype(np.longdouble)
    out = np.zeros((A.n, X.shape[1]), dtype=np.longdouble)
    absb = np.zeros((A.n, X.shape[1]))
    if len(A.val):
        out[nz] = np.add.reduceat(prod, starts, axis=0)
        absb[nz] = np.add.reduceat(np.abs(A.val)[:, None] * np.abs(X[A.col]), starts, axis=0)
    return out, absb


def product(ctx, A, X, pair, scale=None):
    ctx.pair_spmm(pair)
    dA = ctx.matrix(A)
    k = X.shape[1]
    x = ctx.multivec(A.n, k, X)
    y = ctx.multivec(A.n, k)
    G.mat_dot_multivec(dA, x, y, (0, 0), (k, k))
    out = y.download()
    ctx.pair_spmm(False)
    return out


CASES = [
    ("fem_stiffness", lambda: P.fem_q1_cube(9)[0], 64),
    ("fem_mass", lambda: P.fem_q1_cube(9)[1], 56),
    ("fem_stiffness_7", lambda: P.fem_q1_cube(9)[0], 7),
    ("laplace2d", lambda: P.laplace2d(37, 23)[0], 2),
    ("powerlaw", lambda: P.powerlaw_graph(3000, seed=5, dmax=300)[0], 33),
    ("varcoef3d", lambda: P.varcoef3d(nc=12)[0], 100),
]


@pytest.mark.parametrize("name,maker,k", CASES, ids=[c[0] for c in CASES])
def test_pair_product_accuracy(ctx, name, maker, k):
    A = maker()
    rng = np.random.default_rng(7)
    # rows of very different magnitudes, a few exact zeros
    X = rng.standard_normal((A.n, k)) * 10.0 ** rng.uniform(-6, 6, (A.n, 1))
    X[rng.random((A.n, k)) < 0.01] = 0.0
    ex, absb = exact_product(A, X)
    got = product(ctx, A, X, True)
    err = np.abs(got.astype(np.longdouble) - ex).astype(np.float64)
    assert np.all(err <= 2.0 ** -40 * absb), (name, float(np.max(err / np.maximum(absb, 1e-300))))
    assert np.linalg.norm(err) <= 1e-13 * np.linalg.norm(absb)
    # the FP64 pipe on the same product, for scale
    ref64 = product(ctx, A, X, False)
    assert np.linalg.norm(ref64 - got) <= 1e-13 * np.linalg.norm(absb)


@pytest.mark.parametrize("shift", [-600, -300, 300, 650])
def test_pair_matrix_scaled_by_powers_of_two(ctx, shift):
    """The matrix is held as values x 2^-s with max |a| 2^-s in [0.5, 1): scaling A
    by 2^shift scales the product exactly."""
    A = P.fem_q1_cube(7)[0]
    As = P.CSR(A.rowptr, A.col, np.ldexp(A.val, shift))
    X = np.random.default_rng(8).standard_normal((A.n, 24))
    base = product(ctx, A, X, True)
    got = product(ctx, As, X, True)
    assert np.array_equal(np.ldexp(got, -shift), base)


@pytest.mark.parametrize("kind", ["huge_x", "inf_x", "nan_x", "huge_matrix"])
def test_pair_out_of_range_matches_fp64_exactly(ctx, kind):
    A = P.fem_q1_cube(7)[1]
    X = np.random.default_rng(9).standard_normal((A.n, 16))
    if kind == "huge_x":
        X[17, 3] = 2.0 ** 105
    elif kind == "inf_x":
        X[5, 0] = np.inf
    elif kind == "nan_x":
        X[A.n - 1, 15] = np.nan
    else:
        A = P.CSR(A.rowptr, A.col, np.ldexp(A.val, 720))
    got = product(ctx, A, X, True)
    ref = product(ctx, A, X, False)
    assert np.array_equal(got, ref, equal_nan=True)


def test_pair_tiny_values_flush_within_bound(ctx):
    """|x| < 2^-126 is dropped and |x| < 2^-74 keeps only its leading float: the
    absolute error stays below 2^-96 sum_j |a_ij| on such entries."""
    A = P.laplace2d(30, 30)[0]
    rng = np.random.default_rng(10)
    X = rng.standard_normal((A.n, 4))
    X[::7] *= 2.0 ** -100
    X[::11] *= 2.0 ** -140
    ex, absb = exact_product(A, X)
    got = product(ctx, A, X, True)
    err = np.abs(got.astype(np.longdouble) - ex).astype(np.float64)
    rowabs = np.add.reduceat(np.abs(A.val), A.rowptr[:-1])[:, None]
    assert np.all(err <= 2.0 ** -40 * absb + 2.0 ** -96 * rowabs)


def test_pair_matrix_values_follow_set_values(ctx):
    """New values (MatSetValues) replace the pairs kept on the matrix."""
    A = P.fem_q1_cube(6)[0]
    X = np.random.default_rng(11).standard_normal((A.n, 8))
    ctx.pair_spmm(True)
    dA = ctx.matrix(A)
    x, y = ctx.multivec(A.n, 8, X), ctx.multivec(A.n, 8)
    G.mat_dot_multivec(dA, x, y, (0, 0), (8, 8))
    first = y.download()
    dA.set_values(3.0 * A.val)
    G.mat_dot_multivec(dA, x, y, (0, 0), (8, 8))
    second = y.download()
    ctx.pair_spmm(False)
    ex, absb = exact_product(P.CSR(A.rowptr, A.col, 3.0 * A.val), X)
    assert np.all(np.abs(second - ex.astype(np.float64)) <= 2.0 ** -40 * absb)
    assert not np.array_equal(first, second)
