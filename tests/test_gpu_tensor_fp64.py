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
