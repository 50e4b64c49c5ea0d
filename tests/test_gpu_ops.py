"""Per-operation parity of the CUDA path (through the C ABI) against the oracle.

Each GCGE_OPS multivector member is compared with the oracle's restatement of
the reference default (src/gcge_ops.c:115-300) or CSR backend
(app/csr/gcge_app_csr.c:297-378) on seeded inputs. Tolerances: 1e-13 relative
(FP64 arithmetic in a different order, fused multiply-adds).
"""
import numpy as np
import pytest

import gcge_gb300 as G
import pyoracle
from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu
RTOL = 1e-13


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def oracle():
    return pyoracle.Oracle()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def cols_to_oracle(X):
    return np.ascontiguousarray(np.asarray(X).T)


@pytest.mark.parametrize("maker,k", [(lambda: P.laplace2d(37, 23)[0], 1), (lambda: P.laplace2d(37, 23)[0], 7),
                                     (lambda: P.fem_q1_cube(9)[0], 64), (lambda: P.fem_q1_cube(9)[1], 65),
                                     (lambda: P.powerlaw_graph(3000, seed=5, dmax=300)[0], 33)])
@pytest.mark.parametrize("sx,sy", [(2, 4), (1, 3)])      # (1, 3): column ranges off the 16-byte grid
def test_matdotmultivec(ctx, oracle, maker, k, sx, sy):
    A = maker()
    rng = np.random.default_rng(1)
    X = rng.standard_normal((A.n, k + 3))
    dA = ctx.matrix(A)
    x = ctx.multivec(A.n, k + 3, X)
    y = ctx.multivec(A.n, k + 5)
    G.mat_dot_multivec(dA, x, y, (sx, sy), (sx + k, sy + k))
    got = y.download()[:, sy:sy + k]
    ref = oracle.matmultivec(A, cols_to_oracle(X[:, sx:sx + k])).T
    assert rel(got, ref) < RTOL


@pytest.mark.parametrize("a,b", [(0.0, 2.5), (1.0, 0.0), (-3.0, 0.0), (2.0, -0.5), (0.0, 0.0)])
def test_axpby_special_cases(ctx, oracle, a, b):
    rng = np.random.default_rng(2)
    n = 1001
    X, Y = rng.standard_normal((n, 9)), rng.standard_normal((n, 9))
    x, y = ctx.multivec(n, 9, X), ctx.multivec(n, 9, Y)
    G.multivec_axpby(a, x, b, y, (1, 3), (7, 9))
    got = y.download()
    ref = Y.copy()
    for j in range(6):
        ref[:, 3 + j] = oracle.axpby(a, X[:, 1 + j], b, Y[:, 3 + j])
    assert np.array_equal(got[:, :3], Y[:, :3])
    assert rel(got, ref) < RTOL


@pytest.mark.parametrize("n,k1,k2,lda", [(5000, 13, 9, 20), (20000, 70, 40, 70), (333, 1, 1, 1), (4097, 33, 65, 40)])
def test_linear_comb(ctx, oracle, n, k1, k2, lda):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, k1))
    coef = rng.standard_normal(lda * k2)
    x, y = ctx.multivec(n, k1, X), ctx.multivec(n, k2 + 2)
    G.multivec_linear_comb(x, y, (0, 2), (k1, 2 + k2), coef, lda)
    got = y.download()[:, 2:]
    ref = oracle.lincomb(cols_to_oracle(X), coef, k2, lda).T
    assert rel(got, ref) < RTOL


@pytest.mark.parametrize("sym", [False, True])
@pytest.mark.parametrize("n,k1,k2,lda", [(10000, 17, 17, 30), (300000, 64, 64, 64), (777, 40, 40, 45)])
def test_inner_prod(ctx, oracle, sym, n, k1, k2, lda):
    rng = np.random.default_rng(4)
    V, W = rng.standard_normal((n, k1 + 1)), rng.standard_normal((n, k2))
    if sym:
        W = V[:, 1:1 + k2] * 0.5 + W * 1e-3
    v, w = ctx.multivec(n, k1 + 1, V), ctx.multivec(n, k2, W)
    got = G.multivec_inner_prod(v, w, (1, 0), (1 + k1, k2), lda, sym=sym, out=np.full(lda * k2, 7.0))
    ref = np.full(lda * k2, 7.0)
    ref_o = oracle.innerprod(cols_to_oracle(V[:, 1:1 + k1]), cols_to_oracle(W), lda, sym)
    for j in range(k2):
        ref[j * lda:j * lda + k1] = ref_o[j * lda:j * lda + k1]
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.max(np.abs(ref)))


def test_swap(ctx):
    rng = np.random.default_rng(5)
    n = 999
    X, Y = rng.standard_normal((n, 6)), rng.standard_normal((n, 5))
    x, y = ctx.multivec(n, 6, X), ctx.multivec(n, 5, Y)
    G.multivec_swap(x, y, (1, 2), (4, 5))
    gx, gy = x.download(), y.download()
    assert np.array_equal(gx[:, 1:4], Y[:, 2:5]) and np.array_equal(gy[:, 2:5], X[:, 1:4])
    assert np.array_equal(gx[:, [0, 4, 5]], X[:, [0, 4, 5]])


@pytest.mark.parametrize("k,max_it", [(8, 20), (13, 7)])
def test_bcg_fp64_matches_oracle(ctx, oracle, k, max_it):
    """FP64 block CG follows GCGE_BCG's iteration (including its active-column rule)."""
    A, _ = P.laplace2d(40, 30)
    rng = np.random.default_rng(6)
    R0, W0 = rng.standard_normal((A.n, k)), rng.standard_normal((A.n, k)) * 0.1
    dA = ctx.matrix(A)
    r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k + 1)
    w.upload(W0, 1)
    G.bcg(dA, r, 0, w, 1, k, cg_max_it=max_it, cg_rate=1e-2, precision=0)
    Xo, Ro = oracle.bcg(A, cols_to_oracle(R0), cols_to_oracle(W0), max_it, 1e-2)
    assert rel(w.download()[:, 1:], Xo.T) < 1e-9
    assert rel(r.download(), Ro.T) < 1e-7


def test_bcg_fp32_close_to_fp64(ctx):
    A, _ = P.laplace2d(40, 30)
    rng = np.random.default_rng(7)
    k = 10
    R0 = rng.standard_normal((A.n, k))
    dA = ctx.matrix(A, keep_fp32=True)
    out = []
    for prec in (0, 1):
        r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k)
        G.bcg(dA, r, 0, w, 0, k, cg_max_it=20, cg_rate=1e-2, precision=prec)
        out.append((w.download(), r.download()))
    # 19 rounds shrink every residual; the FP32 defect-correction iterate tracks the FP64 one
    Asp = A.to_scipy()
    res = []
    for Wsol, _ in out:
        r = np.linalg.norm(R0 - Asp @ Wsol, axis=0) / np.linalg.norm(R0, axis=0)
        assert np.all(r < 0.5)
        res.append(r)
    assert np.max(np.abs(res[1] - res[0])) < 1e-3
    assert rel(out[1][0], out[0][0]) < 1e-3


@pytest.mark.parametrize("k,max_it,rate", [(2, 8, 1e-2), (4, 10, 1e-2), (7, 10, 1e-2), (10, 10, 1e-2),
                                            (10, 5, 1e-1), (20, 8, 1e-2), (40, 8, 1e-2), (70, 6, 1e-1)])
def test_bcg_fp32_tracks_fp64_while_columns_deactivate(ctx, k, max_it, rate):
    """Columns of very different difficulty leave the active range at different
    rounds; the FP32 rounds' per-block partials must stay aligned with the column
    sums over the full column range, so the FP32 iterate keeps FP32 accuracy."""
    A, _ = P.laplace2d(40, 30)
    Asp = A.to_scipy()
    rng = np.random.default_rng(100 + k)
    R0 = rng.standard_normal((A.n, k)) * np.logspace(0, -3, k)
    R0[:, ::3] = Asp @ rng.standard_normal((A.n, (k + 2) // 3))
    dA = ctx.matrix(A, keep_fp32=True)
    out = []
    for prec in (0, 1):
        r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k)
        G.bcg(dA, r, 0, w, 0, k, cg_max_it=max_it, cg_rate=rate, precision=prec)
        out.append(w.download())
    assert np.all(np.isfinite(out[1]))
    assert rel(out[1], out[0]) < 1e-4


@pytest.mark.parametrize("k", [3, 8, 16, 30, 64, 100, 200])
def test_bcg_fp32_long_rows(ctx, k):
    """A power-law graph whose hub rows exceed the long-row length: those rows go
    to the block-per-row SpMM launch, the rest to the grid-stride one; the FP32
    iterate tracks the FP64 one and repeats bit for bit (fixed-order sums). The
    shift keeps the condition number near 25, so that FP32 rounding, amplified by
    the rounds roughly in proportion to it, stays far below the bound, while a
    wrong sum over a hub row would not."""
    A, _ = P.powerlaw_graph(n=20000, seed=11, shift=100.0)
    assert int(np.sum(np.diff(A.rowptr) > 64)) > 100
    rng = np.random.default_rng(200 + k)
    R0 = rng.standard_normal((A.n, k))
    dA = ctx.matrix(A, keep_fp32=True)
    out = []
    for prec in (0, 1, 1):
        r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k)
        G.bcg(dA, r, 0, w, 0, k, cg_max_it=12, cg_rate=1e-30, precision=prec)
        out.append(w.download())
    assert np.all(np.isfinite(out[1]))
    assert rel(out[1], out[0]) < 1e-4
    assert np.array_equal(out[1], out[2])


@pytest.mark.parametrize("k", [33, 40, 64])
def test_bcg_fp32_fem_cube(ctx, k):
    """Q1 cube stiffness (27 entries per row) at the solver's block widths: the
    FP32 iterate tracks the FP64 one and repeats bit for bit; new values of the
    same structure scale the result exactly (2 A: half the iterate)."""
    A, _ = P.fem_q1_cube(24)
    rng = np.random.default_rng(300 + k)
    R0 = rng.standard_normal((A.n, k))
    dA = ctx.matrix(A, keep_fp32=True)
    out = []
    for prec in (0, 1, 1):
        r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k)
        G.bcg(dA, r, 0, w, 0, k, cg_max_it=12, cg_rate=1e-30, precision=prec)
        out.append(w.download())
    assert np.all(np.isfinite(out[1]))
    assert rel(out[1], out[0]) < 1e-4
    assert np.array_equal(out[1], out[2])
    # new values, same structure: 2 A
    dA.set_values(2.0 * A.val)
    r, w = ctx.multivec(A.n, k, R0), ctx.multivec(A.n, k)
    G.bcg(dA, r, 0, w, 0, k, cg_max_it=12, cg_rate=1e-30, precision=1)
    assert rel(2.0 * w.download(), out[1]) < 1e-5


def test_newton_reciprocal_of_inverse_iteration(ctx):
    """The reciprocal used for the pivots of inverse iteration (hardware
    approximation refined by two Newton-Raphson steps) is within 2 ulp of the
    IEEE quotient 1/x over the normal range; zero, infinities and subnormal
    inputs take the exact division."""
    import ctypes as C
    lib = G.load()
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.uniform(1.0, 2.0, 4000) * np.exp2(rng.integers(-1020, 1020, 4000)),
                        -rng.uniform(1.0, 2.0, 1000) * np.exp2(rng.integers(-60, 60, 1000)),
                        [1.0, -1.0, 3.0, 2.0 ** -1022, 2.0 ** 1023, 0.0, -0.0, np.inf, -np.inf, 5e-324, 1e-310]])
    r = np.zeros_like(x)
    lib.gb_recip_check.restype = C.c_int
    assert lib.gb_recip_check(len(x), x.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p)) == 0
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / x
    normal = np.isfinite(ref) & (np.abs(x) >= 2.0 ** -1022) & np.isfinite(x) & (np.abs(ref) >= 2.0 ** -1022)
    ulp = np.spacing(np.abs(ref[normal]))
    assert np.max(np.abs(r[normal] - ref[normal]) / ulp) <= 2.0
    special = ~normal
    assert np.array_equal(r[special], ref[special]) or np.allclose(r[special], ref[special], rtol=1e-15, equal_nan=True)


@pytest.mark.parametrize("w_orth_type", [None, "cbgs", "scbgs", "bgs"])
@pytest.mark.parametrize("use_b", [False, True])
def test_orthonormalize(ctx, use_b, w_orth_type):
    """B-orthonormalisation of W against B-orthonormal V, every w_orth_type variant:
    orthonormal to 1e-12, the dependent column dropped, the inputs in the span."""
    Aa, Bb = P.fem_q1_cube(12)
    B = Bb if use_b else None
    n = Aa.n
    rng = np.random.default_rng(8)
    k0, k = 9, 12
    V = rng.standard_normal((n, k0 + k))
    V[:, k0 + 5] = V[:, k0 + 2] * 2 - V[:, 3]          # dependent on earlier columns
    Bs = B.to_scipy() if B is not None else None
    # make the first k0 columns B-orthonormal on the host
    Q = V[:, :k0].copy()
    M = Q.T @ (Bs @ Q if Bs is not None else Q)
    L = np.linalg.cholesky(M)
    V[:, :k0] = np.linalg.solve(L, Q.T).T
    v = ctx.multivec(n, k0 + k, V)
    dB = ctx.matrix(B) if B is not None else None
    end = G.orthonormalize(v, k0, k0 + k, dB, w_orth_type=w_orth_type)
    assert end == k0 + k - 1                             # the dependent column was deflated
    Q = v.download()[:, :end]
    BQ = Bs @ Q if Bs is not None else Q
    assert np.max(np.abs(Q.T @ BQ - np.eye(end))) < 1e-12
    # span of the kept columns contains the independent inputs
    keep = [c for c in range(k0 + k) if c != k0 + 5]
    coeffs = Q.T @ (Bs @ V[:, keep] if Bs is not None else V[:, keep])
    resid = V[:, keep] - Q @ coeffs
    assert np.max(np.abs(resid)) / np.max(np.abs(V)) < 1e-10


def test_matrix_csr_validation(ctx):
    A, _ = P.laplace2d(5, 5)
    bad = P.CSR(A.rowptr.copy(), A.col.copy(), A.val.copy())
    bad.col[3] = 999
    with pytest.raises(G.GcgeGpuError) as e:
        ctx.matrix(bad)
    assert e.value.status == 4
    bad2 = P.CSR(A.rowptr.copy(), A.col.copy(), A.val.copy())
    bad2.rowptr[4] = bad2.rowptr[5] + 1
    with pytest.raises(G.GcgeGpuError):
        ctx.matrix(bad2)
    bad3 = P.CSR(A.rowptr.copy(), A.col.copy(), A.val.copy())
    bad3.col[-1] = -1                                   # checked on the device after the upload
    with pytest.raises(G.GcgeGpuError) as e:
        ctx.matrix(bad3)
    assert e.value.status == 4
    dA = ctx.matrix(A)                                  # a valid matrix after the rejected ones
    assert dA.n == A.n


def test_range_checks(ctx):
    x, y = ctx.multivec(100, 4), ctx.multivec(100, 4)
    with pytest.raises(G.GcgeGpuError):
        G.multivec_axpby(1.0, x, 0.0, y, (0, 2), (3, 5))
