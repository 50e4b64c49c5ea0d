"""The GCGE_OPS plug-in table filled by GCGE_GPU_SetOps, called through its
function pointers with the reference's member signatures (src/gcge_ops.h:29-215),
each member compared with the oracle's restatement of the reference default or
CSR backend operation, and the dsyevx-signature eigensolve with LAPACK (scipy)."""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg as sl

import gcge_gb300 as G
import pyoracle
from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu

V_ = C.c_void_p
PP = C.POINTER(C.c_void_p)
PI = C.POINTER(C.c_int)
PD = C.POINTER(C.c_double)
F = C.CFUNCTYPE
FIELDS = [
    ("VecSetRandomValue", F(None, V_)), ("MatDotVec", F(None, V_, V_, V_)),
    ("VecAxpby", F(None, C.c_double, V_, C.c_double, V_)), ("VecInnerProd", F(None, V_, V_, PD)),
    ("VecLocalInnerProd", F(None, V_, V_, PD)), ("VecCreateByVec", F(None, PP, V_)),
    ("VecCreateByMat", F(None, PP, V_)), ("VecDestroy", F(None, PP)), ("LinearSolver", V_),
    ("linear_solver_workspace", V_), ("Orthonormalization", V_), ("DenseMatCreate", V_), ("DenseMatDestroy", V_),
    ("MultiVecCreateByVec", F(None, C.POINTER(PP), C.c_int, V_, V_)),
    ("MultiVecCreateByMat", F(None, C.POINTER(PP), C.c_int, V_, V_)),
    ("MultiVecCreateByMultiVec", F(None, C.POINTER(PP), C.c_int, PP, V_)),
    ("MultiVecDestroy", F(None, C.POINTER(PP), C.c_int, V_)),
    ("MultiVecSetRandomValue", F(None, PP, C.c_int, C.c_int, V_)),
    ("MatDotMultiVec", F(None, V_, PP, PP, PI, PI, V_)),
    ("MultiVecAxpby", F(None, C.c_double, PP, C.c_double, PP, PI, PI, V_)),
    ("MultiVecAxpbyColumn", F(None, C.c_double, PP, C.c_int, C.c_double, PP, C.c_int, V_)),
    ("MultiVecLinearComb", F(None, PP, PP, PI, PI, PD, C.c_int, V_, C.c_int, V_)),
    ("MultiVecInnerProd", F(None, PP, PP, PD, C.c_char_p, PI, PI, C.c_int, V_)),
    ("MultiVecSwap", F(None, PP, PP, PI, PI, V_)), ("MultiVecPrint", V_),
    ("GetVecFromMultiVec", F(None, PP, C.c_int, PP)), ("RestoreVecForMultiVec", F(None, PP, C.c_int, PP)),
    ("SetDirichletBoundary", F(None, PP, C.c_int, V_, V_)),
    ("DenseMatEigenSolver", F(None, C.c_char_p, C.c_char_p, C.c_char_p, PI, PD, PI, PD, PD, PI, PI, PD, PI, PD, PD,
                              PI, PI, PD, PI, PI, PI, PI, PI)),
    ("DenseMatDotDenseMat", V_), ("DenseSymMatDotDenseMat", V_), ("ArrayDotArray", V_), ("ArrayNorm", V_),
    ("ArrayAXPBY", V_), ("ArrayCopy", V_), ("ArrayScale", V_),
]


class OpsTable(C.Structure):
    _fields_ = FIELDS


def ints(*v):
    return (C.c_int * len(v))(*v)


@pytest.fixture(scope="module")
def env():
    ctx = G.Context(0)
    tab = OpsTable()
    assert ctx.lib.GCGE_GPU_SetOps(ctx.h, C.byref(tab)) == 0
    yield ctx, tab
    ctx.close()


def mv_create(ctx, tab, A, k):
    h = PP()
    tab.MultiVecCreateByMat(C.byref(h), k, A.h, None)
    return h


def mv_block(ctx, h):
    blk, col = V_(), C.c_int()
    assert ctx.lib.GCGE_GPU_OpsMultiVecBlock(h, C.byref(blk), C.byref(col)) == 0
    return blk, col.value


def mv_upload(ctx, h, X):
    blk, col = mv_block(ctx, h)
    cm = np.ascontiguousarray(X.T)
    assert ctx.lib.GCGE_GPU_MultiVecUpload(blk, col, X.shape[1], cm.ctypes.data_as(V_)) == 0


def mv_download(ctx, h, k, n):
    blk, col = mv_block(ctx, h)
    cm = np.zeros((k, n))
    assert ctx.lib.GCGE_GPU_MultiVecDownload(blk, col, k, cm.ctypes.data_as(V_)) == 0
    return cm.T


def test_table_members_against_oracle(env):
    ctx, tab = env
    o = pyoracle.Oracle()
    A, Bm = P.fem_q1_cube(11)
    n = A.n
    dA = ctx.matrix(A)
    rng = np.random.default_rng(10)
    Xh = rng.standard_normal((n, 8))
    V = mv_create(ctx, tab, dA, 8)
    W = mv_create(ctx, tab, dA, 8)
    mv_upload(ctx, V, Xh)
    # MatDotMultiVec: W[:, 3:7] = A V[:, 1:5]
    tab.MatDotMultiVec(dA.h, V, W, ints(1, 3), ints(5, 7), None)
    got = mv_download(ctx, W, 8, n)[:, 3:7]
    ref = o.matmultivec(A, np.ascontiguousarray(Xh[:, 1:5].T)).T
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-13
    # MultiVecInnerProd, nonsym with lda 6
    a = np.full(6 * 3, 5.0)
    tab.MultiVecInnerProd(V, W, a.ctypes.data_as(PD), b"nonsym", ints(0, 3), ints(4, 6), 6, None)
    Wh = mv_download(ctx, W, 8, n)
    ref = Xh[:, 0:4].T @ Wh[:, 3:6]
    for j in range(3):
        np.testing.assert_allclose(a[6 * j:6 * j + 4], ref[:, j], rtol=1e-12)
        assert np.all(a[6 * j + 4:6 * j + 6] == 5.0)
    # MultiVecLinearComb: W[:, 0:2] = V[:, 2:6] * coef (lda 5)
    coef = rng.standard_normal(5 * 2)
    tab.MultiVecLinearComb(V, W, ints(2, 0), ints(6, 2), coef.ctypes.data_as(PD), 5, None, 0, None)
    got = mv_download(ctx, W, 8, n)[:, 0:2]
    ref = o.lincomb(np.ascontiguousarray(Xh[:, 2:6].T), coef, 2, 5).T
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-13
    # MultiVecAxpby and AxpbyColumn (CSR_VecAxpby special cases)
    before = mv_download(ctx, W, 8, n)
    tab.MultiVecAxpby(2.0, V, -0.5, W, ints(0, 4), ints(2, 6), None)
    got = mv_download(ctx, W, 8, n)
    np.testing.assert_allclose(got[:, 4:6], 2.0 * Xh[:, 0:2] - 0.5 * before[:, 4:6], rtol=1e-14)
    tab.MultiVecAxpbyColumn(1.0, V, 7, 0.0, W, 7, None)
    assert np.array_equal(mv_download(ctx, W, 8, n)[:, 7], Xh[:, 7])
    # MultiVecSwap moves data, handles stay put
    wb = mv_download(ctx, W, 8, n)
    tab.MultiVecSwap(V, W, ints(0, 6), ints(2, 8), None)
    v2, w2 = mv_download(ctx, V, 8, n), mv_download(ctx, W, 8, n)
    assert np.array_equal(v2[:, 0:2], wb[:, 6:8]) and np.array_equal(w2[:, 6:8], Xh[:, 0:2])
    # single-vector members on columns obtained with GetVecFromMultiVec
    x, y = V_(), V_()
    tab.GetVecFromMultiVec(V, 3, C.byref(x))
    tab.GetVecFromMultiVec(W, 1, C.byref(y))
    tab.MatDotVec(dA.h, x, y)
    got = mv_download(ctx, W, 8, n)[:, 1]
    np.testing.assert_allclose(got, A.to_scipy() @ v2[:, 3], rtol=1e-12, atol=1e-14)
    val = C.c_double()
    tab.VecInnerProd(x, y, C.byref(val))
    assert abs(val.value - v2[:, 3] @ got) < 1e-12 * abs(val.value)
    tab.VecAxpby(0.0, x, 3.0, y)
    np.testing.assert_allclose(mv_download(ctx, W, 8, n)[:, 1], 3.0 * got, rtol=1e-15)
    # standalone vector create/destroy
    z = V_()
    tab.VecCreateByMat(C.byref(z), dA.h)
    tab.VecSetRandomValue(z)
    tab.VecDestroy(C.byref(z))
    tab.MultiVecDestroy(C.byref(V), 8, None)
    tab.MultiVecDestroy(C.byref(W), 8, None)
    assert ctx.last_error() == 0


@pytest.mark.parametrize("m", [57, 130, 300, 520])   # one SM (m < 256); the cluster tridiagonalisation
def test_table_dense_eigensolver_matches_lapack(env, m):
    ctx, tab = env
    rng = np.random.default_rng(12 + m)
    lda = m + 3
    M = rng.standard_normal((m, m))
    M = M + M.T
    M[20, 21] = M[21, 20] = 0.0
    a = np.zeros((m, lda))          # column-major with lda: a[col, row]
    a[:, :m] = M.T
    il, iu = 1, 12
    k = iu - il + 1
    ev = np.zeros(m)
    lde = m + 7
    Z = np.zeros((k, lde))
    nev, info = C.c_int(), C.c_int()
    iv = lambda v: C.byref(C.c_int(v))  # noqa: E731
    dummy = C.c_double()
    tab.DenseMatEigenSolver(b"V", b"I", b"U", iv(m), a.ctypes.data_as(PD), iv(lda), C.byref(dummy),
                            C.byref(dummy), iv(il), iv(iu), C.byref(dummy), C.byref(nev), ev.ctypes.data_as(PD),
                            Z.ctypes.data_as(PD), iv(lde), None, None, iv(8 * m), None, None, None, C.byref(info))
    assert info.value == 0 and nev.value == k
    w, U = sl.eigh(M)
    np.testing.assert_allclose(ev[:k], w[:k], rtol=1e-12, atol=1e-12 * np.abs(w).max())
    for j in range(k):
        assert abs(abs(Z[j, :m] @ U[:, j]) - 1.0) < 1e-10


def test_table_linear_solver_hook(env):
    """GCGE_GPU_OpsSetLinearSolver installs a device Jacobi-preconditioned CG in the
    table's LinearSolver member (the hook GCGE calls per W column in place of its
    block CG, src/gcge_xpw.c:177-191); kind 0 removes it."""
    ctx, tab = env
    import scipy.sparse.linalg as spla
    A, _ = P.varcoef2d(nc=40, seed=3, sigma=1.0)
    n = A.n
    dA = ctx.matrix(A)
    rng = np.random.default_rng(14)
    b = rng.standard_normal(n)
    assert ctx.lib.GCGE_GPU_OpsSetLinearSolver(C.byref(tab), 1, 5000, 1e-12) == 0
    assert tab.LinearSolver
    solve = C.CFUNCTYPE(None, V_, V_, V_, V_)(tab.LinearSolver)
    h = mv_create(ctx, tab, dA, 2)
    mv_upload(ctx, h, np.stack([b, np.zeros(n)], axis=1))
    solve(dA.h, h[0], h[1], C.cast(C.byref(tab), V_))
    assert ctx.last_error() == 0
    out = mv_download(ctx, h, 2, n)
    assert np.array_equal(out[:, 0], b)                      # the right-hand side is left as it was
    x_ref = spla.spsolve(A.to_scipy().tocsc(), b)
    assert np.linalg.norm(out[:, 1] - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    tab.MultiVecDestroy(C.byref(h), 2, None)
    assert ctx.lib.GCGE_GPU_OpsSetLinearSolver(C.byref(tab), 0, 20, 1e-2) == 0
    assert not tab.LinearSolver
    assert ctx.lib.GCGE_GPU_OpsSetLinearSolver(C.byref(tab), 2, 20, 1e-2) == 1
