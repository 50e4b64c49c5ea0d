"""Full GCGE solves on the GPU against the reference's golden results, the
oracle, dense eigensolvers and analytic spectra.

Parity bar:
* eigenvalues within 1e-10 relative of what the reference reported (golden.json)
  under the reference's own parameters and convergence criterion;
* every residual at or below the requested tolerance under the solver's criterion;
* eigenvectors within a largest principal angle of 1e-7 of the reference
  eigenspace, per cluster of (near-)equal eigenvalues. Clusters are formed on an
  extended reference spectrum (nev + 4 pairs) so that a cluster cut by the nev
  boundary is compared by containment in the full eigenspace. The angle bar is
  checked on solves run to a residual of 1e-10 under ||Ax - lBx|| / (|l| ||Bx||),
  where the residual bound implies it (a 1e-8 residual under the reference's "R"
  criterion on an FEM mass matrix only bounds the angle at ~1e-7 * sqrt(||B^-1||)).
"""
import numpy as np
import pytest
import scipy.linalg as sl

import gcge_gb300 as G
import pyoracle
from gcge_gb300 import problems as P
from _golden import case_matrices, golden

pytestmark = pytest.mark.gpu
GOLD = golden()


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def oracle():
    return pyoracle.Oracle()


def clusters(ev, rtol=1e-8):
    out, cur = [], [0]
    for i in range(1, len(ev)):
        if abs(ev[i] - ev[i - 1]) <= rtol * max(abs(ev[i]), 1e-300):
            cur.append(i)
        else:
            out.append(cur)
            cur = [i]
    out.append(cur)
    return out


def _borth(Z, Bs):
    BZ = Bs @ Z if Bs is not None else Z
    L = np.linalg.cholesky(Z.T @ BZ)
    return np.linalg.solve(L, Z.T).T


def containment_angle(X, Q, Bs=None):
    """Largest principal angle from span(X) into span(Q) (dim X <= dim Q), B inner product."""
    Qx, Qq = _borth(X, Bs), _borth(Q, Bs)
    M = Qx.T @ (Bs @ Qq if Bs is not None else Qq)
    s = np.linalg.svd(M, compute_uv=False)
    return float(np.arccos(np.clip(s.min(), -1.0, 1.0)))


def residuals(A, B, ev, X, conv_type="R"):
    As = A.to_scipy()
    Bs = B.to_scipy() if B is not None else None
    out = []
    for j in range(len(ev)):
        x = X[:, j]
        bx = Bs @ x if Bs is not None else x
        rn = np.linalg.norm(As @ x - ev[j] * bx)
        if conv_type == "R":
            out.append(rn / np.linalg.norm(x) / max(1.0, abs(ev[j])))
        elif conv_type == "BR":
            out.append(rn / (abs(ev[j]) * np.linalg.norm(bx)))
        else:
            out.append(rn / np.linalg.norm(x))
    return np.array(out)


def reference_eigenspace(A, B, k, oracle):
    """Reference eigenpairs covering at least the k smallest: the complete dense spectrum
    (LAPACK dsygvd through scipy) for small n, else the oracle run to 1e-11 for k + 8
    pairs, so that every cluster touching the first k pairs is closed."""
    if A.n <= 3000:
        Ad = A.to_scipy().toarray()
        if B is None:
            w, Z = sl.eigh(Ad)
        else:
            # Dirichlet rows of the reference fixtures make B singular: keep the rows/
            # columns where B is nonzero (the constrained dofs carry no eigenvector mass)
            Bd = B.to_scipy().toarray()
            keep = np.where(np.abs(Bd).sum(axis=1) > 0)[0]
            w, Zk = sl.eigh(Ad[np.ix_(keep, keep)], Bd[np.ix_(keep, keep)])
            Z = np.zeros((A.n, len(w)))
            Z[keep] = Zk
        return w, Z
    ev, X, st = oracle.solve(A, B, oracle.params(nev=k + 8, conv_type="BR", ev_tol=1e-11, ev_max_it=500,
                                                 init_rng=1, seed=3))
    assert st.num_unlock == 0
    return ev, X


def check_vectors(A, B, ev, X, w_ext, Z_ext, angle=1e-7):
    nev = len(ev)
    Bs = B.to_scipy() if B is not None else None
    for c in clusters(w_ext):
        mine = [i for i in c if i < nev]
        if not mine:
            continue
        assert c[-1] < len(w_ext) - 1, "reference spectrum too short to close the cluster"
        assert containment_angle(X[:, mine], Z_ext[:, c], Bs) < angle, (c, ev[mine])


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("name", sorted(GOLD))
def test_eigenvalues_match_reference_golden(ctx, name, precision):
    """The reference's own parameters and criterion; eigenvalues against what it reported."""
    g = GOLD[name]
    A, B = case_matrices(name)
    kw = dict(g["params"], seed=1234, precision=precision)
    kw["ev_max_it"] = max(kw.get("ev_max_it", 30), 100)
    dA, dB = ctx.matrix(A, keep_fp32=precision >= 1), (ctx.matrix(B) if B is not None else None)
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw))
    assert st.num_unlock == 0
    np.testing.assert_allclose(ev, g["eval"], rtol=1e-10, atol=0)
    tol = g["params"].get("ev_tol", 1e-8)
    assert np.all(residuals(A, B, ev, X, g["params"].get("conv_type", "R")) <= tol * 1.05)


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("name", sorted(GOLD))
def test_eigenvectors_principal_angles(ctx, oracle, name, precision):
    g = GOLD[name]
    A, B = case_matrices(name)
    nev = g["params"]["nev"]
    kw = dict(g["params"], seed=99, precision=precision, conv_type="BR", ev_tol=1e-10, ev_max_it=300)
    dA, dB = ctx.matrix(A, keep_fp32=precision >= 1), (ctx.matrix(B) if B is not None else None)
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw))
    assert st.num_unlock == 0
    w, Z = reference_eigenspace(A, B, nev + 4, oracle)
    assert np.max(np.abs(ev - w[:nev]) / np.abs(w[:nev])) < 1e-10
    check_vectors(A, B, ev, X, w, Z)
    assert np.all(residuals(A, B, ev, X, "BR") <= 1.05e-10)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_laplace_analytic(ctx, precision):
    A, _ = P.laplace2d(100, 100)
    dA = ctx.matrix(A, keep_fp32=True)
    ev, X, st = ctx.solve(dA, None, ctx.params(nev=10, seed=3, precision=precision, conv_type="BR", ev_max_it=300))
    assert st.num_unlock == 0
    ex = P.laplace2d_eigs(100, 100, 10)
    assert np.max(np.abs(ev - ex) / ex) < 1e-10
    assert np.all(residuals(A, None, ev, X, "BR") <= 1.05e-8)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_fem_cube_generalized_vs_dense(ctx, oracle, precision):
    A, B = P.fem_q1_cube(10)
    dA, dB = ctx.matrix(A, keep_fp32=True), ctx.matrix(B)
    ev, X, st = ctx.solve(dA, dB, ctx.params(nev=12, block_size=8, seed=5, conv_type="BR", ev_tol=1e-10,
                                             ev_max_it=300, precision=precision))
    assert st.num_unlock == 0
    w, Z = reference_eigenspace(A, B, 16, oracle)
    assert np.max(np.abs(ev - w[:12]) / w[:12]) < 1e-10
    check_vectors(A, B, ev, X, w, Z)
    np.testing.assert_allclose(ev, P.fem_q1_cube_eigs(10, 12), rtol=1e-10)


def test_given_initial_vectors_and_host_entry(ctx, oracle):
    A, B = P.fem_q1_cube(8)
    rng = np.random.default_rng(0)
    X0 = rng.random((A.n, 5))
    p = ctx.params(nev=5, seed=1, ev_max_it=200, conv_type="BR", ev_tol=1e-10)
    ev, X, st = ctx.solve_host(A, B, p, init=X0)
    assert st.num_unlock == 0
    w, Z = reference_eigenspace(A, B, 9, oracle)
    assert np.max(np.abs(ev - w[:5]) / w[:5]) < 1e-10
    check_vectors(A, B, ev, X, w, Z)


@pytest.mark.parametrize("nev,bs", [(1, 0), (9, 3), (20, 7)])
def test_small_nev_and_blocks(ctx, nev, bs):
    A, _ = P.laplace2d(20, 17)
    ev, X, st = ctx.solve(ctx.matrix(A), None, ctx.params(nev=nev, block_size=bs, seed=2, ev_max_it=500))
    assert st.num_unlock == 0
    ex = P.laplace2d_eigs(20, 17, nev)
    assert np.max(np.abs(ev - ex) / ex) < 1e-10


@pytest.mark.parametrize("precision", [1, 2])
def test_varcoef3d_mixed(ctx, oracle, precision):
    """7-point variable-coefficient diffusion (exp of a sigma-1 Gaussian field, lumped
    diagonal mass U[1, 2]): the family of the 160^3 configuration at 16^3 cells."""
    A, B = P.varcoef3d(nc=16)
    dA, dB = ctx.matrix(A, keep_fp32=True), ctx.matrix(B)
    ev, X, st = ctx.solve(dA, dB, ctx.params(nev=20, block_size=24, seed=8, conv_type="BR", ev_tol=1e-10,
                                             ev_max_it=800, precision=precision))
    assert st.num_unlock == 0
    oe, oX, ost = oracle.solve(A, B, oracle.params(nev=24, conv_type="BR", ev_tol=1e-11, ev_max_it=800,
                                                   init_rng=1, seed=4))
    assert ost.num_unlock == 0
    assert np.max(np.abs(ev - oe[:20]) / np.abs(oe[:20])) < 1e-10
    assert np.all(residuals(A, B, ev, X, "BR") <= 1.05e-10)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_jacobi_preconditioned_inner_solve(ctx, oracle, precision):
    """precond = 1 (the role of a linear solver installed in ops->LinearSolver):
    Jacobi-preconditioned block CG gives the same eigenpairs as the oracle in no
    more outer iterations than plain block CG on a variable-coefficient problem."""
    A, B = P.varcoef3d(nc=16, seed=21)
    dA, dB = ctx.matrix(A, keep_fp32=True), ctx.matrix(B)
    its = {}
    for pc in (0, 1):
        ev, X, st = ctx.solve(dA, dB, ctx.params(nev=20, block_size=24, seed=8, conv_type="BR", ev_max_it=500,
                                                 precision=precision, precond=pc))
        assert st.num_unlock == 0
        assert np.all(residuals(A, B, ev, X, "BR") <= 1.05e-8)
        its[pc] = st.num_iter
        if pc == 1:
            oe, oX, ost = oracle.solve(A, B, oracle.params(nev=24, conv_type="BR", ev_tol=1e-11, ev_max_it=800,
                                                           init_rng=1, seed=4))
            assert np.max(np.abs(ev - oe[:20]) / np.abs(oe[:20])) < 1e-9
    assert its[1] <= its[0], its


@pytest.mark.parametrize("precision", [1, 2])
def test_irregular_graph_mixed(ctx, oracle, precision):
    """Power-law graph Laplacian (irregular rows up to 300 nonzeros), B = diag U[1,2]."""
    A, B = P.powerlaw_graph(4000, seed=11, dmax=300)
    dA, dB = ctx.matrix(A, keep_fp32=True), ctx.matrix(B)
    ev, X, st = ctx.solve(dA, dB, ctx.params(nev=16, block_size=16, seed=8, conv_type="BR", ev_tol=1e-10,
                                             ev_max_it=800, precision=precision))
    assert st.num_unlock == 0
    oe, oX, ost = oracle.solve(A, B, oracle.params(nev=20, conv_type="BR", ev_tol=1e-11, ev_max_it=800,
                                                   init_rng=1, seed=4))
    assert np.max(np.abs(ev - oe[:16]) / np.abs(oe[:16])) < 1e-10
    assert np.all(residuals(A, B, ev, X, "BR") <= 1.05e-10)


@pytest.mark.parametrize("form", ["text", "binary"])
def test_reference_pencil_from_file(ctx, tmp_path, form):
    """The reference's A_5/M_5 pencil written out in its text CSR layout (and in
    the binary form), read and uploaded by GCGE_GPU_MatCreateFromFile, solved with
    the reference's parameters: eigenvalues within 1e-10 of what it reported."""
    from test_csrio import write_text
    g = GOLD["fem33_nev10_dirichlet"]
    A, B = case_matrices("fem33_nev10_dirichlet")
    paths = []
    for name, M in (("A_5", A), ("M_5", B)):
        p = str(tmp_path / (name + (".txt" if form == "text" else ".bin")))
        write_text(p, M) if form == "text" else G.write_csr_binary(p, M)
        paths.append(p)
    dA, dB = ctx.matrix_from_file(paths[0]), ctx.matrix_from_file(paths[1])
    assert dA.n == A.n
    kw = dict(g["params"], seed=1234)
    kw["ev_max_it"] = max(kw.get("ev_max_it", 30), 100)
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw))
    assert st.num_unlock == 0
    np.testing.assert_allclose(ev, g["eval"], rtol=1e-10, atol=0)


@pytest.mark.parametrize("w_orth_type", ["scbgs", "bgs", "gs"])
@pytest.mark.parametrize("name", ["fem33_nev10_dirichlet", "laplace30x20_nev12_block4"])
def test_w_orth_type_variants(ctx, name, w_orth_type):
    """The reference's W-orthonormalisation variants (w_orth_type, src/gcge_eigsol.c:448-472):
    the same eigenvalues as the reference reported, every residual within the tolerance.
    The reference build itself converges with scbgs / bgs / gs in the iterations of
    the default (13 and 33 here); its cbgs does not (6 and 7 pairs left, eigenvalues
    off by O(1) after 100 / 200 iterations), so cbgs is checked as an
    orthonormalisation only (test_gpu_ops.test_orthonormalize)."""
    g = GOLD[name]
    A, B = case_matrices(name)
    kw = dict(g["params"], seed=1234, w_orth_type=w_orth_type)
    kw["ev_max_it"] = max(kw.get("ev_max_it", 30), 100)
    dA, dB = ctx.matrix(A), (ctx.matrix(B) if B is not None else None)
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw))
    assert st.num_unlock == 0
    np.testing.assert_allclose(ev, g["eval"], rtol=1e-10, atol=0)
    tol = g["params"].get("ev_tol", 1e-8)
    assert np.all(residuals(A, B, ev, X, g["params"].get("conv_type", "R")) <= tol * 1.05)


@pytest.mark.parametrize("name", ["fem33_nev10_dirichlet", "laplace30x20_nev12_block4", "laplace100_nev10",
                                  "femcube10_nev6_abs"])
def test_soft_locking(ctx, name):
    """opt_rr_eig_partly = 1 (soft locking, src/gcge_rayleighritz.c:364-400): the
    converged leading pairs are kept and only the trailing projected block is
    solved. The reference build converges with it in the iterations of its default
    (13 / 33 / 23 / 18 on these cases); here: the reference's eigenvalues, every
    residual within the tolerance, and no more than two extra outer iterations."""
    g = GOLD[name]
    A, B = case_matrices(name)
    kw = dict(g["params"], seed=1234)
    kw["ev_max_it"] = max(kw.get("ev_max_it", 30), 100)
    dA, dB = ctx.matrix(A), (ctx.matrix(B) if B is not None else None)
    ev0, X0, st0 = ctx.solve(dA, dB, ctx.params(**kw))
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw, opt_rr_eig_partly=1))
    assert st.num_unlock == 0
    np.testing.assert_allclose(ev, g["eval"], rtol=1e-10, atol=0)
    tol = g["params"].get("ev_tol", 1e-8)
    assert np.all(residuals(A, B, ev, X, g["params"].get("conv_type", "R")) <= tol * 1.05)
    assert st.num_iter <= st0.num_iter + 2, (st.num_iter, st0.num_iter)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["fem33_nev10_dirichlet", "laplace30x20_nev12_block4", "femcube10_nev6_abs",
                                  "fem9_nev4_dirichlet"])
def test_a_orthogonal_mode(ctx, oracle, name, precision):
    """orth_type "A" (src/gcge_eigsol.c:100-113): the basis is A-orthonormal and the
    projected matrix is V^T B V, whose largest eigenvalues give lambda = 1/mu. The
    reference build's own A mode fails (a segmentation fault without B, NaN or Inf
    eigenvalues with it: its GCGE_SortEigenpairs reverses the smallest eigenvalues of
    V^T B V instead of taking the largest), so the bar is the dense generalized
    eigensolver (LAPACK dsygvd): eigenvalues within 1e-10, every residual within
    the tolerance, eigenvectors within a principal angle of 1e-7 per cluster, and
    the returned vectors A-orthonormal."""
    g = GOLD[name]
    A, B = case_matrices(name)
    nev = g["params"]["nev"]
    kw = dict(g["params"], seed=1234, precision=precision, conv_type="BR", ev_tol=1e-10, ev_max_it=300,
              orth_type="A")
    dA, dB = ctx.matrix(A, keep_fp32=precision >= 1), (ctx.matrix(B) if B is not None else None)
    ev, X, st = ctx.solve(dA, dB, ctx.params(**kw))
    assert st.num_unlock == 0
    w, Z = reference_eigenspace(A, B, nev, oracle)
    np.testing.assert_allclose(ev, w[:nev], rtol=1e-10, atol=0)
    assert np.all(residuals(A, B, ev, X, "BR") <= 1e-10 * 1.05)
    check_vectors(A, B, ev, X, w[:nev + 4], Z[:, :nev + 4])
    XtAX = X.T @ (A.to_scipy() @ X)
    assert np.max(np.abs(XtAX - np.eye(nev))) < 1e-10


def test_orth_type_rejects_unknown_value(ctx):
    A, _ = P.laplace2d(20, 20)
    dA = ctx.matrix(A)
    with pytest.raises(G.GcgeGpuError) as e:
        ctx.solve(dA, None, ctx.params(nev=4, orth_type="C"))
    assert e.value.status == G.ERR_ARG
