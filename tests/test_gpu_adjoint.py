"""Adjoint (differentiation) kernels on the GPU through the C ABI: the pattern
gradient (SDDMM) against numpy, the eigenvector adjoint solve against a dense
eigendecomposition, and the gradient of an eigenpair loss against torch autograd
through a dense eigensolver and against central finite differences.

The torch.autograd.Function below exists only in this test harness: its forward
runs the GPU eigensolver, its backward the adjoint entry points."""
import numpy as np
import pytest

import gcge_gb300 as G
from gcge_gb300 import problems as P
import adjoint_dense as AD

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("r", [1, 3, 8, 9, 40])
def test_pattern_grad_matches_numpy(ctx, r):
    A, _ = P.powerlaw_graph(2000, seed=4, dmax=200)
    rng = np.random.default_rng(r)
    U, V = rng.standard_normal((A.n, r + 2)), rng.standard_normal((A.n, r + 1))
    s = rng.standard_normal(r)
    dA = ctx.matrix(A)
    u, v = ctx.multivec(A.n, r + 2, U), ctx.multivec(A.n, r + 1, V)
    rows, cols = AD.pattern(A)
    ref = np.einsum("et,et,t->e", U[rows, 2:2 + r], V[cols, 1:1 + r], s)
    g = G.pattern_grad(dA, u, 2, v, 1, r, s, len(A.val))
    assert rel(g, ref) < 1e-14
    g2 = G.pattern_grad(dA, u, 2, v, 1, r, s, len(A.val), grad=np.ones(len(A.val)))
    assert rel(g2, ref + 1.0) < 1e-14


@pytest.mark.parametrize("generalized,k", [(False, 0), (True, 0), (True, 3)])
def test_eigvec_adjoint_matches_dense(ctx, generalized, k):
    """mu of the GPU solve (explicit components along the m computed eigenvectors,
    CG on their B-complement) equals the dense sum over all n eigenpairs."""
    A, _ = P.varcoef2d(nc=16, seed=21, sigma=0.5)
    B = AD.diag_csr(np.random.default_rng(22).uniform(1.0, 2.0, A.n)) if generalized else None
    w, X = AD.eig_dense(A, B)
    m = 12
    g = np.random.default_rng(23).standard_normal(A.n)
    c = X.T @ g
    a = np.zeros_like(c)
    others = np.arange(A.n) != k
    a[others] = c[others] / (w[others] - w[k])
    mu_ref = X @ a
    dA, dB = ctx.matrix(A), (ctx.matrix(B) if B is not None else None)
    Xd = ctx.multivec(A.n, m, X[:, :m])
    Gd = ctx.multivec(A.n, 1, g)
    MU = ctx.multivec(A.n, 1)
    it = G.eigvec_adjoint(dA, dB, Xd, m, w[:m], k, Gd, 0, MU, 0, tol=1e-13, max_it=4000)
    assert 0 < it < 4000
    mu = MU.download()[:, 0]
    assert rel(mu, mu_ref) < 1e-9
    Bd = B.to_scipy() if B is not None else None
    assert abs(X[:, k] @ (Bd @ mu if Bd is not None else mu)) < 1e-10 * np.linalg.norm(mu)


# ---- the autograd harness
torch = pytest.importorskip("torch")


class GpuEigLoss(torch.autograd.Function):
    """forward(a_vals, b_vals or None) -> (lambda_0..q-1, x_0) of the GPU solve;
    backward: Hellmann-Feynman for the eigenvalues, the adjoint solve for x_0.
    Gradients are returned per stored value of a symmetric pattern as the
    average of the pair (the matrix the solver sees is (M + M^T) / 2)."""

    @staticmethod
    def forward(fctx, a_vals, b_vals, env):
        A, B, q, nev, gctx = env["A"], env["B"], env["q"], env["nev"], env["ctx"]
        dA = gctx.matrix(P.CSR(A.rowptr, A.col, a_vals.detach().numpy()))
        dB = gctx.matrix(P.CSR(B.rowptr, B.col, b_vals.detach().numpy())) if B is not None else None
        params = gctx.params(nev=nev, ev_tol=1e-10, conv_type="BR", ev_max_it=1000, seed=77)
        X = gctx.multivec(A.n, nev)
        ev, Xh, st = gctx.solve(dA, dB, params, evec=X)
        assert st.num_unlock == 0
        fctx.env, fctx.saved = env, (dA, dB, X, ev, Xh)
        return torch.from_numpy(ev[:q].copy()), torch.from_numpy(Xh[:, 0].copy())

    @staticmethod
    def backward(fctx, g_ev, g_x):
        env = fctx.env
        A, B, q, nev, gctx = env["A"], env["B"], env["q"], env["nev"], env["ctx"]
        dA, dB, X, ev, Xh = fctx.saved
        gl = g_ev.numpy().astype(np.float64)
        gx = g_x.numpy().astype(np.float64)
        gA = G.pattern_grad(dA, X, 0, X, 0, q, gl, len(A.val))
        gB = G.pattern_grad(dB, X, 0, X, 0, q, -ev[:q] * gl, len(B.val)) if B is not None else None
        if np.any(gx != 0):
            Gd, MU = gctx.multivec(A.n, 1, gx), gctx.multivec(A.n, 1)
            G.eigvec_adjoint(dA, dB, X, nev, ev, 0, Gd, 0, MU, 0, tol=1e-13, max_it=20000)
            G.pattern_grad(dA, MU, 0, X, 0, 1, [-1.0], len(A.val), grad=gA)
            if B is not None:
                c = float(gx @ Xh[:, 0])
                G.pattern_grad(dB, MU, 0, X, 0, 1, [ev[0]], len(B.val), grad=gB)
                G.pattern_grad(dB, X, 0, X, 0, 1, [-0.5 * c], len(B.val), grad=gB)
        ga = torch.from_numpy(AD.sym_pairs(A, gA))
        gb = torch.from_numpy(AD.sym_pairs(B, gB)) if B is not None else None
        return ga, gb, None


def gpu_loss_grad(ctx, A, B, q, nev, wvec):
    av = torch.tensor(A.val, dtype=torch.float64, requires_grad=True)
    bv = torch.tensor(B.val, dtype=torch.float64, requires_grad=True) if B is not None else None
    env = dict(A=A, B=B, q=q, nev=nev, ctx=ctx)
    ev, x0 = GpuEigLoss.apply(av, bv, env)
    loss = ev.sum() + (torch.from_numpy(wvec) * x0 * x0).sum()
    loss.backward()
    return float(loss.detach()), av.grad.numpy(), (bv.grad.numpy() if bv is not None else None)


def test_loss_gradient_c4_small_instance_vs_dense_autograd(ctx):
    """The 64^2 instance of the variable-coefficient 5-point problem (B = I):
    L = sum of the 20 smallest eigenvalues + sum_r w_r x_1[r]^2; GPU gradient
    against torch autograd through a dense eigh."""
    A, B = P.varcoef2d(nc=64, seed=20240302, sigma=0.5)
    q, nev = 20, 24
    wvec = np.random.default_rng(20240303).uniform(0.0, 1.0, A.n)
    loss_g, gA, _ = gpu_loss_grad(ctx, A, B, q, nev, wvec)
    loss_t, tA, _ = AD.torch_grad(A, B, q, wvec)
    assert abs(loss_g - loss_t) <= 1e-10 * abs(loss_t)
    assert rel(gA, tA) < 1e-7


def test_loss_gradient_generalized_vs_formulas_and_differences(ctx):
    """Generalized pencil (B = diag U[1, 2]): GPU gradient against the dense
    formulas and, on random stored pairs, against central differences of the
    dense loss (h = 1e-6, relative to the largest gradient entry)."""
    A, _ = P.varcoef2d(nc=24, seed=5, sigma=0.5)
    B = AD.diag_csr(np.random.default_rng(6).uniform(1.0, 2.0, A.n))
    q, nev = 6, 10
    wvec = np.random.default_rng(7).uniform(0.0, 1.0, A.n)
    loss_g, gA, gB = gpu_loss_grad(ctx, A, B, q, nev, wvec)
    loss_f, fA, fB, _, _ = AD.formula_grad(A, B, q, wvec)
    assert abs(loss_g - loss_f) <= 1e-10 * abs(loss_f)
    assert rel(gA, AD.sym_pairs(A, fA)) < 1e-7
    assert rel(gB, AD.sym_pairs(B, fB)) < 1e-7
    h = 1e-6
    rng = np.random.default_rng(8)
    for M, g, which in ((A, gA, "A"), (B, gB, "B")):
        t = AD.transpose_index(M)
        scale = np.max(np.abs(2 * g))
        for e in rng.choice(len(M.val), size=6, replace=False):
            def loss_at(delta):
                v = M.val.copy()
                v[e] += delta
                if t[e] != e:
                    v[t[e]] += delta
                Mp = P.CSR(M.rowptr, M.col, v)
                w, X = AD.eig_dense(Mp if which == "A" else A, Mp if which == "B" else B)
                return AD.loss_of(w, X, q, wvec)
            fd = (loss_at(h) - loss_at(-h)) / (2 * h)
            an = 2 * g[e] if t[e] != e else g[e]
            assert abs(fd - an) <= 1e-6 * scale, (which, e, fd, an)
