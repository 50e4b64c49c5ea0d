"""The gradient of the C4 loss against central finite differences on the full
512^2 instance (n = 262,144).

Problem: 5-point variable-coefficient Laplacian on 512^2 cells with log-normal
coefficients (sigma 0.5, seeded), B = I; loss L = sum of the 20 smallest
eigenvalues + sum_r w_r x_1[r]^2, w ~ U[0, 1] seeded. Variables: 64 seeded random
stored entries of A, each taken as a symmetric parameter (the entry and its
transpose move together), so its gradient is the sum of the two stored entries'
gradients. The gradient comes from this library's adjoint entry points
(Hellmann-Feynman on the pattern, the eigenvector adjoint solve); the
differences are (L(a + h) - L(a - h)) / 2h with h = 1e-6.

A difference of two FP64 losses would carry their rounding error divided by 2h
(~1e-10 relative in an eigenvalue, ~1e-11 in the eigenvector term, against
changes of ~1e-8), so each perturbed loss is evaluated beyond one FP64
rounding: an FP64 GPU solve of the perturbed problem from the seeded initial
vectors (residual <= 1e-9, mixed form: FP32 Jacobi-preconditioned inner
solve, every outer product FP64), its 20
eigenvalues as Rayleigh quotients in double-double arithmetic (error quadratic
in the residual: ~1e-22 here), and x_1 refined by one correction step
(residual in double-double, the shifted system solved on the GPU by the
eigenvector adjoint solve) with its double-double residual checked, the
eigenvector term summed in double-double; the difference is taken in exact
rational arithmetic. The base eigenpair x_1 that the adjoint uses is refined
the same way. Bar: |FD - adjoint| <= 1e-6 |adjoint| on every sampled entry."""
from fractions import Fraction as F

import numpy as np
import pytest

import gcge_gb300 as G
import pyoracle
from gcge_gb300 import problems as P
import adjoint_dense as AD

pytestmark = pytest.mark.gpu


def test_c4_gradient_matches_central_differences_512():
    A, _ = P.varcoef2d(nc=512, seed=20240302, sigma=0.5)
    n, nnz = A.n, len(A.val)
    q, nev, h = 20, 24, 1e-6
    wvec = np.random.default_rng(20240303).uniform(0.0, 1.0, n)
    o = pyoracle.Oracle()
    ctx = G.Context(0)
    try:
        dA = ctx.matrix(A, keep_fp32=True)
        X = ctx.multivec(n, nev)
        R, D = ctx.multivec(n, 1), ctx.multivec(n, 1)
        base = dict(nev=nev, ev_tol=1e-9, conv_type="BR", ev_max_it=3000, seed=77, precision=1, precond=1)

        def refine_x1(Ap, Xd, ev):
            """x_1 + the correction of one step on (A' - theta) d = -r, x_1^T d = 0,
            as a double-double vector (xh, xl), with its residual checked."""
            xh, xl = np.ascontiguousarray(Xd.download(0, 1)[:, 0]), np.zeros(n)
            th = o.dd_rayleigh(Ap, xh, xl)
            R.upload(-o.dd_residual(Ap, xh, xl, th))
            evs = ev.copy()
            evs[0] = th[0]
            G.eigvec_adjoint(dA, None, Xd, nev, evs, 0, R, 0, D, 0, tol=1e-10, max_it=40000)
            o.dd_add_vec(xh, xl, D.download()[:, 0])
            th2 = o.dd_rayleigh(Ap, xh, xl)
            r2 = o.dd_residual(Ap, xh, xl, th2)
            # residual far below the eigenvector term's resolution: an x_1 error of e
            # moves the term by ~e, the differences resolve ~1e-14
            assert np.linalg.norm(r2) <= 1e-14 * abs(th2[0]) * np.linalg.norm(xh), np.linalg.norm(r2)
            return xh, xl

        ev, Xh, st = ctx.solve(dA, None, ctx.params(**base), evec=X)
        assert st.num_unlock == 0
        x1h, x1l = refine_x1(A, X, ev)
        # ---- the adjoint gradient over every stored entry
        gA = G.pattern_grad(dA, X, 0, X, 0, q, np.ones(q), nnz)
        x1 = x1h + x1l
        Gd, MU = ctx.multivec(n, 1, 2.0 * wvec * x1 / np.linalg.norm(x1) ** 2), ctx.multivec(n, 1)
        G.eigvec_adjoint(dA, None, X, nev, ev, 0, Gd, 0, MU, 0, tol=1e-12, max_it=40000)
        G.pattern_grad(dA, MU, 0, X, 0, 1, [-1.0], nnz, grad=gA)
        t = AD.transpose_index(A)
        # ---- the loss of a perturbed problem, beyond one FP64 rounding
        Xp = ctx.multivec(n, nev)

        def loss(vals):
            dA.set_values(vals)
            Ap = P.CSR(A.rowptr, A.col, vals)
            evp, Xph, stp = ctx.solve(dA, None, ctx.params(**base), evec=Xp)
            assert stp.num_unlock == 0
            L = F(0)
            for k in range(q):
                hi, lo = o.dd_rayleigh(Ap, Xph[:, k])
                L += F(hi) + F(lo)
            xh, xl = refine_x1(Ap, Xp, evp)
            s = o.dd_weighted_sq(wvec, xh, xl)
            return L + (F(s[0]) + F(s[1])) / (F(s[2]) + F(s[3])), stp.num_iter

        rng = np.random.default_rng(20240304)
        entries = rng.choice(nnz, size=64, replace=False)
        errs, iters = [], []
        for e in entries:
            an = gA[e] + gA[t[e]] if t[e] != e else gA[e]
            lp, ip = loss(_shift(A.val, e, t[e], h))
            lm, im = loss(_shift(A.val, e, t[e], -h))
            fd = float((lp - lm) / (2 * F(h)))
            errs.append((abs(fd - an) / abs(an), e, fd, an))
            iters += [ip, im]
        dA.set_values(A.val)
    finally:
        ctx.close()
    worst = max(errs)
    print("FD vs adjoint on %d entries: max rel %.3e (entry %d: fd %.12e adjoint %.12e); median rel %.3e; "
          "perturbed solves %d-%d iterations" % (len(errs), worst[0], worst[1], worst[2], worst[3],
                                                     float(np.median([x[0] for x in errs])), min(iters),
                                                     max(iters)))
    assert worst[0] <= 1e-6, worst


def _shift(val, e, te, d):
    v = val.copy()
    v[e] += d
    if te != e:
        v[te] += d
    return v
