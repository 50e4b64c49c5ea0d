"""The eigenpair adjoint formulas that the GPU kernels implement, checked on the CPU
against torch autograd through a dense eigensolver and against central finite
differences (no GPU)."""
import numpy as np
import pytest

from gcge_gb300 import problems as P
import adjoint_dense as AD

torch = pytest.importorskip("torch")


def small_pencil(generalized, nc=10, seed=3):
    A, _ = P.varcoef2d(nc=nc, seed=seed, sigma=0.5)
    B = None
    if generalized:
        rng = np.random.default_rng(seed + 1)
        B = AD.diag_csr(rng.uniform(1.0, 2.0, A.n))
    return A, B


@pytest.mark.parametrize("generalized", [False, True])
def test_formulas_match_autograd(generalized):
    A, B = small_pencil(generalized)
    q = 4
    wvec = np.random.default_rng(7).uniform(0.0, 1.0, A.n)
    loss_f, gA, gB, _, _ = AD.formula_grad(A, B, q, wvec)
    loss_t, tA, tB = AD.torch_grad(A, B, q, wvec)
    assert abs(loss_f - loss_t) <= 1e-12 * abs(loss_t)
    sA = AD.sym_pairs(A, gA)
    np.testing.assert_allclose(sA, tA, rtol=0, atol=1e-9 * np.max(np.abs(tA)))
    if generalized:
        np.testing.assert_allclose(AD.sym_pairs(B, gB), tB, rtol=0, atol=1e-9 * np.max(np.abs(tB)))


@pytest.mark.parametrize("h,per_entry", [(1e-6, False), (1e-4, True)])
def test_formulas_match_central_differences(h, per_entry):
    """A symmetric perturbation of a stored pair (i, j), (j, i) by h changes L by
    h (g_ij + g_ji). Central differences agree to 1e-6: relative to the largest
    gradient entry at h = 1e-6 (round-off of the O(1) loss, 1e-16 / h, dominates
    there), per entry at h = 1e-4 (truncation O(h^2))."""
    A, B = small_pencil(True, nc=8, seed=11)
    q = 3
    wvec = np.random.default_rng(5).uniform(0.0, 1.0, A.n)
    _, gA, gB, _, _ = AD.formula_grad(A, B, q, wvec)
    tA, tB = AD.transpose_index(A), AD.transpose_index(B)
    rng = np.random.default_rng(9)
    for M, g, t, which in ((A, gA, tA, "A"), (B, gB, tB, "B")):
        scale = np.max(np.abs(g + g[t]))
        for e in rng.choice(len(M.val), size=8, replace=False):
            def loss_at(delta):
                v = M.val.copy()
                v[e] += delta
                if t[e] != e:
                    v[t[e]] += delta
                Mp = P.CSR(M.rowptr, M.col, v)
                w, X = AD.eig_dense(Mp if which == "A" else A, Mp if which == "B" else B)
                return AD.loss_of(w, X, q, wvec)
            fd = (loss_at(h) - loss_at(-h)) / (2 * h)
            an = g[e] + (g[t[e]] if t[e] != e else 0.0)
            ref = abs(an) if per_entry else scale
            assert abs(fd - an) <= 1e-6 * ref, (which, e, fd, an)
