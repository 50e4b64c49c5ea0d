"""Dense FP64 reference of the eigenpair adjoints (test infrastructure only).

The GPU adjoint entry points compute gradients of a function of computed
eigenpairs of A x = lambda B x with respect to the stored CSR entries of A and B.
This module evaluates the same gradients two independent ways on small dense
problems:

* ``formula_grad``: the first-order perturbation formulas with a full dense
  eigendecomposition (scipy.linalg.eigh, B-orthonormal eigenvectors),
      d lambda / d A_ij = x_i x_j,   d lambda / d B_ij = -lambda x_i x_j,
      d L(x) / d A_ij = -mu_i x_j,   d L(x) / d B_ij = lambda mu_i x_j - (g.x / 2) x_i x_j,
  mu = sum_{j != k} x_j (x_j . g) / (lambda_j - lambda_k), g = dL/dx;
* ``torch_grad``: torch autograd through torch.linalg.eigh of the Cholesky-
  reduced pencil built from the CSR values.

Each stored entry is one variable; ``sym_pairs`` averages the gradients of the
two stored entries of an off-diagonal pair, the gradient that autograd returns
when the dense matrix is built as (M + M^T) / 2 from the values.
"""
import numpy as np
import scipy.linalg as sl


def pattern(csr):
    rows = np.repeat(np.arange(csr.n), np.diff(csr.rowptr))
    return rows, csr.col.astype(np.int64)


def transpose_index(csr):
    """For each stored entry (i, j), the position of the stored entry (j, i)."""
    rows, cols = pattern(csr)
    key = rows * csr.n + cols
    tkey = cols * csr.n + rows
    order = np.argsort(key)
    pos = np.searchsorted(key[order], tkey)
    t = order[pos]
    assert np.array_equal(key[t], tkey), "pattern is not symmetric"
    return t


def sym_pairs(csr, g):
    return 0.5 * (g + g[transpose_index(csr)])


def eig_dense(A, B):
    Ad = A.to_scipy().toarray()
    Bd = B.to_scipy().toarray() if B is not None else np.eye(A.n)
    return sl.eigh(Ad, Bd)


def loss_of(w, X, q, wvec):
    """L = sum of the q smallest eigenvalues + sum_r wvec_r x_1[r]^2."""
    return float(np.sum(w[:q]) + wvec @ (X[:, 0] ** 2))


def formula_grad(A, B, q, wvec):
    """Loss and per-entry gradients (gA, gB or None) by the perturbation formulas."""
    w, X = eig_dense(A, B)
    lam, x = w[0], X[:, 0]
    g = 2.0 * wvec * x
    c = X.T @ g
    a = np.zeros_like(c)
    a[1:] = c[1:] / (w[1:] - lam)
    mu = X @ a
    ra, ca = pattern(A)
    gA = np.einsum("ei,ei->e", X[ra, :q], X[ca, :q]) - mu[ra] * x[ca]
    gB = None
    if B is not None:
        rb, cb = pattern(B)
        gB = (-np.einsum("ei,ei,i->e", X[rb, :q], X[cb, :q], w[:q]) + lam * mu[rb] * x[cb]
              - 0.5 * (g @ x) * x[rb] * x[cb])
    return loss_of(w, X, q, wvec), gA, gB, mu, (w, X)


def torch_grad(A, B, q, wvec):
    """Loss and gradients with respect to the CSR values by torch autograd."""
    import torch
    dt = torch.float64

    def dense(csr, vals):
        rows, cols = pattern(csr)
        M = torch.zeros((csr.n, csr.n), dtype=dt)
        M = M.index_put((torch.from_numpy(rows), torch.from_numpy(cols)), vals, accumulate=True)
        return 0.5 * (M + M.T)

    av = torch.tensor(A.val, dtype=dt, requires_grad=True)
    As = dense(A, av)
    if B is not None:
        bv = torch.tensor(B.val, dtype=dt, requires_grad=True)
        L = torch.linalg.cholesky(dense(B, bv))
        Cm = torch.linalg.solve_triangular(L, torch.linalg.solve_triangular(L, As, upper=False).T, upper=False).T
    else:
        bv, L, Cm = None, None, As
    e, Y = torch.linalg.eigh(0.5 * (Cm + Cm.T))
    x = Y[:, 0] if L is None else torch.linalg.solve_triangular(L.T, Y[:, :1], upper=True)[:, 0]
    loss = e[:q].sum() + (torch.from_numpy(wvec) * x * x).sum()
    loss.backward()
    return float(loss.detach()), av.grad.numpy(), (bv.grad.numpy() if bv is not None else None)


def diag_csr(vals):
    from gcge_gb300 import problems as P
    n = len(vals)
    return P.CSR(np.arange(n + 1), np.arange(n), np.asarray(vals, dtype=np.float64))
