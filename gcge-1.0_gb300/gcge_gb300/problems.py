"""Seeded synthetic CSR pencils (A, B) for the GCGE eigensolver workloads.

Every generator returns CSR arrays in the reference's CSR layout
(``RowPtr[n+1]``, ``KCol[nnz]``, ``Entries[nnz]``; app/csr/gcge_app_csr.h:27-40):
int32 row pointers and column indices (sorted within a row) and float64 values.
B is ``None`` for the standard problem (B = I).

Workloads (all randomness from one documented numpy PCG64 seed each):

* ``laplace2d(100, 100)``            2-D 5-point Dirichlet Laplacian, diag 4 / off -1.
* ``fem_q1_cube(96)``                Q1 trilinear stiffness + consistent mass on the unit
                                     cube, 96^3 elements, Dirichlet by elimination
                                     (95^3 = 857,375 interior nodes, 27-point stencil).
* ``varcoef3d(160, seed)``           7-point variable-coefficient diffusion, face coefficient
                                     = harmonic mean of exp(g), g a Gaussian random field
                                     (sigma 1, correlation length 8 cells); B = diag U[1,2].
* ``varcoef2d(512, seed)``           5-point variable-coefficient Laplacian with log-normal
                                     coefficients (sigma 0.5); B = I.
* ``powerlaw_graph(2_000_000, seed)`` weighted graph Laplacian + 1e-3 I of a configuration-
                                     model graph with power-law degrees; B = diag U[1,2].
"""
import numpy as np
import scipy.sparse as sp


class CSR:
    """A CSR matrix in the reference's layout (int32 indices, float64 values)."""

    def __init__(self, rowptr, col, val):
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self.n = len(self.rowptr) - 1
        self.nnz = len(self.col)

    @classmethod
    def from_scipy(cls, m):
        m = sp.csr_matrix(m)
        m.sum_duplicates()
        m.sort_indices()
        return cls(m.indptr, m.indices, m.data)

    def to_scipy(self):
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=(self.n, self.n))

    def check(self):
        """Host-side structural checks (monotone row pointers, column range)."""
        rp = self.rowptr
        if rp[0] != 0 or rp[-1] != self.nnz or np.any(np.diff(rp) < 0):
            raise ValueError("CSR row pointers are not monotone")
        if self.nnz and (self.col.min() < 0 or self.col.max() >= self.n):
            raise ValueError("CSR column index out of range")
        return self


def _tridiag(n, lo, mid, hi):
    return sp.diags([np.full(n - 1, lo), np.full(n, mid), np.full(n - 1, hi)], [-1, 0, 1], format="csr")


def laplace2d(nx=100, ny=100):
    """5-point Laplacian, diagonal 4, off-diagonals -1 (unit spacing), B = I."""
    Tx = _tridiag(nx, -1.0, 2.0, -1.0)
    Ty = _tridiag(ny, -1.0, 2.0, -1.0)
    A = sp.kron(sp.identity(ny), Tx) + sp.kron(Ty, sp.identity(nx))
    return CSR.from_scipy(A), None


def laplace2d_eigs(nx, ny, k):
    """The k smallest eigenvalues 4 - 2cos(i pi/(nx+1)) - 2cos(j pi/(ny+1))."""
    ix = 2.0 - 2.0 * np.cos(np.arange(1, nx + 1) * np.pi / (nx + 1))
    iy = 2.0 - 2.0 * np.cos(np.arange(1, ny + 1) * np.pi / (ny + 1))
    return np.sort((ix[:, None] + iy[None, :]).ravel())[:k]


def fem_q1_cube(ne=96):
    """Q1 stiffness A and consistent mass B on the unit cube with ne^3 elements.

    With trilinear elements on a uniform mesh the element matrices factor as
    tensor products of the 1-D linear element, so the assembled interior-node
    matrices are A = K(x)M(x)M + M(x)K(x)M + M(x)M(x)K and B = M(x)M(x)M with
    K = tridiag(-1, 2, -1)/h and M = tridiag(1, 4, 1) h/6 on the ne-1 interior
    nodes per direction (Dirichlet by elimination). 2x2x2 Gauss quadrature is
    exact for these element integrals, so this equals the quadrature assembly.
    """
    N = ne - 1
    h = 1.0 / ne
    K = _tridiag(N, -1.0 / h, 2.0 / h, -1.0 / h)
    M = _tridiag(N, h / 6.0, 4.0 * h / 6.0, h / 6.0)
    A = sp.kron(sp.kron(K, M), M) + sp.kron(sp.kron(M, K), M) + sp.kron(sp.kron(M, M), K)
    B = sp.kron(sp.kron(M, M), M)
    return CSR.from_scipy(A), CSR.from_scipy(B)


def fem_q1_cube_eigs(ne, k):
    """Exact generalized eigenvalues of fem_q1_cube(ne): sums of three 1-D ratios."""
    N = ne - 1
    h = 1.0 / ne
    th = np.arange(1, N + 1) * np.pi / ne
    mu = 6.0 * (2.0 - 2.0 * np.cos(th)) / (h * h * (4.0 + 2.0 * np.cos(th)))
    m = np.sort(mu)[: min(N, k + 2)]
    s = (m[:, None, None] + m[None, :, None] + m[None, None, :]).ravel()
    return np.sort(s)[:k]


def _gaussian_field(shape, corr_len, rng):
    """Unit-variance Gaussian random field: white noise filtered by a Gaussian
    kernel of correlation length ``corr_len`` cells (FFT convolution)."""
    w = rng.standard_normal(shape)
    F = np.fft.rfftn(w)
    freqs = np.meshgrid(*[np.fft.fftfreq(s) for s in shape[:-1]], np.fft.rfftfreq(shape[-1]),
                        indexing="ij")
    k2 = sum(f * f for f in freqs)
    F *= np.exp(-0.5 * (2.0 * np.pi) ** 2 * k2 * corr_len * corr_len)
    g = np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))
    g -= g.mean()
    g /= g.std()
    return g


def _diffusion_from_cells(kc):
    """Cell-centred finite-volume diffusion matrix on a grid of cell coefficients kc.
    Interior faces use the harmonic mean 2 k1 k2 / (k1 + k2); boundary faces (Dirichlet
    wall half a cell away) use 2 k. Unit cell size."""
    shape = kc.shape
    n = kc.size
    idx = np.arange(n).reshape(shape)
    rows, cols, vals = [], [], []
    diag = np.zeros(shape)
    for ax in range(kc.ndim):
        a = [slice(None)] * kc.ndim
        b = [slice(None)] * kc.ndim
        a[ax] = slice(0, -1)
        b[ax] = slice(1, None)
        k1, k2 = kc[tuple(a)], kc[tuple(b)]
        f = 2.0 * k1 * k2 / (k1 + k2)
        i1, i2 = idx[tuple(a)].ravel(), idx[tuple(b)].ravel()
        rows += [i1, i2]
        cols += [i2, i1]
        vals += [-f.ravel(), -f.ravel()]
        diag[tuple(a)] += f
        diag[tuple(b)] += f
        lo = [slice(None)] * kc.ndim
        hi = [slice(None)] * kc.ndim
        lo[ax] = slice(0, 1)
        hi[ax] = slice(-1, None)
        diag[tuple(lo)] += 2.0 * kc[tuple(lo)]
        diag[tuple(hi)] += 2.0 * kc[tuple(hi)]
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.ravel())
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    return CSR.from_scipy(A)


def varcoef3d(nc=160, seed=20240301):
    """7-point diffusion on nc^3 cells, k = exp(g) with g a unit Gaussian field of
    correlation length 8 cells; B = lumped diagonal mass U[1, 2]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = _gaussian_field((nc, nc, nc), 8.0, rng)
    A = _diffusion_from_cells(np.exp(g))
    n = A.n
    B = CSR(np.arange(n + 1), np.arange(n), rng.uniform(1.0, 2.0, n))
    return A, B


def varcoef2d(nc=512, seed=20240302, sigma=0.5):
    """5-point variable-coefficient Laplacian on nc^2 cells, log-normal cell
    coefficients k = exp(sigma * xi), xi standard normal; B = I."""
    rng = np.random.Generator(np.random.PCG64(seed))
    k = np.exp(sigma * rng.standard_normal((nc, nc)))
    return _diffusion_from_cells(k), None


def powerlaw_graph(n=2_000_000, seed=20240305, exponent=2.5, dmin=4, dmax=2000, shift=1e-3):
    """Weighted graph Laplacian + shift*I of a configuration-model graph whose degrees follow
    a truncated power law; self-loops and repeated edges are dropped (the realised nnz is what
    it is). Edge weights U[0.5, 1.5]; B = diag U[1, 2]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = np.arange(dmin, dmax + 1, dtype=np.float64)
    p = d ** (-exponent)
    p /= p.sum()
    deg = rng.choice(np.arange(dmin, dmax + 1), size=n, p=p)
    if deg.sum() % 2:
        deg[0] += 1
    stubs = np.repeat(np.arange(n, dtype=np.int64), deg)
    rng.shuffle(stubs)
    u, v = stubs[0::2], stubs[1::2]
    keep = u != v
    u, v = u[keep], v[keep]
    lo, hi = np.minimum(u, v), np.maximum(u, v)
    key = np.unique(lo * n + hi)
    lo, hi = key // n, key % n
    w = rng.uniform(0.5, 1.5, len(lo))
    W = sp.coo_matrix((np.concatenate([w, w]), (np.concatenate([lo, hi]), np.concatenate([hi, lo]))),
                      shape=(n, n)).tocsr()
    L = sp.diags(np.asarray(W.sum(axis=1)).ravel() + shift) - W
    B = CSR(np.arange(n + 1), np.arange(n), rng.uniform(1.0, 2.0, n))
    return CSR.from_scipy(L), B


def read_csr_text(path):
    """Reader for the reference's text CSR format (app/csr/gcge_app_csr.c:185-236):
    nrow, ncol, nnz, then RowPtr[nrow+1], KCol[nnz], Entries[nnz], one per line."""
    with open(path) as f:
        tok = f.read().split()
    nrow, ncol, nnz = int(tok[0]), int(tok[1]), int(tok[2])
    if nrow != ncol:
        raise ValueError("square matrices only")
    o = 3
    rp = np.array(tok[o:o + nrow + 1], dtype=np.int64)
    o += nrow + 1
    ci = np.array(tok[o:o + nnz], dtype=np.int64)
    o += nnz
    v = np.array(tok[o:o + nnz], dtype=np.float64)
    return CSR(rp, ci, v)
