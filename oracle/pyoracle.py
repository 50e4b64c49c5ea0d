"""ctypes binding for the oracle (test infrastructure only).

``Oracle()`` loads ``oracle/libgcge_oracle.so`` (the C restatement); when the
reference build ``oracle/_ref/libgcge_ref.so`` exists, ``reference()`` returns
a binding with the same ``solve`` signature over the compiled GCGE-1.0.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class Params(C.Structure):
    _fields_ = [
        ("nev", C.c_int), ("block_size", C.c_int), ("ev_max_it", C.c_int), ("cg_max_it", C.c_int),
        ("max_reorth_time", C.c_int), ("dirichlet_boundary", C.c_int), ("given_init_evec", C.c_int),
        ("ev_tol", C.c_double), ("cg_rate", C.c_double), ("orth_zero_tol", C.c_double),
        ("reorth_tol", C.c_double), ("scbgs_reorth_tol", C.c_double), ("criterion_tol", C.c_double),
        ("conv_type", C.c_char * 4), ("init_rng", C.c_int), ("seed", C.c_ulonglong),
        ("print_level", C.c_int), ("w_orth_type", C.c_char * 8), ("orth_type", C.c_char * 4),
        ("opt_rr_eig_partly", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [("num_iter", C.c_int), ("num_unlock", C.c_int), ("max_res", C.c_double),
                ("min_res", C.c_double), ("sum_res", C.c_double), ("wall_s", C.c_double),
                ("status", C.c_int)]


_I = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_D = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _Lib:
    def __init__(self, path, solve_name):
        self.lib = C.CDLL(path)
        self._solve = getattr(self.lib, solve_name)
        self._solve.restype = C.c_int
        self._solve.argtypes = [C.c_int] + [C.c_void_p] * 6 + [C.POINTER(Params), C.c_void_p,
                                                                C.c_void_p, C.POINTER(Stats)]

    def params(self, **kw):
        p = Params()
        self.defaults(p)
        for k, v in kw.items():
            if k in ("conv_type", "w_orth_type", "orth_type"):
                v = v.encode()
            setattr(p, k, v)
        return p

    @staticmethod
    def defaults(p):
        p.nev, p.block_size, p.ev_max_it, p.cg_max_it, p.max_reorth_time = 1, 0, 30, 20, 3
        p.dirichlet_boundary, p.given_init_evec = 0, 0
        p.ev_tol, p.cg_rate, p.orth_zero_tol, p.reorth_tol = 1e-8, 1e-2, 1e-16, 0.75
        p.scbgs_reorth_tol, p.criterion_tol = 1e-16, 1e-6
        p.conv_type, p.init_rng, p.seed, p.print_level = b"R", 0, 1, 0

    def solve(self, A, B, params, evec0=None):
        """Run a full solve; returns (eval[nev], evec[n, nev] column-major as (nev, n).T, stats)."""
        n, nev = A.n, params.nev
        ev = np.zeros(nev)
        X = np.zeros((nev, n))
        if evec0 is not None:
            X[:] = np.asarray(evec0, dtype=np.float64).T
            params.given_init_evec = 1
        st = Stats()
        rc = self._solve(n, _ptr(A.rowptr), _ptr(A.col), _ptr(A.val),
                         _ptr(B.rowptr) if B else None, _ptr(B.col) if B else None,
                         _ptr(B.val) if B else None, C.byref(params), _ptr(ev), _ptr(X), C.byref(st))
        if rc not in (0,):
            raise RuntimeError("solve returned %d" % rc)
        return ev, X.T, st


class Oracle(_Lib):
    def __init__(self):
        path = os.path.join(HERE, "libgcge_oracle.so")
        if not os.path.exists(path):
            import importlib.util
            spec = importlib.util.spec_from_file_location("gcge_oracle_build", os.path.join(HERE, "build_oracle.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        super().__init__(path, "gcge_oracle_solve")
        L = self.lib
        L.gcge_oracle_csr_matmultivec.argtypes = [C.c_int, C.c_int, _I, _I, _D, _D, _D]
        L.gcge_oracle_vec_axpby.argtypes = [C.c_int, C.c_double, _D, C.c_double, _D]
        L.gcge_oracle_multivec_lincomb.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D, C.c_int]
        L.gcge_oracle_multivec_innerprod.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D, C.c_int, C.c_int]
        L.gcge_oracle_bcg.argtypes = [C.c_int, C.c_int, _I, _I, _D, _D, _D, C.c_int, C.c_double]
        L.gcge_oracle_stable_multi_orth.argtypes = [C.c_int, C.c_int, _D, C.c_int, C.c_int, C.c_void_p,
                                                    C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.gcge_oracle_stable_multi_orth.restype = C.c_int
        L.gcge_oracle_hash_uniform.argtypes = [C.c_ulonglong, C.c_ulonglong]
        L.gcge_oracle_hash_uniform.restype = C.c_double
        VP = C.c_void_p
        L.gcge_oracle_solve_table.argtypes = [VP, VP, VP, C.c_int, C.POINTER(Params), VP, VP, C.POINTER(Stats)]
        L.gcge_oracle_solve_table.restype = C.c_int
        L.gcge_oracle_table_bytes.restype = C.c_size_t
        L.gcge_oracle_host_table.argtypes = [VP]
        L.gcge_oracle_csr_handle.argtypes = [C.c_int, VP, VP, VP]
        L.gcge_oracle_csr_handle.restype = VP
        L.gcge_oracle_csr_handle_free.argtypes = [VP]
        L.gcge_oracle_table_mv_create.argtypes = [VP, VP, C.c_int, C.POINTER(VP)]
        L.gcge_oracle_table_mv_create.restype = C.c_int
        L.gcge_oracle_table_mv_destroy.argtypes = [VP, C.POINTER(VP), C.c_int]
        L.gcge_oracle_host_mv_read.argtypes = [VP, C.c_int, C.c_int, VP]
        L.gcge_oracle_dd_rayleigh.argtypes = [C.c_int, _I, _I, _D, _D, VP, _D]
        L.gcge_oracle_dd_residual.argtypes = [C.c_int, _I, _I, _D, _D, VP, C.c_double, C.c_double, _D]
        L.gcge_oracle_dd_add_vec.argtypes = [C.c_int, _D, _D, _D]
        L.gcge_oracle_dd_weighted_sq.argtypes = [C.c_int, _D, _D, VP, _D]

    # ---- double-double checker arithmetic (x = xh + xl; xl may be None)
    @staticmethod
    def _csr(A):
        return (np.ascontiguousarray(A.rowptr, dtype=np.int32), np.ascontiguousarray(A.col, dtype=np.int32),
                np.ascontiguousarray(A.val, dtype=np.float64))

    def dd_rayleigh(self, A, xh, xl=None):
        """(x^T A x) / (x^T x) as a double-double pair (hi, lo)."""
        rp, ci, v = self._csr(A)
        out = np.zeros(2)
        self.lib.gcge_oracle_dd_rayleigh(A.n, rp, ci, v, np.ascontiguousarray(xh, dtype=np.float64),
                                         _ptr(None if xl is None else np.ascontiguousarray(xl)), out)
        return float(out[0]), float(out[1])

    def dd_residual(self, A, xh, xl, theta):
        """A x - theta x (theta a double-double pair), rounded once per entry."""
        rp, ci, v = self._csr(A)
        r = np.zeros(A.n)
        self.lib.gcge_oracle_dd_residual(A.n, rp, ci, v, np.ascontiguousarray(xh, dtype=np.float64),
                                         _ptr(None if xl is None else np.ascontiguousarray(xl)), theta[0],
                                         theta[1], r)
        return r

    def dd_add_vec(self, xh, xl, d):
        """x += d in place (x = xh + xl, both contiguous float64 arrays)."""
        self.lib.gcge_oracle_dd_add_vec(len(xh), xh, xl, np.ascontiguousarray(d, dtype=np.float64))

    def dd_weighted_sq(self, w, xh, xl=None):
        """((sum w x^2) hi, lo, (sum x^2) hi, lo)."""
        out = np.zeros(4)
        self.lib.gcge_oracle_dd_weighted_sq(len(xh), np.ascontiguousarray(w, dtype=np.float64),
                                            np.ascontiguousarray(xh, dtype=np.float64),
                                            _ptr(None if xl is None else np.ascontiguousarray(xl)), out)
        return tuple(float(t) for t in out)

    # ---- GCGE's solver core over a GCGE_OPS table (the drop-in boundary)
    def new_table(self, host=False):
        """A zeroed GCGE_OPS-layout table (host=True: the oracle's host CSR table)."""
        t = C.create_string_buffer(self.lib.gcge_oracle_table_bytes())
        if host:
            self.lib.gcge_oracle_host_table(t)
        return t

    def table_multivec(self, table, mat, k):
        """A k-column multivector made by the table's MultiVecCreateByMat (a void ** handle)."""
        h = C.c_void_p()
        if self.lib.gcge_oracle_table_mv_create(table, mat, k, C.byref(h)) != 0:
            raise RuntimeError("MultiVecCreateByMat failed")
        return h

    def table_multivec_destroy(self, table, h, k):
        self.lib.gcge_oracle_table_mv_destroy(table, C.byref(h), k)

    def solve_table(self, table, A, B, n, params, evec):
        """The GCGE_Solve restatement driven through `table` alone; A, B: the table's
        matrix handles (B may be None), evec: its eigenvector multivector. Returns
        (eval, stats)."""
        ev = np.zeros(params.nev)
        st = Stats()
        rc = self.lib.gcge_oracle_solve_table(table, A, B, n, C.byref(params), _ptr(ev), evec, C.byref(st))
        if rc != 0:
            raise RuntimeError("solve_table returned %d" % rc)
        return ev, st

    # Column-major n x k blocks are held as numpy arrays of shape (k, n) (C order).
    def matmultivec(self, A, X):
        X = np.ascontiguousarray(X, dtype=np.float64)
        Y = np.zeros_like(X)
        self.lib.gcge_oracle_csr_matmultivec(A.n, X.shape[0], A.rowptr, A.col, A.val, X, Y)
        return Y

    def axpby(self, a, x, b, y):
        y = np.array(y, dtype=np.float64)
        self.lib.gcge_oracle_vec_axpby(len(y), a, np.ascontiguousarray(x, dtype=np.float64), b, y)
        return y

    def lincomb(self, X, coef, ny, lda):
        X = np.ascontiguousarray(X, dtype=np.float64)
        Y = np.zeros((ny, X.shape[1]))
        self.lib.gcge_oracle_multivec_lincomb(X.shape[1], X.shape[0], ny, X, Y,
                                              np.ascontiguousarray(coef, dtype=np.float64), lda)
        return Y

    def innerprod(self, V, W, lda, sym):
        V = np.ascontiguousarray(V, dtype=np.float64)
        W = np.ascontiguousarray(W, dtype=np.float64)
        a = np.zeros(lda * W.shape[0])
        self.lib.gcge_oracle_multivec_innerprod(V.shape[1], V.shape[0], W.shape[0], V, W, a, lda, int(sym))
        return a

    def bcg(self, A, RHS, W, cg_max_it=20, cg_rate=1e-2):
        R = np.array(RHS, dtype=np.float64, order="C")
        X = np.array(W, dtype=np.float64, order="C")
        self.lib.gcge_oracle_bcg(A.n, X.shape[0], A.rowptr, A.col, A.val, R, X, cg_max_it, cg_rate)
        return X, R

    def stable_multi_orth(self, V, start, end, B=None, max_reorth_time=3, orth_zero_tol=1e-16,
                          scbgs_reorth_tol=1e-16):
        V = np.array(V, dtype=np.float64, order="C")
        ne = self.lib.gcge_oracle_stable_multi_orth(
            V.shape[1], V.shape[0], V.ctypes.data_as(C.c_void_p), start, end,
            _ptr(B.rowptr) if B else None, _ptr(B.col) if B else None, _ptr(B.val) if B else None,
            max_reorth_time, orth_zero_tol, scbgs_reorth_tol)
        return V, ne

    def hash_uniform(self, seed, index):
        return self.lib.gcge_oracle_hash_uniform(seed, index)


def reference():
    """Binding over the compiled reference (oracle/_ref), or None when it was not built."""
    path = os.path.join(HERE, "_ref", "libgcge_ref.so")
    if not os.path.exists(path):
        return None
    try:
        return _Lib(path, "gcge_ref_solve")
    except OSError:
        return None
