"""ctypes binding of libgcge_gb300.so, the GB300-native GCGE CSR eigensolver.

Every call goes through the C ABI declared in include/gcge_gb300.h. There is no
CPU fallback: if the shared library is missing or no CUDA device is present,
``load()`` / ``Context()`` raise.

Host multivectors are numpy arrays of shape (n, k) (any order); the library
stores them on the device as row-major blocks.
"""
import ctypes as C
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "libgcge_gb300.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_CSR, ERR_NONFINITE, ERR_BREAKDOWN, ERR_EIGSOLVE, ERR_TIMEOUT, ERR_IO = range(1, 10)
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "device allocation failed",
          4: "malformed CSR matrix", 5: "non-finite value", 6: "orthogonalisation lost every column",
          7: "projected eigensolve failed", 8: "tensor-core kernel wait timed out",
          9: "file missing, unreadable, truncated or not CSR"}


class GcgeGpuError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s: status %d (%s)" % (what, status, STATUS.get(status, "?")))


class Params(C.Structure):
    _fields_ = [("nev", C.c_int), ("block_size", C.c_int), ("ev_max_it", C.c_int), ("cg_max_it", C.c_int),
                ("max_reorth_time", C.c_int), ("dirichlet_boundary", C.c_int), ("given_init_evec", C.c_int),
                ("ev_tol", C.c_double), ("cg_rate", C.c_double), ("orth_zero_tol", C.c_double),
                ("conv_type", C.c_char * 4), ("precision", C.c_int), ("seed", C.c_ulonglong),
                ("print_level", C.c_int), ("precond", C.c_int), ("w_orth_type", C.c_char * 8),
                ("opt_rr_eig_partly", C.c_int), ("multi_tol_for_lock", C.c_double), ("orth_type", C.c_char * 4)]


class Stats(C.Structure):
    _fields_ = [("num_iter", C.c_int), ("num_unlock", C.c_int), ("max_res", C.c_double),
                ("min_res", C.c_double), ("sum_res", C.c_double), ("res", C.c_double * 8),
                ("solve_ms", C.c_double), ("phase_ms", C.c_double * 9), ("kernel_launches", C.c_longlong),
                ("spmm_calls", C.c_longlong)]

    PHASES = ("x_axpy", "x_orth", "p_axpy", "p_orth", "w_line", "w_orth", "rr_mat", "rr_eigen", "conv")

    def as_dict(self):
        d = {k: getattr(self, k) for k in ("num_iter", "num_unlock", "max_res", "min_res", "sum_res",
                                           "solve_ms", "kernel_launches", "spmm_calls")}
        d["phase_ms"] = {p: self.phase_ms[i] for i, p in enumerate(self.PHASES)}
        return d


_lib = None
_P = C.c_void_p
_I = C.c_int
_D = C.c_double


def load():
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError("libgcge_gb300.so not built (run __graft_entry__.build()): %s" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    sig = {
        "GCGE_GPU_Init": (_I, [_I, C.POINTER(_P)]),
        "GCGE_GPU_Finalize": (_I, [_P]),
        "GCGE_GPU_GetLastError": (_I, [_P]),
        "GCGE_GPU_ErrorString": (C.c_char_p, [_I]),
        "GCGE_GPU_Synchronize": (_I, [_P]),
        "GCGE_GPU_MatCreate": (_I, [_P, _I, _P, _P, _P, _I, C.POINTER(_P)]),
        "GCGE_GPU_MatSetValues": (_I, [_P, _P]),
        "GCGE_GPU_MatDestroy": (_I, [_P]),
        "GCGE_GPU_MatGetSize": (_I, [_P, C.POINTER(_I), C.POINTER(_I)]),
        "GCGE_GPU_MultiVecCreate": (_I, [_P, _I, _I, C.POINTER(_P)]),
        "GCGE_GPU_MultiVecDestroy": (_I, [_P]),
        "GCGE_GPU_MultiVecUpload": (_I, [_P, _I, _I, _P]),
        "GCGE_GPU_MultiVecDownload": (_I, [_P, _I, _I, _P]),
        "GCGE_GPU_MultiVecSetRandomValue": (_I, [_P, _I, _I, C.c_ulonglong]),
        "GCGE_GPU_MatDotMultiVec": (_I, [_P, _P, _P, _P, _P]),
        "GCGE_GPU_MultiVecAxpby": (_I, [_D, _P, _D, _P, _P, _P]),
        "GCGE_GPU_MultiVecLinearComb": (_I, [_P, _P, _P, _P, _P, _I]),
        "GCGE_GPU_MultiVecInnerProd": (_I, [_P, _P, _P, C.c_char_p, _P, _P, _I]),
        "GCGE_GPU_MultiVecSwap": (_I, [_P, _P, _P, _P]),
        "GCGE_GPU_BCG": (_I, [_P, _P, _I, _P, _I, _I, _I, _D, _I]),
        "GCGE_GPU_Orthonormalize": (_I, [_P, _I, C.POINTER(_I), _P, _I, _D]),
        "GCGE_GPU_OrthonormalizeType": (_I, [_P, _I, C.POINTER(_I), _P, _I, _D, C.c_char_p]),
        "GCGE_GPU_ParamsDefault": (None, [C.POINTER(Params)]),
        "GCGE_GPU_Solve": (_I, [_P, _P, _P, C.POINTER(Params), _P, _P, C.POINTER(Stats)]),
        "GCGE_GPU_SolveHost": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, C.POINTER(Params), _P, _P, C.POINTER(Stats)]),
        "GCGE_GPU_LaunchCount": (C.c_longlong, [_P]),
        "GCGE_GPU_SetOps": (_I, [_P, _P]),
        "GCGE_GPU_OpsSeed": (None, [C.c_ulonglong]),
        "GCGE_GPU_OpsMultiVecBlock": (_I, [_P, C.POINTER(_P), C.POINTER(_I)]),
        "GCGE_GPU_OpsSetLinearSolver": (_I, [_P, _I, _I, _D]),
        "GCGE_GPU_ProfileEnable": (_I, [_P, _I]),
        "GCGE_GPU_ProfileRead": (_I, [_P, _I, _P, _P, _P, _P, _I]),
        "GCGE_GPU_SetTensorEmulation": (_I, [_P, _I]),
        "GCGE_GPU_SetPairSpMM": (_I, [_P, _I]),
        "GCGE_GPU_TestStallTensorWait": (_I, [_P, _I]),
        "GCGE_GPU_InnerProdNoAlloc": (_I, [_I, _I, _I, _P, C.c_long, _P, C.c_long, _P, _I, _I, _P]),
        "GCGE_GPU_PatternGrad": (_I, [_P, _P, _I, _P, _I, _I, _P, _I, _P]),
        "GCGE_GPU_EigvecAdjoint": (_I, [_P, _P, _P, _I, _P, _I, _P, _I, _P, _I, _D, _D, _I, C.POINTER(_I)]),
        "GCGE_GPU_CSRReadText": (_I, [C.c_char_p, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I),
                                      C.POINTER(C.POINTER(_I)), C.POINTER(C.POINTER(_I)),
                                      C.POINTER(C.POINTER(_D))]),
        "GCGE_GPU_CSRReadBinary": (_I, [C.c_char_p, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I),
                                        C.POINTER(C.POINTER(_I)), C.POINTER(C.POINTER(_I)),
                                        C.POINTER(C.POINTER(_D))]),
        "GCGE_GPU_CSRWriteBinary": (_I, [C.c_char_p, _I, _I, _I, _P, _P, _P]),
        "GCGE_GPU_CSRFree": (None, [C.POINTER(_I), C.POINTER(_I), C.POINTER(_D)]),
        "GCGE_GPU_MatCreateFromFile": (_I, [_P, C.c_char_p, _I, C.POINTER(_P)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def declared_symbols():
    """Names of the entry points declared in include/*.h (parsed from the headers)."""
    import re
    inc = os.path.join(os.path.dirname(os.path.dirname(_HERE)), "include")
    names = set()
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"\b(GCGE_GPU_[A-Za-z0-9_]+)\s*\(", txt))
    return sorted(names)


def _chk(st, what):
    if st != OK:
        raise GcgeGpuError(st, what)


def _arr(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _ints(*v):
    return (C.c_int * len(v))(*v)


class Context:
    """One CUDA device and the stream every call is ordered on."""

    def __init__(self, device=0):
        self.lib = load()
        h = _P()
        _chk(self.lib.GCGE_GPU_Init(device, C.byref(h)), "GCGE_GPU_Init")
        self.h = h
        self._children = weakref.WeakSet()

    def _adopt(self, obj):
        self._children.add(obj)
        return obj

    def close(self):
        """Free every matrix and multivector of this context, then the context."""
        if self.h:
            for c in list(self._children):
                c.close()
            self.lib.GCGE_GPU_Finalize(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def sync(self):
        _chk(self.lib.GCGE_GPU_Synchronize(self.h), "sync")

    def tensor_emulation(self, on):
        """Dense FP64 contractions on the tensor cores (error-free splitting) or the FP64 pipe."""
        _chk(self.lib.GCGE_GPU_SetTensorEmulation(self.h, int(on)), "SetTensorEmulation")

    def pair_spmm(self, on):
        """Sparse products with two or more columns in FP32-pair arithmetic (1) or FP64 (0)."""
        _chk(self.lib.GCGE_GPU_SetPairSpMM(self.h, int(on)), "SetPairSpMM")

    def last_error(self):
        return self.lib.GCGE_GPU_GetLastError(self.h)

    def launches(self):
        return self.lib.GCGE_GPU_LaunchCount(self.h)

    PROFILE_CLASSES = ("spmm_fp64", "spmm_fp32", "gram", "lincomb", "bcg_vec", "blas1", "dense_gemm",
                       "dense_eig", "reduce", "spmm_pair")

    def profile(self, on):
        _chk(self.lib.GCGE_GPU_ProfileEnable(self.h, int(on)), "ProfileEnable")

    def profile_read(self, reset=True):
        """Per kernel class: dict(ms, launches, bytes, flops) accumulated while profiling was on."""
        k = len(self.PROFILE_CLASSES)
        ms, nl = np.zeros(k), np.zeros(k, dtype=np.int64)
        by, fl = np.zeros(k), np.zeros(k)
        self.lib.GCGE_GPU_ProfileRead(self.h, k, _ptr(ms), _ptr(nl), _ptr(by), _ptr(fl), int(reset))
        return {c: dict(ms=float(ms[i]), launches=int(nl[i]), bytes=float(by[i]), flops=float(fl[i]))
                for i, c in enumerate(self.PROFILE_CLASSES)}

    # -- data
    def matrix(self, csr, keep_fp32=False):
        return Matrix(self, csr, keep_fp32)

    def matrix_from_file(self, path, keep_fp32=False):
        """Read a CSR file (the reference's text format or the binary form) and upload it."""
        return Matrix(self, None, keep_fp32, path=path)

    def multivec(self, n, k, data=None):
        mv = MultiVec(self, n, k)
        if data is not None:
            mv.upload(data)
        return mv

    # -- solver
    def params(self, **kw):
        p = Params()
        self.lib.GCGE_GPU_ParamsDefault(C.byref(p))
        for k, v in kw.items():
            if k in ("conv_type", "w_orth_type", "orth_type"):
                v = v.encode()
            setattr(p, k, v)
        return p

    def solve(self, A, B, params, evec=None, init=None):
        """Device-resident solve; A, B are Matrix (B may be None). Returns (eval, X (n x nev), stats)."""
        nev = params.nev
        X = evec if evec is not None else MultiVec(self, A.n, nev)
        if init is not None:
            X.upload(init, 0)
            params.given_init_evec = 1
        ev = np.zeros(nev)
        st = Stats()
        _chk(self.lib.GCGE_GPU_Solve(self.h, A.h, B.h if B is not None else None, C.byref(params), _ptr(ev), X.h,
                                     C.byref(st)), "GCGE_GPU_Solve")
        out = X.download(0, nev)
        return ev, out, st

    def solve_host(self, A, B, params, init=None, out=None):
        """Host-buffer entry (uploads, solves, downloads). A, B: problems.CSR.
        out: optional C-contiguous float64 (nev, n) host array (page-locked, say)
        that receives the eigenvectors, one per row."""
        nev = params.nev
        ev = np.zeros(nev)
        if out is not None:
            if out.dtype != np.float64 or out.shape != (nev, A.n) or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("out must be a C-contiguous float64 array of shape (nev, n)")
            X = out
        else:
            X = np.zeros((nev, A.n))
        if init is not None:
            X[:] = np.asarray(init, dtype=np.float64).T
            params.given_init_evec = 1
        st = Stats()
        _chk(self.lib.GCGE_GPU_SolveHost(
            self.h, A.n, _ptr(A.rowptr), _ptr(A.col), _ptr(A.val),
            _ptr(B.rowptr) if B is not None else None, _ptr(B.col) if B is not None else None,
            _ptr(B.val) if B is not None else None, C.byref(params), _ptr(ev), _ptr(X), C.byref(st)),
            "GCGE_GPU_SolveHost")
        return ev, X.T, st


class Matrix:
    def __init__(self, ctx, csr, keep_fp32=False, path=None):
        self.ctx, self.lib = ctx, ctx.lib
        if path is not None:
            # read and upload in the library (GCGE_GPU_MatCreateFromFile): text or binary
            h = _P()
            _chk(self.lib.GCGE_GPU_MatCreateFromFile(ctx.h, os.fsencode(path), int(keep_fp32), C.byref(h)),
                 "GCGE_GPU_MatCreateFromFile")
            self.h = h
            n, nnz = _I(), _I()
            _chk(self.lib.GCGE_GPU_MatGetSize(h, C.byref(n), C.byref(nnz)), "GCGE_GPU_MatGetSize")
            self.n = n.value
            ctx._adopt(self)
            return
        self.n = csr.n
        self._rp, self._ci, self._v = _arr(csr.rowptr, np.int32), _arr(csr.col, np.int32), _arr(csr.val, np.float64)
        h = _P()
        _chk(self.lib.GCGE_GPU_MatCreate(ctx.h, self.n, _ptr(self._rp), _ptr(self._ci), _ptr(self._v),
                                         int(keep_fp32), C.byref(h)), "GCGE_GPU_MatCreate")
        self.h = h
        ctx._adopt(self)

    def set_values(self, val):
        v = _arr(val, np.float64)
        _chk(self.lib.GCGE_GPU_MatSetValues(self.h, _ptr(v)), "GCGE_GPU_MatSetValues")

    def close(self):
        if self.h and self.ctx.h:
            self.lib.GCGE_GPU_MatDestroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiVec:
    def __init__(self, ctx, n, k):
        self.ctx, self.lib, self.n, self.k = ctx, ctx.lib, n, k
        h = _P()
        _chk(self.lib.GCGE_GPU_MultiVecCreate(ctx.h, n, k, C.byref(h)), "GCGE_GPU_MultiVecCreate")
        self.h = h
        ctx._adopt(self)

    def upload(self, X, col0=0):
        X = np.asarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X[:, None]
        cm = np.ascontiguousarray(X.T)  # column-major n x k
        _chk(self.lib.GCGE_GPU_MultiVecUpload(self.h, col0, X.shape[1], _ptr(cm)), "upload")

    def download(self, col0=0, k=None):
        k = self.k - col0 if k is None else k
        cm = np.zeros((k, self.n))
        _chk(self.lib.GCGE_GPU_MultiVecDownload(self.h, col0, k, _ptr(cm)), "download")
        return cm.T

    def random(self, start, nvec, seed):
        _chk(self.lib.GCGE_GPU_MultiVecSetRandomValue(self.h, start, nvec, seed), "random")

    def close(self):
        if self.h and self.ctx.h:
            self.lib.GCGE_GPU_MultiVecDestroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- block operations (semantics of GCGE_OPS members)
def mat_dot_multivec(A, x, y, start, end):
    _chk(A.lib.GCGE_GPU_MatDotMultiVec(A.h, x.h, y.h, _ints(*start), _ints(*end)), "MatDotMultiVec")


def multivec_axpby(a, x, b, y, start, end):
    _chk(x.lib.GCGE_GPU_MultiVecAxpby(a, x.h, b, y.h, _ints(*start), _ints(*end)), "MultiVecAxpby")


def multivec_linear_comb(x, y, start, end, a, lda):
    a = _arr(a, np.float64)
    _chk(x.lib.GCGE_GPU_MultiVecLinearComb(x.h, y.h, _ints(*start), _ints(*end), _ptr(a), lda), "LinearComb")


def multivec_inner_prod(V, W, start, end, lda, sym=False, out=None):
    k2 = end[1] - start[1]
    a = np.zeros(lda * k2) if out is None else out
    _chk(V.lib.GCGE_GPU_MultiVecInnerProd(V.h, W.h, _ptr(a), b"sym" if sym else b"nonsym", _ints(*start),
                                          _ints(*end), lda), "InnerProd")
    return a


def multivec_swap(V1, V2, start, end):
    _chk(V1.lib.GCGE_GPU_MultiVecSwap(V1.h, V2.h, _ints(*start), _ints(*end)), "Swap")


def bcg(A, RHS, r_start, W, w_start, k, cg_max_it=20, cg_rate=1e-2, precision=0):
    _chk(A.lib.GCGE_GPU_BCG(A.h, RHS.h, r_start, W.h, w_start, k, cg_max_it, cg_rate, precision), "BCG")


# ---- differentiation (adjoint kernels)
def pattern_grad(M, U, u0, V, v0, r, scale, nnz, grad=None):
    """grad[e] (+)= sum_t scale[t] U[i, u0+t] V[j, v0+t] over the stored entries
    e = (i, j) of M (CSR order); with grad given, the sums are added to it."""
    sc = _arr(scale, np.float64)
    acc = grad is not None
    g = np.zeros(nnz) if grad is None else grad
    _chk(M.lib.GCGE_GPU_PatternGrad(M.h, U.h, u0, V.h, v0, r, _ptr(sc), int(acc), _ptr(g)), "PatternGrad")
    return g


def eigvec_adjoint(A, B, X, m, eval_, k, G, g_col, MU, mu_col, cluster_tol=1e-10, tol=1e-12, max_it=2000):
    """mu (column mu_col of MU) of the eigenvector functional adjoint; returns the CG iterations."""
    ev = _arr(eval_, np.float64)
    it = C.c_int(0)
    _chk(A.lib.GCGE_GPU_EigvecAdjoint(A.h, B.h if B is not None else None, X.h, m, _ptr(ev), k, G.h, g_col, MU.h,
                                      mu_col, cluster_tol, tol, max_it, C.byref(it)), "EigvecAdjoint")
    return it.value


def orthonormalize(W, start, end, B=None, max_reorth_time=3, orth_zero_tol=1e-16, w_orth_type=None):
    e = C.c_int(end)
    if w_orth_type is None:
        _chk(W.lib.GCGE_GPU_Orthonormalize(W.h, start, C.byref(e), B.h if B is not None else None, max_reorth_time,
                                           orth_zero_tol), "Orthonormalize")
    else:
        _chk(W.lib.GCGE_GPU_OrthonormalizeType(W.h, start, C.byref(e), B.h if B is not None else None,
                                               max_reorth_time, orth_zero_tol, w_orth_type.encode()),
             "OrthonormalizeType")
    return e.value


def read_csr(path, binary=False):
    """A CSR file read by the library (GCGE_GPU_CSRReadText / CSRReadBinary), as problems.CSR."""
    from .problems import CSR
    L = load()
    nr, nc, nz = _I(), _I(), _I()
    rp, ci, v = C.POINTER(_I)(), C.POINTER(_I)(), C.POINTER(_D)()
    f = L.GCGE_GPU_CSRReadBinary if binary else L.GCGE_GPU_CSRReadText
    _chk(f(os.fsencode(path), C.byref(nr), C.byref(nc), C.byref(nz), C.byref(rp), C.byref(ci), C.byref(v)),
         "GCGE_GPU_CSRRead")
    try:
        rowptr = np.ctypeslib.as_array(rp, shape=(nr.value + 1,)).astype(np.int64)
        col = np.ctypeslib.as_array(ci, shape=(max(nz.value, 1),))[:nz.value].astype(np.int64)
        val = np.ctypeslib.as_array(v, shape=(max(nz.value, 1),))[:nz.value].copy()
    finally:
        L.GCGE_GPU_CSRFree(rp, ci, v)
    if nr.value != nc.value:
        raise ValueError("square matrices only (%d x %d)" % (nr.value, nc.value))
    return CSR(rowptr, col, val)


def write_csr_binary(path, csr):
    """Write the binary CSR form (GCGE_GPU_CSRWriteBinary)."""
    L = load()
    rp, ci, v = _arr(csr.rowptr, np.int32), _arr(csr.col, np.int32), _arr(csr.val, np.float64)
    _chk(L.GCGE_GPU_CSRWriteBinary(os.fsencode(path), csr.n, csr.n, len(v), _ptr(rp), _ptr(ci), _ptr(v)),
         "GCGE_GPU_CSRWriteBinary")
