"""The drop-in boundary end to end: GCGE's solver core over the GB300 table.

GCGE_GPU_SetOps fills a GCGE_OPS table (src/gcge_ops.h:29-215) with device
implementations; GCGE's own solver core then runs unchanged. The reference core
is compiled C for the build machine only, so its restatement (the oracle, which
is bit-identical to it on the CPU: test_oracle_golden.py, test_oracle_table.py)
plays GCGE_SOLVER_Solve here: every n-sized operation of the solve - the CSR
products, the vector and multivector updates, inner products, swaps, the
Dirichlet zeroing, the initial random vectors - and the projected eigensolve go
through the table's function pointers to this library's kernels, with the
matrices uploaded by GCGE_GPU_MatCreate and the eigenvector multivector made by
the table's MultiVecCreateByMat, as GCGE_CSR_Solver_Init does
(app/csr/gcge_app_csr.c:92-124). The eigenvalues must match what the reference
reported on the same problems (golden.json) to 1e-10 and every residual must
meet the case's own criterion.
"""
import ctypes as C

import numpy as np
import pytest

import gcge_gb300 as G
import pyoracle
from _golden import case_matrices, golden

pytestmark = pytest.mark.gpu
GOLD = golden()


def residuals(A, B, ev, X, conv_type):
    As = A.to_scipy()
    AX = As @ X
    BX = B.to_scipy() @ X if B is not None else X
    rn = np.linalg.norm(AX - BX * ev[None, :], axis=0)
    xn = np.linalg.norm(X, axis=0)
    if conv_type == "R":
        return rn / xn / np.maximum(1.0, np.abs(ev))
    return rn / xn


@pytest.mark.parametrize("name", sorted(GOLD))
def test_gcge_core_over_gb300_table(name):
    g = GOLD[name]
    A, B = case_matrices(name)
    o = pyoracle.Oracle()
    ctx = G.Context(0)
    lib = ctx.lib
    table = o.new_table()
    assert lib.GCGE_GPU_SetOps(ctx.h, table) == 0
    lib.GCGE_GPU_OpsSeed(2024)
    dA = ctx.matrix(A)
    dB = ctx.matrix(B) if B is not None else None
    nev = g["params"]["nev"]
    kw = dict(g["params"])
    kw["ev_max_it"] = max(kw.get("ev_max_it", 30), 100)
    evec = o.table_multivec(table, dA.h, nev)
    launches0 = ctx.launches()
    try:
        ev, st = o.solve_table(table, dA.h, dB.h if dB is not None else None, A.n, o.params(**kw), evec)
        assert lib.GCGE_GPU_GetLastError(ctx.h) == 0
        blk, c0 = C.c_void_p(), C.c_int()
        assert lib.GCGE_GPU_OpsMultiVecBlock(evec, C.byref(blk), C.byref(c0)) == 0
        cm = np.zeros((nev, A.n))
        assert lib.GCGE_GPU_MultiVecDownload(blk, c0.value, nev, cm.ctypes.data) == 0
    finally:
        o.table_multivec_destroy(table, evec, nev)
    launches = ctx.launches() - launches0
    ctx.close()
    assert st.num_unlock == 0
    assert launches > 50 * st.num_iter, launches        # the n-sized work ran as this library's kernels
    np.testing.assert_allclose(ev, g["eval"], rtol=1e-10, atol=0)
    tol = g["params"].get("ev_tol", 1e-8)
    assert np.all(residuals(A, B, ev, cm.T, g["params"].get("conv_type", "R")) <= tol * 1.05)
