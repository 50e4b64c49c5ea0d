"""GCGE's solver core driven through a GCGE_OPS table, on the CPU.

The oracle's GCGE_Solve restatement sends every n-sized operation through a
table with the GCGE_OPS layout, as the reference's core does
(src/gcge_ops.h:29-215). Here the table is the oracle's host CSR table (the
reference's GCGE_CSR_SetOps plus the GCGE_OPS_Setup defaults), with the
multivectors made by the table's own MultiVecCreateByMat and the initial vectors
by its MultiVecSetRandomValue, as GCGE_CSR_Solver_Init and GCGE_Solve do
(app/csr/gcge_app_csr.c:92-124, src/gcge_eigsol.c:126-135). The result must be
bit-identical to the restatement's direct entry, which is itself bit-identical
to the compiled reference (test_oracle_golden.py).
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from _golden import case_matrices, golden

G = golden()


@pytest.fixture(scope="module")
def oracle():
    return pyoracle.Oracle()


def _handle(o, M):
    M.rowptr = np.ascontiguousarray(M.rowptr, dtype=np.int32)
    M.col = np.ascontiguousarray(M.col, dtype=np.int32)
    M.val = np.ascontiguousarray(M.val, dtype=np.float64)
    return o.lib.gcge_oracle_csr_handle(M.n, M.rowptr.ctypes.data, M.col.ctypes.data, M.val.ctypes.data)


@pytest.mark.parametrize("name", sorted(G))
def test_table_solve_bitwise_equals_direct_restatement(oracle, name):
    g = G[name]
    A, B = case_matrices(name)
    table = oracle.new_table(host=True)
    hA = _handle(oracle, A)
    hB = _handle(oracle, B) if B is not None else None
    nev = g["params"]["nev"]
    evec = oracle.table_multivec(table, hA, nev)
    try:
        ev_t, st_t = oracle.solve_table(table, hA, hB, A.n, oracle.params(**g["params"]), evec)
        X_t = np.zeros((nev, A.n))
        oracle.lib.gcge_oracle_host_mv_read(evec, nev, A.n, X_t.ctypes.data)
    finally:
        oracle.table_multivec_destroy(table, evec, nev)
        oracle.lib.gcge_oracle_csr_handle_free(hA)
        if hB:
            oracle.lib.gcge_oracle_csr_handle_free(hB)
    ev_d, X_d, st_d = oracle.solve(A, B, oracle.params(**g["params"]))
    assert st_t.num_iter == st_d.num_iter == g["num_iter"]
    assert np.array_equal(ev_t, ev_d)
    assert np.array_equal(X_t.T, X_d)


def test_table_solve_rejects_incomplete_table(oracle):
    A, _ = case_matrices("laplace30x20_nev12_block4")
    table = oracle.new_table(host=False)        # every member NULL
    hA = _handle(oracle, A)
    st = pyoracle.Stats()
    ev = np.zeros(4)
    rc = oracle.lib.gcge_oracle_solve_table(table, hA, None, A.n, C.byref(oracle.params(nev=4)), ev.ctypes.data,
                                            None, C.byref(st))
    oracle.lib.gcge_oracle_csr_handle_free(hA)
    assert rc == 1
