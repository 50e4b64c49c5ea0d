"""The failure path of the tensor-core kernels, made to run on purpose.

Every mbarrier wait of the tcgen05 Gram and linear-combination kernels is
bounded (1 s of %globaltimer). GCGE_GPU_TestStallTensorWait makes the next
tensor-core launch's MMA-issuing thread wait for an arrival that cannot come,
so that wait runs out: the kernel must return (no hang), report
GCGE_GPU_ERR_TIMEOUT through GCGE_GPU_Synchronize, leave later tensor-core
launches on that context without effect, and free its TMEM, so that a fresh
context on the same GPU computes correct results afterwards. No fault, trap or
endless loop is involved: the only change is one wait that nothing satisfies."""
import time

import numpy as np
import pytest

import gcge_gb300 as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("op", ["lincomb", "gram"])
def test_bounded_tensor_wait_runs_out_and_recovers(op):
    rng = np.random.default_rng(11)
    n, k1, k2 = 262144, 64, 48
    X = rng.standard_normal((n, k1))
    W = rng.standard_normal((n, k2))
    Cm = np.asfortranarray(rng.standard_normal((k1, k2)))
    exact_lc = X @ Cm
    exact_gram = X.T @ W

    def run(ctx, sentinel=False):
        mx, mw = ctx.multivec(n, k1, X), ctx.multivec(n, k2, W)
        Y = ctx.multivec(n, k2, np.full((n, k2), np.nan) if sentinel else None)
        if op == "lincomb":
            G.multivec_linear_comb(mx, Y, (0, 0), (k1, k2), Cm.ravel(order="F"), k1)
            return Y.download()
        a = np.full(k1 * k2, np.nan)
        ctx.lib.GCGE_GPU_MultiVecInnerProd(mx.h, mw.h, a.ctypes.data, b"nonsym", G._ints(0, 0), G._ints(k1, k2), k1)
        return a.reshape(k2, k1).T

    ctx = G.Context(0)
    try:
        assert ctx.lib.GCGE_GPU_TestStallTensorWait(ctx.h, 1) == 0
        t0 = time.time()
        try:
            run(ctx)
        except G.GcgeGpuError as e:                   # the call may already see the status
            assert e.status == G.ERR_TIMEOUT
        st = ctx.lib.GCGE_GPU_Synchronize(ctx.h)
        elapsed = time.time() - t0
        assert st == G.ERR_TIMEOUT, st
        assert elapsed < 30.0, elapsed               # bounded: a few 1 s waits, not a hang
        # later tensor-core launches on the failed context do no work
        if op == "lincomb":
            try:
                out = run(ctx, sentinel=True)
                assert np.all(np.isnan(out))
            except G.GcgeGpuError as e:
                assert e.status == G.ERR_TIMEOUT
        assert ctx.lib.GCGE_GPU_Synchronize(ctx.h) == G.ERR_TIMEOUT
    finally:
        ctx.close()
    # TMEM was released: a fresh context on the same GPU runs the tensor-core kernels
    ctx2 = G.Context(0)
    try:
        out = run(ctx2)
        assert ctx2.lib.GCGE_GPU_Synchronize(ctx2.h) == 0
    finally:
        ctx2.close()
    ref = exact_lc if op == "lincomb" else exact_gram
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))
