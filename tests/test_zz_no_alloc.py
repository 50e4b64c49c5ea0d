"""GCGE_GPU_InnerProdNoAlloc: the Gram product for callers that own all device
memory through their own pool and may not call cudaMalloc / cudaFree.

torch plays such a caller here: it owns V, W and the output on the device; the
library is given raw device pointers and allocates nothing. Each result must
match the allocating entry point (GCGE_GPU_MultiVecInnerProd) on the same data,
within the tolerance of the other inner-product tests, on two calls in a row
(the fixed partial-sum array keeps the previous call's contents)."""
import numpy as np
import pytest

import gcge_gb300 as G

pytestmark = pytest.mark.gpu


def test_no_alloc_gram_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    ctx = G.Context(0)
    lib = ctx.lib
    rng = np.random.default_rng(21)
    # the last case has k1 * k2 = 262,144, the largest the fixed array takes (room
    # for four row splits of partials; the SM count asks for two at that size)
    cases = [(200003, 40, 40, True, False), (150000, 33, 17, False, True), (4099, 96, 80, False, False),
             (300007, 512, 512, False, True)]
    side = torch.cuda.Stream()
    for n, k1, k2, sym, on_side in cases:
        ldv, ldw, lda = k1 + 3, k2 + 1, k1 + 2
        V = rng.standard_normal((n, ldv))
        W = rng.standard_normal((n, ldw))
        if sym:
            W[:, :k2] = 0.5 * V[:, :k1] + 1e-3 * W[:, :k2]
        mv_v, mv_w = ctx.multivec(n, ldv, V), ctx.multivec(n, ldw, W)
        ref = G.multivec_inner_prod(mv_v, mv_w, (0, 0), (k1, k2), lda, sym=sym)
        scale = np.max(np.abs(ref))
        tV = torch.from_numpy(V).cuda()
        tW = torch.from_numpy(W).cuda()
        del V, W
        for _ in range(2):
            ta = torch.full((k2, lda), float("nan"), dtype=torch.float64, device="cuda")
            if on_side:
                # the caller's own stream: the call is ordered on it and on nothing else
                side.wait_stream(torch.cuda.current_stream())
                st = lib.GCGE_GPU_InnerProdNoAlloc(n, k1, k2, tV.data_ptr(), ldv, tW.data_ptr(), ldw,
                                                   ta.data_ptr(), lda, int(sym), side.cuda_stream)
                side.synchronize()
            else:
                st = lib.GCGE_GPU_InnerProdNoAlloc(n, k1, k2, tV.data_ptr(), ldv, tW.data_ptr(), ldw,
                                                   ta.data_ptr(), lda, int(sym), None)
            assert st == 0
            torch.cuda.synchronize()
            got = ta.cpu().numpy().ravel()
            for j in range(k2):
                np.testing.assert_allclose(got[j * lda:j * lda + k1], ref[j * lda:j * lda + k1], rtol=1e-12,
                                           atol=1e-12 * scale)
                assert np.all(np.isnan(got[j * lda + k1:(j + 1) * lda]))   # padding rows untouched
        del tV, tW, mv_v, mv_w
    # sizes beyond the fixed array are rejected before any launch
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    assert lib.GCGE_GPU_InnerProdNoAlloc(1000, 600, 600, small.data_ptr(), 600, small.data_ptr(), 600,
                                         small.data_ptr(), 600, 0, None) == 1
    assert lib.GCGE_GPU_InnerProdNoAlloc(1000, 8, 8, None, 8, small.data_ptr(), 8, small.data_ptr(), 8, 0, None) == 1
    ctx.close()
