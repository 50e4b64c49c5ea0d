"""The C-ABI boundary without a GPU: the library loads, exports every entry point
declared in include/*.h, fails loudly when no device is present, and the
GCGE_OPS layout restated in include/gcge_gb300_ops.h matches the reference's."""
import ctypes as C
import os
import subprocess
import sys

import pytest

import gcge_gb300 as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)
import build_oracle  # noqa: E402  (the oracle recipe knows where the reference sources are)

REF = build_oracle.reference_root()


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_library_exports_every_declared_symbol():
    L = G.load()
    declared = G.declared_symbols()
    assert len(declared) >= 28
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_error_strings():
    L = G.load()
    for st in range(8):
        assert L.GCGE_GPU_ErrorString(st)
    assert L.GCGE_GPU_ErrorString(99) == b"unknown status"


@pytest.mark.skipif(has_gpu(), reason="a CUDA device is present")
def test_init_fails_loudly_without_gpu():
    with pytest.raises(G.GcgeGpuError) as e:
        G.Context(0)
    assert e.value.status == 2


def test_null_arguments_rejected():
    L = G.load()
    assert L.GCGE_GPU_Init(0, None) == 1
    assert L.GCGE_GPU_MatCreate(None, 10, None, None, None, 0, None) == 1
    assert L.GCGE_GPU_SetOps(None, None) == 1


@pytest.mark.skipif(REF is None, reason="reference source tree absent (set GCGE_REFERENCE_ROOT to a GCGE-1.0 checkout)")
def test_ops_layout_matches_reference(tmp_path):
    cmd = ["gcc", "-std=gnu99", "-c", "-o", str(tmp_path / "x.o"), "-include", os.path.join(ROOT, "oracle", "ref_config.h"),
           "-I" + os.path.join(REF, "src"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi", "ops_layout_check.c")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_python_structs_match_c_headers():
    """ctypes mirrors of gcge_gpu_params / gcge_gpu_stats have the C sizes."""
    src = tmp = None
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "s.c")
        open(src, "w").write('#include <stdio.h>\n#include "gcge_gb300.h"\nint main(){printf("%zu %zu\\n",'
                             ' sizeof(gcge_gpu_params), sizeof(gcge_gpu_stats));return 0;}\n')
        exe = os.path.join(d, "s")
        subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), src, "-o", exe])
        a, b = map(int, subprocess.check_output([exe]).split())
    assert C.sizeof(G.Params) == a
    assert C.sizeof(G.Stats) == b


def test_long_row_list_host_logic():
    """The host pass that lists the rows the FP32 block-CG SpMM gives a block
    each: rows longer than the threshold, longest first, ties by row index, and
    their entry count (no GPU: a host function of the library)."""
    import numpy as np
    L = G.load()
    L.gb_long_rows_host.restype = C.c_int
    L.gb_long_rows_host.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_long)]
    rng = np.random.default_rng(5)
    for n, thresh in ((1, 0), (50, 64), (5000, 64), (5000, 5)):
        lens = rng.integers(0, 200, n).astype(np.int32)
        lens[rng.integers(0, n, max(1, n // 10))] = 130             # ties
        rp = np.zeros(n + 1, dtype=np.int32)
        rp[1:] = np.cumsum(lens)
        out = np.full(n, -1, dtype=np.int32)
        nz = C.c_long(-1)
        cnt = L.gb_long_rows_host(n, rp.ctypes.data, thresh, out.ctypes.data, C.byref(nz))
        want = [r for r in range(n) if lens[r] > thresh]
        want.sort(key=lambda r: (-int(lens[r]), r))
        assert cnt == len(want)
        assert out[:cnt].tolist() == want
        assert nz.value == int(sum(int(lens[r]) for r in want))
