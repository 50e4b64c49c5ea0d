"""CSR files through the C ABI (host code, no GPU): the reference's text format
(CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236) and the binary form.

The committed fixtures fem33_A/M are the reference's own A_5/M_5 test pencil
(tests/golden/make_golden.py); they are written back out in the reference's text
layout and read by the library, which must return the same arrays bit for bit
(values printed with the shortest round-trip repr, parsed with strtod)."""
import os

import numpy as np
import pytest

import gcge_gb300 as G
from gcge_gb300 import problems as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    return P.CSR(z["rowptr"], z["col"], z["val"])


def write_text(path, csr, ncol=None, sep="\n"):
    """The reference's layout: nrow, ncol, nnz, RowPtr, KCol, Entries, one per line."""
    toks = [str(csr.n), str(csr.n if ncol is None else ncol), str(len(csr.val))]
    toks += [str(int(x)) for x in csr.rowptr] + [str(int(x)) for x in csr.col] + [repr(float(x)) for x in csr.val]
    with open(path, "w") as f:
        f.write(sep.join(toks) + "\n")


def same(a, b):
    return (np.array_equal(a.rowptr, b.rowptr) and np.array_equal(a.col, b.col)
            and np.array_equal(a.val.view(np.int64), b.val.view(np.int64)))


@pytest.mark.parametrize("name", ["fem33_A", "fem33_M", "fem9_A", "fem9_M"])
def test_text_reader_matches_fixture(tmp_path, name):
    M = load_fixture(name)
    path = str(tmp_path / (name + ".txt"))
    write_text(path, M)
    got = G.read_csr(path)
    assert same(got, M)
    assert same(got, P.read_csr_text(path))


def test_text_reader_any_white_space(tmp_path):
    M = P.laplace2d(7, 5)[0]
    path = str(tmp_path / "ws.txt")
    write_text(path, M, sep=" \t ")
    assert same(G.read_csr(path), M)


@pytest.mark.parametrize("maker", [lambda: load_fixture("fem33_A"), lambda: P.powerlaw_graph(500, seed=3, dmax=60)[0],
                                   lambda: P.CSR(np.array([0, 0, 1]), np.array([1]), np.array([-2.5e-300]))])
def test_binary_round_trip(tmp_path, maker):
    M = maker()
    path = str(tmp_path / "m.bin")
    G.write_csr_binary(path, M)
    assert os.path.getsize(path) == 24 + 4 * (M.n + 1) + 12 * len(M.val)
    assert same(G.read_csr(path, binary=True), M)


def status(fn):
    with pytest.raises(G.GcgeGpuError) as e:
        fn()
    return e.value.status


def test_missing_and_truncated_files(tmp_path):
    assert status(lambda: G.read_csr(str(tmp_path / "none.txt"))) == G.ERR_IO
    assert status(lambda: G.read_csr(str(tmp_path / "none.bin"), binary=True)) == G.ERR_IO
    M = load_fixture("fem9_A")
    path = str(tmp_path / "t.txt")
    write_text(path, M)
    txt = open(path).read().split("\n")
    open(path, "w").write("\n".join(txt[:-10]))          # last entries missing
    assert status(lambda: G.read_csr(path)) == G.ERR_IO
    b = str(tmp_path / "t.bin")
    G.write_csr_binary(b, M)
    data = open(b, "rb").read()
    open(b, "wb").write(data[:-8])
    assert status(lambda: G.read_csr(b, binary=True)) == G.ERR_IO
    open(b, "wb").write(b"GCGECSR\x02" + data[8:])       # unknown header
    assert status(lambda: G.read_csr(b, binary=True)) == G.ERR_IO


def test_malformed_structure(tmp_path):
    M = load_fixture("fem9_A")
    path = str(tmp_path / "bad.txt")
    bad_col = P.CSR(M.rowptr, M.col.copy(), M.val)
    bad_col.col[5] = M.n                                # column out of range
    write_text(path, bad_col)
    assert status(lambda: G.read_csr(path)) == G.ERR_CSR
    rp = M.rowptr.copy()
    rp[3], rp[4] = rp[4], rp[3] - 1                     # decreasing row pointers
    write_text(path, P.CSR(rp, M.col, M.val))
    assert status(lambda: G.read_csr(path)) == G.ERR_CSR
    with pytest.raises(G.GcgeGpuError):
        G.write_csr_binary(str(tmp_path / "x.bin"), bad_col)
