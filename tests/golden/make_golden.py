"""Generate the golden fixtures under tests/golden/ from the compiled GCGE-1.0
reference (oracle/_ref). Run here, where the reference source tree exists:

    python oracle/build_oracle.py && python tests/golden/make_golden.py

Outputs:
* fem33_A.npz / fem33_M.npz: the reference's own FEM test pencil (test/data/A_5.txt,
  M_5.txt: 33x33-node stiffness/mass with Dirichlet rows), converted to CSR arrays.
* golden.json: eigenvalues, iteration counts and residual summaries that the
  reference reports on each case, plus checksums of its eigenvectors.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "gcge-1.0_gb300"))

import pyoracle  # noqa: E402
from gcge_gb300 import problems as P  # noqa: E402

import build_oracle  # noqa: E402  (the oracle recipe knows where the reference sources are)

if build_oracle.reference_root() is None:
    sys.exit("reference source tree absent: set GCGE_REFERENCE_ROOT to a GCGE-1.0 checkout")
REF_DATA = os.path.join(build_oracle.reference_root(), "test", "data")


def save_csr(path, M):
    np.savez_compressed(path, rowptr=M.rowptr, col=M.col, val=M.val)


def cases():
    """(name, A, B, params) for every golden case."""
    A5 = P.read_csr_text(os.path.join(REF_DATA, "A_5.txt"))
    M5 = P.read_csr_text(os.path.join(REF_DATA, "M_5.txt"))
    A3 = P.read_csr_text(os.path.join(REF_DATA, "A_3.txt"))
    M3 = P.read_csr_text(os.path.join(REF_DATA, "M_3.txt"))
    L1, _ = P.laplace2d(100, 100)
    Lsm, _ = P.laplace2d(30, 20)
    Fa, Fb = P.fem_q1_cube(10)
    return [
        ("fem33_nev10_dirichlet", A5, M5, dict(nev=10, dirichlet_boundary=1, seed=12345), ("fem33", "fem33")),
        ("fem9_nev4_dirichlet", A3, M3, dict(nev=4, dirichlet_boundary=1, seed=99), ("fem9", "fem9")),
        ("laplace100_nev10", L1, None, dict(nev=10, seed=777), None),
        ("laplace30x20_nev12_block4", Lsm, None, dict(nev=12, block_size=4, seed=5, ev_max_it=200), None),
        ("femcube10_nev6_abs", Fa, Fb, dict(nev=6, seed=31, conv_type="A", ev_max_it=100), None),
    ]


def main():
    ref = pyoracle.reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libgcge_ref.so is missing: run python oracle/build_oracle.py here")
    A5 = P.read_csr_text(os.path.join(REF_DATA, "A_5.txt"))
    M5 = P.read_csr_text(os.path.join(REF_DATA, "M_5.txt"))
    save_csr(os.path.join(HERE, "fem33_A.npz"), A5)
    save_csr(os.path.join(HERE, "fem33_M.npz"), M5)
    save_csr(os.path.join(HERE, "fem9_A.npz"), P.read_csr_text(os.path.join(REF_DATA, "A_3.txt")))
    save_csr(os.path.join(HERE, "fem9_M.npz"), P.read_csr_text(os.path.join(REF_DATA, "M_3.txt")))
    out = {}
    for name, A, B, kw, _ in cases():
        p = ref.params(**kw)
        ev, X, st = ref.solve(A, B, p)
        out[name] = dict(
            params=kw, n=A.n, nnz=A.nnz,
            eval=[float(v) for v in ev],
            num_iter=st.num_iter, num_unlock=st.num_unlock, max_res=st.max_res,
            evec_colsum=[float(v) for v in X.sum(axis=0)],
            evec_colnorm=[float(v) for v in np.linalg.norm(X, axis=0)],
        )
        print(name, st.num_iter, ev[:4])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
