"""Helpers to load the golden fixtures (tests/golden/)."""
import json
import os

import numpy as np

from gcge_gb300 import problems as P

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_csr(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    return P.CSR(z["rowptr"], z["col"], z["val"])


def golden():
    with open(os.path.join(HERE, "golden.json")) as f:
        return json.load(f)


def case_matrices(name):
    """Rebuild (A, B) of a golden case without the reference tree."""
    if name.startswith("fem33"):
        return load_csr("fem33_A"), load_csr("fem33_M")
    if name.startswith("fem9"):
        return load_csr("fem9_A"), load_csr("fem9_M")
    if name == "laplace100_nev10":
        return P.laplace2d(100, 100)
    if name == "laplace30x20_nev12_block4":
        return P.laplace2d(30, 20)
    if name == "femcube10_nev6_abs":
        return P.fem_q1_cube(10)
    raise KeyError(name)
