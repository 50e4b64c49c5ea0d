"""Build recipe for the oracle (test infrastructure only).

* ``oracle/libgcge_oracle.so``: the C restatement in ``gcge_oracle.c``.
* ``oracle/_ref/libgcge_ref.so``: the GCGE-1.0 reference itself, compiled from
  its own sources where they lie (``src/*.c`` and ``app/csr/gcge_app_csr.c``),
  with MPI switched off through ``ref_config.h`` and BLAS/LAPACK forwarded to
  SciPy's OpenBLAS by ``ref_blas_shim.c``. Built only where the reference
  source tree is present; outputs go to ``oracle/_ref/`` only.

Both link the OpenBLAS that SciPy bundles (symbols prefixed ``scipy_``); the
vendored Fortran BLAS/LAPACK of the reference cannot be built (no gfortran).
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference source tree this recipe compiles from: GCGE_REFERENCE_ROOT when set,
# else the read-only checkout of the build container. This recipe is the one place
# that names it; tests and fixture scripts ask reference_root() below.
REF_ROOT = os.environ.get("GCGE_REFERENCE_ROOT", "/root/reference")


def reference_root():
    """The reference source tree, or None where it is absent (as on the GPU host)."""
    return REF_ROOT if os.path.isdir(os.path.join(REF_ROOT, "src")) else None
REF_SOURCES = [
    "src/gcge_cg.c", "src/gcge_eigsol.c", "src/gcge_ops.c", "src/gcge_orthogonal.c",
    "src/gcge_para.c", "src/gcge_rayleighritz.c", "src/gcge_solver.c", "src/gcge_statistics.c",
    "src/gcge_utilities.c", "src/gcge_workspace.c", "src/gcge_xpw.c", "app/csr/gcge_app_csr.c",
]


def openblas():
    """Return (directory, file name) of SciPy's bundled OpenBLAS."""
    import scipy
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    for pat in ("scipy.libs/libscipy_openblas*.so*", "scipy/.libs/libscipy_openblas*.so*"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return os.path.dirname(hits[0]), os.path.basename(hits[0])
    raise RuntimeError("SciPy's bundled OpenBLAS (libscipy_openblas*.so) not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_oracle(verbose=False):
    out = os.path.join(HERE, "libgcge_oracle.so")
    src = os.path.join(HERE, "gcge_oracle.c")
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = [src, os.path.join(HERE, "gcge_oracle.h"), os.path.join(inc, "gcge_gb300_ops.h"),
            os.path.join(inc, "gcge_gb300.h"), __file__]
    if _newer(out, deps):
        return out
    d, f = openblas()
    cmd = ["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-Wall", "-o", out, src, "-I" + inc,
           "-L" + d, "-l:" + f, "-Wl,-rpath," + d, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_reference(verbose=False):
    """Compile the reference into oracle/_ref/libgcge_ref.so (None if absent)."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libgcge_ref.so")
    srcs = [os.path.join(REF_ROOT, s) for s in REF_SOURCES]
    mine = [os.path.join(HERE, "ref_entry.c"), os.path.join(HERE, "ref_blas_shim.c")]
    deps = srcs + mine + [os.path.join(HERE, "ref_config.h"), __file__]
    if _newer(out, deps):
        return out
    d, f = openblas()
    cmd = ["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-w",
           "-include", os.path.join(HERE, "ref_config.h"),
           "-I" + os.path.join(REF_ROOT, "src"), "-I" + os.path.join(REF_ROOT, "app/csr"), "-I" + HERE,
           "-o", out] + srcs + mine + ["-L" + d, "-l:" + f, "-Wl,-rpath," + d, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build(verbose=False):
    build_oracle(verbose)
    build_reference(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
