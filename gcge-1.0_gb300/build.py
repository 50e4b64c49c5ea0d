"""Build libgcge_gb300.so in-tree for sm_103a.

CUDA sources are compiled in parallel with nvcc (one -gencode, sm_103a only),
the C host driver with gcc, and everything is linked into
gcge-1.0_gb300/libgcge_gb300.so (static CUDA runtime). No cmake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libgcge_gb300.so")
OBJ = os.path.join(HERE, "_build")
CU = ["gb_blas.cu", "gb_bcg.cu", "gb_dense.cu", "gb_api.cu", "gb_noalloc.cu", "gb_ozaki.cu", "gb_adjoint.cu"]
C = ["gb_solver.c", "gb_ops_table.c", "gb_csrio.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return files + [__file__]


def up_to_date():
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(verbose=False, force=False):
    if not force and up_to_date():
        return OUT
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    jobs = []
    for f in CU:
        o = os.path.join(OBJ, f + ".o")
        jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
                                     os.path.join(CSRC, f), "-o", o] + inc)
    for f in C:
        o = os.path.join(OBJ, f + ".o")
        jobs.append(["gcc", "-std=c99", "-O2", "-fPIC", "-Wall", "-Wno-unused-function", "-c",
                     os.path.join(CSRC, f), "-o", o, "-I" + os.path.join(cuda, "include")] + inc)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OBJ, f + ".o") for f in CU + C]
    tmp = OUT + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lm"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
