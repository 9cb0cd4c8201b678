"""Build pyLOM's own compiled SVD path into oracle/_ref/ -- TEST INFRASTRUCTURE.

The reference's compiled path for tsqr_svd is plain C over LAPACKE/CBLAS
(pyLOM/vmmath/src/svd.c: stsqr/dtsqr, ssvd/dsvd, stsqr_svd/dtsqr_svd;
pyLOM/vmmath/src/vector_matrix.c: smatmul/dmatmul and the other products).
This recipe compiles those two files as they are, against:

* oracle/ref_shim/mpi.h -- a single-rank MPI stand-in (no MPI is installed);
* oracle/ref_shim/cblas.h, lapacke.h -- the CBLAS/LAPACKE declarations mapped
  onto the prefixed symbols of the OpenBLAS build SciPy bundles
  (scipy_cblas_*, scipy_LAPACKE_*; LP64), linked by its path.

Outputs go to oracle/_ref/ only (git-ignored): src/ (the reference's files,
staged from the pyLowOrder sources so that the recipe can compile them again
on a machine without those sources) and libpylom_ref.so.  Only tests/ and
bench.py's CPU-baseline / reference legs load the result (oracle/plom_ref.py).

Usage: python oracle/build_ref.py [path to the pyLowOrder sources]
(without a path: the sources at DEFAULT_SOURCES when they are there, else the
copy staged under oracle/_ref/src).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
SHIM = os.path.join(HERE, "ref_shim")
LIB = os.path.join(OUT, "libpylom_ref.so")
FILES = ["svd.c", "svd.h", "vector_matrix.c", "vector_matrix.h"]
DEFAULT_SOURCES = "/root/reference"  # where the build container mounts pyLowOrder


def stage(refroot):
    src = os.path.join(refroot, "pyLOM", "vmmath", "src")
    if not all(os.path.exists(os.path.join(src, f)) for f in FILES):
        return False
    os.makedirs(SRC, exist_ok=True)
    for f in FILES:
        shutil.copy2(os.path.join(src, f), os.path.join(SRC, f))
    return True


def openblas():
    """Path of the OpenBLAS library SciPy bundles (scipy.libs/libscipy_openblas*.so)."""
    import scipy
    d = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__))), "scipy.libs")
    cands = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so*")))
    cands = [c for c in cands if "64_" not in os.path.basename(c)]
    return cands[0] if cands else None


def build(refroot=None, quiet=True):
    """Compile libpylom_ref.so; returns its path, or raises RuntimeError with the
    reason it cannot be built here."""
    if refroot is None and os.path.isdir(DEFAULT_SOURCES):
        refroot = DEFAULT_SOURCES
    if refroot and os.path.isdir(refroot):
        stage(refroot)
    if not all(os.path.exists(os.path.join(SRC, f)) for f in FILES):
        raise RuntimeError("pyLOM's C sources are not staged under oracle/_ref/src")
    ob = openblas()
    if ob is None:
        raise RuntimeError("SciPy's bundled OpenBLAS (scipy.libs/libscipy_openblas*.so) not found")
    cc = os.environ.get("CC", "gcc")
    tmp = LIB + ".tmp"
    cmd = [cc, "-O3", "-std=gnu11", "-fPIC", "-shared", "-w", "-I", SHIM, "-I", SRC,
           os.path.join(SRC, "svd.c"), os.path.join(SRC, "vector_matrix.c"), "-o", tmp, ob,
           "-Wl,-rpath," + os.path.dirname(ob), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    if not quiet:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else None, quiet=False)
