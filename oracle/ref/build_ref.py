"""Build oracle/_ref/libref_krylov.so: the reference's own pAMP, GMRES and pIRAM templates.

    python oracle/ref/build_ref.py [/path/to/pyprop-source-tree]

Test infrastructure only. Nothing is copied out of the reference tree: its bundled blitz++
(extern/blitz/source) is configured out of tree into oracle/_build/blitz, and
oracle/ref/ref_krylov.cpp (this project's driver) is compiled with the reference's
core/krylov/{pamp/pamp/pamp.h, gmres/gmres.h, piram/piram/piram.h} straight from the tree.
The headers' outside dependencies are replaced by the shims in oracle/ref/shim: a one-rank
mpi.h, boost/shared_ptr.hpp over std::shared_ptr, cblas.h declarations, and LAPACK names -
all bound to the BLAS/LAPACK that ships inside scipy (symbols prefixed "scipy_").
-D__GCCXML__ selects the reference's own non-boost.python branch of
core/utility/boostpythonhack.h. Build products go to oracle/_build and oracle/_ref (both
git-ignored).
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
BUILD = os.path.join(ORACLE, "_build")
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref_krylov.so")


def reference_tree():
    """The PyProp source tree to build from: $PYPROP_REFERENCE, else /root/reference, when it
    holds core/krylov; None when neither does (e.g. on a machine without the reference)."""
    for cand in (os.environ.get("PYPROP_REFERENCE"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, "core", "krylov")):
            return cand
    return None


def scipy_blas():
    """Path of the BLAS/LAPACK library bundled with scipy."""
    import scipy
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    libs = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    return libs[0]


def configure_blitz(reference):
    bdir = os.path.join(BUILD, "blitz")
    if os.path.exists(os.path.join(bdir, "blitz", "gnu", "bzconfig.h")):
        return bdir
    os.makedirs(bdir, exist_ok=True)
    configure = os.path.join(reference, "extern", "blitz", "source", "configure")
    res = subprocess.run([configure, "--with-pic"], cwd=bdir, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("blitz++ configure failed:\n" + res.stdout[-2000:] + res.stderr[-2000:])
    return bdir


def build(reference, force=False):
    """Compile the library if it is missing or older than its sources; returns its path."""
    src = os.path.join(HERE, "ref_krylov.cpp")
    shims = glob.glob(os.path.join(HERE, "shim", "**", "*.h*"), recursive=True)
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(p) for p in [src, __file__] + shims)):
        return LIB
    if not os.path.isdir(os.path.join(reference, "core", "krylov")):
        raise RuntimeError("not a PyProp source tree: %s" % reference)
    bdir = configure_blitz(reference)
    blas = scipy_blas()
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-O2", "-std=gnu++14", "-shared", "-fPIC", "-w", "-D__GCCXML__",
           "-include", os.path.join(HERE, "shim", "prelude.h"),
           "-I", os.path.join(HERE, "shim"), "-I", bdir, "-I", os.path.join(reference, "extern", "blitz", "source"),
           "-I", reference, "-I", os.path.join(reference, "core"),
           src, "-o", LIB + ".tmp", blas, "-Wl,-rpath," + os.path.dirname(blas)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference Krylov build failed:\n%s\n%s" % (" ".join(cmd), res.stderr[-6000:]))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else reference_tree()
    if tree is None:
        sys.exit("usage: build_ref.py /path/to/pyprop-source-tree (or set PYPROP_REFERENCE)")
    print(build(tree, force=True))
