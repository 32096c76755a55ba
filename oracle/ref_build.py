"""Build the reference-compiled pins under oracle/_ref/ (test infrastructure).

Compiles oracle/ref_morton.cpp against the reference's own
prtcl/util/morton_order.hpp, read in place from the reference checkout at
/root/reference (or $PRTCL_REFERENCE), into oracle/_ref/libref_morton.so.
Nothing else of the reference's hot path builds from its own sources: the
grid (util/grouped_uniform_grid.hpp) needs Boost.Sort and, through
math.hpp, Eigen and the generated prtcl/config.hpp; the kernels and schemes
need Eigen.  Without the reference checkout this script does nothing.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root():
    return os.environ.get("PRTCL_REFERENCE", "/root/reference")


def build(verbose=False):
    src_root = os.path.join(reference_root(), "src")
    if not os.path.exists(os.path.join(src_root, "prtcl", "util", "morton_order.hpp")):
        if verbose:
            print("reference sources absent: nothing to build")
        return None
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libref_morton.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", src_root,
           os.path.join(HERE, "ref_morton.cpp"), "-o", so]
    subprocess.run(cmd, check=True)
    if verbose:
        print(so)
    return so


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
