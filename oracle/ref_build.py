"""Build the reference-compiled pins under oracle/_ref/ (test infrastructure).

Runs the `ref` target of oracle/Makefile, which compiles
oracle/ref_morton.cpp against the reference's own
prtcl/util/morton_order.hpp, read in place from the reference checkout,
into oracle/_ref/libref_morton.so.  The Makefile names the checkout's
location (PRTCL_REFERENCE overrides it); without the checkout nothing is
built.  Nothing else of the reference's hot path builds from its own
sources: the grid (util/grouped_uniform_grid.hpp) needs Boost.Sort and,
through math.hpp, Eigen and the generated prtcl/config.hpp; the kernels and
schemes need Eigen.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root():
    """The reference checkout the recipe reads, or None where it is absent."""
    r = subprocess.run(["make", "-s", "-C", HERE, "print-reference"], capture_output=True, text=True)
    root = r.stdout.strip()
    return root or None


def build(verbose=False):
    r = subprocess.run(["make", "-s", "-C", HERE, "ref"], capture_output=True, text=True, check=True)
    so = os.path.join(OUT, "libref_morton.so")
    if verbose:
        print(r.stdout.strip())
    return so if os.path.exists(so) and "absent" not in r.stdout else None


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
