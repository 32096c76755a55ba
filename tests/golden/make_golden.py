"""Generate the golden fixtures of this directory from the reference itself.

Needs the reference checkout (the Morton comparison is compiled from its
own prtcl/util/morton_order.hpp by oracle/ref_build.py into
oracle/_ref/libref_morton.so); the fixtures it writes are committed so that
the tests run without the reference.

morton_pairs.npz   a, b (int32 triples), cmp = morton_order_fn::compare(a, b)
                   on edge values (INT32_MIN, INT32_MIN + 1, -1, 0, 1,
                   INT32_MAX, ...), full-range random values and small
                   ranges with many ties.
morton_cells.npz   for each cell set S: S_gi_sorted, the distinct cells in the
                   reference's Morton order (std::stable_sort under
                   morton_order_fn::operator()).  Sets:
                   box12    all cells of [-6, 5]^3 (cells across the bias
                            boundary at 0),
                   wide20   4,000 distinct random cells in [-2^19, 2^19)^3,
                   full32   2,000 distinct random cells over the whole int32
                            range plus every triple of edge values,
                   dam27k   the occupied cells of the 27,000-particle dam
                            break (prtcl_gb300.scenes.dam_break(), radius
                            2 * (double)(float)0.025), gi = floor(double(x)/r).

Run:  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

EDGES = np.array([-2**31, -2**31 + 1, -2**30, -65536, -2, -1, 0, 1, 2, 65535, 2**30, 2**31 - 2, 2**31 - 1],
                 np.int64).astype(np.int32)


def ref_lib():
    from oracle import ref_build
    so = ref_build.build()
    if so is None:
        raise SystemExit("the reference sources are needed to generate the fixtures")
    L = C.CDLL(so)
    L.ref_morton_compare_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    L.ref_morton_sort.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    return L


def ref_compare(L, a, b):
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    out = np.empty(len(a), np.int8)
    L.ref_morton_compare_many(a.ctypes.data, b.ctypes.data, len(a), out.ctypes.data)
    return out


def ref_sorted(L, gi):
    gi = np.ascontiguousarray(gi, np.int32)
    order = np.empty(len(gi), np.int64)
    L.ref_morton_sort(gi.ctypes.data, len(gi), order.ctypes.data)
    return gi[order]


def distinct(rng, gi):
    _, first = np.unique(gi, axis=0, return_index=True)
    gi = gi[np.sort(first)]
    return gi[rng.permutation(len(gi))]


def main():
    L = ref_lib()
    rng = np.random.default_rng(20240611)
    n = 8000
    edge_a = EDGES[rng.integers(0, len(EDGES), (n, 3))]
    edge_b = EDGES[rng.integers(0, len(EDGES), (n, 3))]
    full_a = rng.integers(-2**31, 2**31, (n, 3), dtype=np.int64).astype(np.int32)
    full_b = rng.integers(-2**31, 2**31, (n, 3), dtype=np.int64).astype(np.int32)
    small_a = rng.integers(-8, 8, (n, 3)).astype(np.int32)
    small_b = small_a.copy()
    flip = rng.random((n, 3)) < 0.5
    small_b[flip] = rng.integers(-8, 8, int(flip.sum())).astype(np.int32)
    a = np.concatenate([edge_a, full_a, small_a])
    b = np.concatenate([edge_b, full_b, small_b])
    np.savez_compressed(os.path.join(HERE, "morton_pairs.npz"), a=a, b=b, cmp=ref_compare(L, a, b))

    ax = np.arange(-6, 6)
    box12 = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    wide20 = distinct(rng, rng.integers(-2**19, 2**19, (4000, 3)))
    edge_triples = np.stack(np.meshgrid(EDGES, EDGES, EDGES, indexing="ij"), -1).reshape(-1, 3)
    full32 = distinct(rng, np.concatenate([rng.integers(-2**31, 2**31, (2000, 3), dtype=np.int64),
                                           edge_triples.astype(np.int64)]))
    from prtcl_gb300 import scenes
    sc = scenes.dam_break()
    r = 2.0 * float(np.float32(0.025))
    pts = np.concatenate([sc["boundary"], sc["fluid"]]).astype(np.float64)
    dam = np.unique(np.floor(pts / r).astype(np.int64), axis=0)
    sets = {"box12": box12, "wide20": wide20, "full32": full32, "dam27k": dam}
    out = {}
    for name, gi in sets.items():
        gi = np.asarray(gi, np.int64).astype(np.int32)
        gi = gi[rng.permutation(len(gi))]
        out[name + "_gi_sorted"] = ref_sorted(L, gi)
    out["dam27k_radius"] = np.float64(r)
    np.savez_compressed(os.path.join(HERE, "morton_cells.npz"), **out)
    for k, v in out.items():
        print(k, np.shape(v))


if __name__ == "__main__":
    main()
