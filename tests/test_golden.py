"""Pins of the oracle (and of the device grid) against fixtures made by the
reference's own compiled Morton comparison (tests/golden/make_golden.py,
prtcl/util/morton_order.hpp:19-95).

* every pair of morton_pairs.npz: oracle compare == reference compare;
* every cell set of morton_cells.npz: the grid's cell sequence (oracle on
  the CPU, device on the GPU) equals the reference's Morton order of the
  same cells; for the full-int32 set, which no float position can reach,
  consecutive cells are checked to be strictly increasing under the oracle
  compare (for distinct cells of a total order that fixes the sequence);
* with the reference build present (the reference checkout is around), the
  oracle is compared live with the reference on fresh random pairs.
"""
import ctypes as C
import os

import numpy as np
import pytest

from prtcl_gb300 import scenes
from tests.helpers import assert_bitwise, point_scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_SO = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libref_morton.so")


def pairs():
    return np.load(os.path.join(GOLDEN, "morton_pairs.npz"))


def cells():
    return np.load(os.path.join(GOLDEN, "morton_cells.npz"))


def cell_points(gi):
    # one point at the centre of each cell of edge 1: x = gi + 0.5 (exact in f32
    # for |gi| < 2^23)
    return (np.asarray(gi, np.float64) + 0.5).astype(np.float32)


def point_sets():
    c = cells()
    out = {}
    for name in ("box12", "wide20"):
        gi = c[name + "_gi_sorted"]
        pts = cell_points(gi[np.random.default_rng(1).permutation(len(gi))])
        out[name] = ([("p", "fluid", pts, [])], 1.0, gi)
    sc = scenes.dam_break()
    out["dam27k"] = ([("b", "boundary", sc["boundary"], []), ("f", "fluid", sc["fluid"], ["dynamic"])],
                     float(c["dam27k_radius"]), c["dam27k_gi_sorted"])
    return out


def test_oracle_morton_compare_matches_reference_pairs(oracle_mod):
    p = pairs()
    assert len(p["cmp"]) == 24000
    got = oracle_mod.morton_compare(p["a"], p["b"])
    assert_bitwise(got, p["cmp"], "morton compare")
    # all three outcomes occur
    assert set(np.unique(p["cmp"]).tolist()) == {-1, 0, 1}


def test_oracle_full_range_cell_sequence(oracle_mod):
    gi = cells()["full32_gi_sorted"]
    assert len(np.unique(gi, axis=0)) == len(gi)
    c = oracle_mod.morton_compare(gi[:-1], gi[1:])
    assert (c == -1).all()


@pytest.mark.parametrize("name", ["box12", "wide20", "dam27k"])
def test_oracle_grid_cell_order_matches_reference(oracle_mod, name):
    groups, r, gi = point_sets()[name]
    o = oracle_mod.Scene(np.float32)
    point_scene(o, groups, r)
    o.update()
    assert_bitwise(o.grid()["cell_gi"], gi, f"{name} cell order")


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build absent")
def test_oracle_morton_compare_live_against_reference(oracle_mod):
    L = C.CDLL(REF_SO)
    L.ref_morton_compare_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    rng = np.random.default_rng(99)
    n = 200_000
    for lo, hi in ((-2**31, 2**31), (-4, 4), (-2**20, 2**20)):
        a = rng.integers(lo, hi, (n, 3), dtype=np.int64).astype(np.int32)
        b = rng.integers(lo, hi, (n, 3), dtype=np.int64).astype(np.int32)
        ref = np.empty(n, np.int8)
        L.ref_morton_compare_many(a.ctypes.data, b.ctypes.data, n, ref.ctypes.data)
        assert_bitwise(oracle_mod.morton_compare(a, b), ref, f"live [{lo}, {hi})")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["box12", "wide20", "dam27k"])
def test_device_grid_cell_order_matches_reference(name):
    from prtcl_gb300.core import DeviceScene
    groups, r, gi = point_sets()[name]
    d = DeviceScene()
    point_scene(d, groups, r)
    d.update()
    assert_bitwise(d.nhood.grid()["cell_gi"], gi, f"{name} cell order")


def test_archive_fixture_is_consistent():
    """model_small.bin (the reference's native format, read back by the
    reference's own reader when it was made) against its values."""
    import struct
    data = open(os.path.join(GOLDEN, "model_small.bin"), "rb").read()
    exp = dict(np.load(os.path.join(GOLDEN, "model_small.npz")))
    pos = [0]

    def size():
        v = struct.unpack_from("<Q", data, pos[0])[0]
        pos[0] += 8
        return v

    def string():
        n = size()
        s = data[pos[0]:pos[0] + n].decode()
        pos[0] += n
        return s

    def ttype():
        ct = string()
        shape = [size() for _ in range(size())]
        return {"f32": np.float32, "s32": np.int32}[ct], shape

    def values(dt, n):
        a = np.frombuffer(data, dt, n, pos[0])
        pos[0] += a.nbytes
        return a

    for _ in range(size()):
        name = string()
        dt, shape = ttype()
        np.testing.assert_array_equal(values(dt, int(np.prod(shape))), np.ravel(exp["global/" + name]))
    for _ in range(size()):
        g, _type = string(), string()
        [string() for _ in range(size())]
        count = size()
        for _ in range(size()):
            name = string()
            dt, shape = ttype()
            assert size() == count
            v = values(dt, count * int(np.prod(shape)))
            np.testing.assert_array_equal(v, np.ravel(exp[f"{g}/varying/{name}"]))
        for _ in range(size()):
            name = string()
            dt, shape = ttype()
            np.testing.assert_array_equal(values(dt, int(np.prod(shape))), np.ravel(exp[f"{g}/uniform/{name}"]))
    assert pos[0] == len(data)
