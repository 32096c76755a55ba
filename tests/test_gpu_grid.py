"""Device neighbourhood vs the oracle: cell assignment, cell order, cell
ranges, adjacency and neighbour sets must be bit-exact (grid contract of
util/grouped_uniform_grid.hpp with the (group, raw index) within-cell
tie-break)."""
import numpy as np
import pytest

from prtcl_gb300 import scenes
from tests.helpers import assert_bitwise, point_scene

pytestmark = pytest.mark.gpu


def make(oracle_mod, groups, radius, knobs=None):
    from prtcl_gb300.core import DeviceScene
    d = DeviceScene()
    for k, v in (knobs or {}).items():
        d.model.tune_set(k, v)
    o = oracle_mod.Scene(np.float32)
    point_scene(d, groups, radius)
    point_scene(o, groups, radius)
    d.update()
    o.update()
    return d, o


def compare(d, o, groups):
    gd, go = d.nhood.grid(), o.grid()
    for k in ("cell_gi", "cell_range", "cell_adj", "sorted"):
        assert_bitwise(gd[k], go[k], k)
    G = len(groups)
    names = sorted(g[0] for g in groups)
    counts = {g[0]: len(g[2]) for g in groups}
    for q in range(G):
        n = counts[names[q]]
        for ng in range(G):
            od, idd = d.nhood.neighbor_lists(q, ng, n)
            oo, ido = o.neighbor_lists(q, ng, n)
            assert_bitwise(od, oo, f"offsets {q}->{ng}")
            assert_bitwise(idd, ido, f"indices {q}->{ng}")


# 150k points: sorts and scans of several tiles per pass
@pytest.mark.parametrize("dist,n", [("uniform", 60000), ("blobs", 60000), ("uniform", 150000)])
def test_random_points(oracle_mod, dist, n):
    pts = scenes.search_points(n, dist, seed=1 if dist == "uniform" else 2)
    r = scenes.uniform_radius_for_mean_neighbours(n, 40.0) * (0.4 if dist == "blobs" else 1.0)
    groups = [("p", "fluid", pts, [])]
    d, o = make(oracle_mod, groups, r)
    compare(d, o, groups)
    offs, _ = o.neighbor_lists(0, 0, n)
    assert d.nhood.query(0, count_pairs=True) == int(offs[-1])


def test_negative_coordinates_and_exact_radius(oracle_mod):
    # a lattice straddling the origin whose spacing is r/2: axis neighbours at
    # two spacings sit at |d| = r up to rounding, the strict d^2 < r^2 test
    # must agree bit for bit; cells cross the INT32_MAX bias boundary at 0
    s = 0.025
    ax = (np.arange(-10, 10) + 0.5) * s
    g = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    pts = g.astype(np.float32)
    rng = np.random.default_rng(5)
    pts2 = (rng.random((3000, 3)) * 0.6 - 0.3).astype(np.float32)
    groups = [("a", "fluid", pts, []), ("b", "boundary", pts2, [])]
    d, o = make(oracle_mod, groups, 2 * np.float64(np.float32(s)))
    compare(d, o, groups)


def test_cannot_be_neighbor_group(oracle_mod):
    rng = np.random.default_rng(7)
    a = (rng.random((20000, 3)) * 2 - 1).astype(np.float32)
    c = (rng.random((500, 3)) * 2.4 - 1.2).astype(np.float32)  # some far outside any cell
    groups = [("a", "fluid", a, []), ("c", "probe", c, ["cannot_be_neighbor"])]
    d, o = make(oracle_mod, groups, 0.06)
    compare(d, o, groups)


def test_dam_break_initial_grid(oracle_mod):
    sc = scenes.dam_break()
    groups = [("f", "fluid", sc["fluid"], ["dynamic"]), ("b", "boundary", sc["boundary"], [])]
    d, o = make(oracle_mod, groups, 2 * np.float64(np.float32(0.025)))
    compare(d, o, groups)


def test_permute_round_trip(oracle_mod):
    rng = np.random.default_rng(11)
    a = (rng.random((30000, 3))).astype(np.float32)
    groups = [("a", "fluid", a, [])]
    d, o = make(oracle_mod, groups, 0.03)
    extra = rng.random((30000, 3)).astype(np.float32)
    d.set_varying("a", "payload", extra)
    o.set_varying("a", "payload", extra)
    d.permute()
    o.permute()
    pd, po = d.get_varying("a", "position"), o.get_varying("a", "position", 3)
    assert_bitwise(pd, po, "permuted positions")
    assert_bitwise(d.get_varying("a", "payload"), o.get_varying("a", "payload", 3), "permuted payload")
    # the permutation is a bijection of the original rows
    assert sorted(map(tuple, pd.tolist())) == sorted(map(tuple, a.tolist()))
    compare(d, o, groups)


def test_full_size_search_properties():
    """4M uniform points (the search workload): symmetric neighbour relation,
    every pair within the radius, cells sorted by Morton key and ranges
    partitioning the sorted sequence."""
    from prtcl_gb300.core import DeviceScene
    n = 4_000_000
    pts = scenes.search_points(n, "uniform", seed=1)
    r = scenes.uniform_radius_for_mean_neighbours(n, 40.0)
    d = DeviceScene()
    point_scene(d, [("p", "fluid", pts, [])], r)
    d.update()
    g = d.nhood.grid()
    rng_ = g["cell_range"]
    assert rng_[0, 0] == 0 and rng_[-1, 1] == n
    assert (rng_[1:, 0] == rng_[:-1, 1]).all() and (rng_[:, 1] > rng_[:, 0]).all()
    assert np.array_equal(np.sort(g["sorted"] & 0x0FFFFFFF), np.arange(n, dtype=np.uint32))
    offs, idx = d.nhood.neighbor_lists(0, 0, n)
    cnt = np.diff(offs)
    assert 35 < cnt.mean() < 45
    # sample: symmetric relation and distance test
    rng = np.random.default_rng(3)
    for i in rng.integers(0, n, 2000):
        js = idx[offs[i]:offs[i + 1]]
        assert i in js  # self is a neighbour
        d2 = ((pts[i] - pts[js]) ** 2).sum(1)
        assert (d2 < r * r * 1.0001).all()
        for j in js[:8]:
            assert i in idx[offs[j]:offs[j + 1]]


def test_rows_turning_wide_mid_list(oracle_mod):
    """A lattice in storage order (neighbour deltas fit 16 bits) with 1 % of
    its points swapped with points 100,000 indices away: rows become wide at
    every position of the list (first, mid-chunk, in a later chunk), and the
    entries written before are converted; lists must match the oracle."""
    m = 56
    ax = np.arange(m, dtype=np.float32) * np.float32(0.01)
    pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3).copy()
    n = len(pts)
    rng = np.random.default_rng(5)
    for a in rng.choice(n, n // 100, replace=False):
        b = (a + 100_000) % n
        pts[[a, b]] = pts[[b, a]]
    groups = [("p", "fluid", pts, [])]
    d, o = make(oracle_mod, groups, 0.0205)
    compare(d, o, groups)


@pytest.mark.parametrize("levels,near", [
    ((0, 2, 8, 10), True),          # informative key bits in two runs
    ((0, -3, 70, -70), True),       # three runs, negative indices
    ((1, 11, 33, 513), False),      # four runs
    ((1, 683, 547, 137), False),    # five runs: the general bit gather
])
def test_scattered_grid_indices(oracle_mod, levels, near):
    """Small clusters at grid indices whose bit patterns leave one to more
    than four runs of informative key bits (`near`: with a cluster in the
    next cell along x of each, so adjacency is not empty): cells, adjacency
    and lists must match the oracle."""
    r = 0.1
    rng = np.random.default_rng(sum(abs(v) for v in levels))
    pts = []
    for a in levels:
        for b in levels[:3]:
            for c in levels[::-1][:3]:
                centre = (np.array([a, b, c], np.float64) + 0.5) * r
                pts.append(centre + rng.uniform(-0.45 * r, 0.45 * r, (12, 3)))
                if near:
                    pts.append(centre + np.array([r, 0.0, 0.0]) + rng.uniform(-0.45 * r, 0.45 * r, (3, 3)))
    pts = np.concatenate(pts).astype(np.float32)
    groups = [("p", "fluid", pts, [])]
    d, o = make(oracle_mod, groups, r)
    compare(d, o, groups)


@pytest.mark.parametrize("then_permute", [False, True])
def test_key_layout_change_between_updates(oracle_mod, then_permute):
    """An update reuses the previous cell-key layout and confirms it at the
    next synchronisation (the list build, or a permute first).  Points moved
    to cells whose indices carry new bit patterns change the layout: the
    grid must be rebuilt with the new one before anything reads it, and the
    lists equal the oracle's."""
    rng = np.random.default_rng(21)
    pts = (rng.random((20000, 3)) * 0.5).astype(np.float32)
    groups = [("p", "fluid", pts, [])]
    d, o = make(oracle_mod, groups, 0.02)
    compare(d, o, groups)
    moved = pts.copy()
    moved[:300] -= np.float32(3.0)    # negative cells: bit 31 of the biased index flips
    moved[300:600] += np.float32(40.0)  # far cells: new high bits
    groups = [("p", "fluid", moved, [])]
    for m in (d, o):
        m.set_varying("p", "position", moved)
        m.update()
        if then_permute:
            m.permute()
    compare(d, o, groups)
    # and back: the layout shrinks again
    back = o.get_varying("p", "position", 3)
    back[np.abs(back).max(axis=1) > 1.0] = np.float32(0.25)
    for m in (d, o):
        m.set_varying("p", "position", back)
        m.update()
    compare(d, o, [("p", "fluid", back, [])])


@pytest.mark.parametrize("grid_sort,list_split", [(0, 0), (1, 0), (1, 1)])
@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 8193])
def test_cell_pass_tile_boundaries(oracle_mod, n, grid_sort, list_split):
    """The cell pass counts cell starts per tile of 4,096 sorted items and
    fills the tables per tile: sizes at the tile boundaries (about 38 items
    a cell, so cells straddle the tiles' ends) equal the oracle's grid and
    lists, with either sort.  A second update of moved points takes the
    previous key layout (the keyed first pass) and must agree too."""
    rng = np.random.default_rng(31 + n)
    pts = (rng.random((n, 3)) * 0.3).astype(np.float32)
    groups = [("p", "fluid", pts, [])]
    d, o = make(oracle_mod, groups, 0.05, {"grid_sort": grid_sort, "list_split": list_split})
    compare(d, o, groups)
    moved = (pts + (rng.random((n, 3)).astype(np.float32) - 0.5) * np.float32(0.01)).astype(np.float32)
    for m in (d, o):
        m.set_varying("p", "position", moved)
        m.update()
    compare(d, o, [("p", "fluid", moved, [])])


@pytest.mark.parametrize("n", [1000, 64000, 64001, 100000, 128000])
def test_cluster_sort_sizes(oracle_mod, n):
    """The one-launch cluster sort (grid_sort 1): 8 CTAs up to 64,000 grid
    items, 16 up to 128,000, with two groups so that handles of both sit in
    the sort; the grid and the lists equal the oracle's."""
    rng = np.random.default_rng(41)
    a = (rng.random((n - n // 3, 3)) * 0.6).astype(np.float32)
    b = (rng.random((n // 3, 3)) * 0.6).astype(np.float32)
    groups = [("a", "fluid", a, []), ("b", "boundary", b, [])]
    r = scenes.uniform_radius_for_mean_neighbours(n, 20.0) * 0.6
    d, o = make(oracle_mod, groups, r, {"grid_sort": 1})
    compare(d, o, groups)


@pytest.mark.parametrize("case", ["dam_break", "wide_rows", "negative"])
def test_split_list_build(oracle_mod, case):
    """The list build with four threads per query (list_split 1) equals the
    oracle's lists: the 27k dam break (two groups, narrow rows), an
    unpermuted group whose rows are wide (scattered raw indices walked in
    grid order), and a lattice straddling the origin with neighbours at
    exactly the radius."""
    if case == "dam_break":
        sc = scenes.dam_break()
        groups = [("f", "fluid", sc["fluid"], ["dynamic"]), ("b", "boundary", sc["boundary"], [])]
        r = 2 * np.float64(np.float32(0.025))
    elif case == "wide_rows":
        rng = np.random.default_rng(13)
        pts = rng.random((60000, 3)).astype(np.float32)
        groups = [("p", "fluid", pts, [])]
        r = scenes.uniform_radius_for_mean_neighbours(60000, 40.0)
    else:
        s = 0.025
        ax = (np.arange(-10, 10) + 0.5) * s
        g = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
        rng = np.random.default_rng(5)
        b = (rng.random((3000, 3)) * 0.6 - 0.3).astype(np.float32)
        groups = [("a", "fluid", g, []), ("b", "boundary", b, [])]
        r = 2 * np.float64(np.float32(s))
    d, o = make(oracle_mod, groups, r, {"list_split": 1})
    compare(d, o, groups)
