"""Parity at the workloads' own sizes, bit for bit against the oracle.

* The neighbour search on 4,000,000 points in the unit cube (uniform, seed
  1; 64 Gaussian blobs, seed 2), at the radius for 40 mean neighbours:
  cell grid indices, cell ranges, adjacency, sorted handles and every row of
  the neighbour lists (offsets and indices, in traversal order) must equal
  the oracle's (util/grouped_uniform_grid.hpp:139-359 for the grid,
  :407-531 for the query).
* The IISPH + WKBB18 dam break with 1,000,000 fluid and 363,436 boundary
  particles (dt 5e-4 s): the reference driver's step
  (share/scripts/prtcl-lua.example.lua:363-461) procedure by procedure, on
  the device and in the f32 oracle with FP64 convergence reductions.  Every
  field each procedure writes must be bit-identical, and the Jacobi and PCG
  iteration counts equal, in the first step (lattice start) and in the
  eighth (the first one after a permute).  The FP64 density-error sums agree
  to 1e-6 relative (the device sums in a fixed tree, the oracle
  sequentially).

At these sizes wide rows, list-capacity growth and the compressed cell keys
are all exercised; the smaller grid tests cover the edge cases.
"""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise, both_scenes, point_scene

pytestmark = pytest.mark.gpu

N_SEARCH = 4_000_000


def _grid_and_lists(d, o, counts, names):
    gd, go = d.nhood.grid(), o.grid()
    for k in ("cell_gi", "cell_range", "cell_adj", "sorted"):
        assert_bitwise(gd[k], go[k], k)
    del gd, go
    for q, qn in enumerate(names):
        if qn not in counts:
            continue
        for ng, nn in enumerate(names):
            od, idd = d.nhood.neighbor_lists(q, ng, counts[qn])
            oo, ido = o.neighbor_lists(q, ng, counts[qn], cap=int(od[-1]) + 16)
            assert_bitwise(od, oo, f"offsets {qn}->{nn}")
            assert_bitwise(idd, ido, f"indices {qn}->{nn}")


@pytest.mark.parametrize("dist,seed", [("uniform", 1), ("blobs", 2)])
def test_search_4m_bitexact(oracle_mod, dist, seed):
    from prtcl_gb300.core import DeviceScene
    n = N_SEARCH
    pts = scenes.search_points(n, dist, seed=seed)
    d = DeviceScene()
    point_scene(d, [("p", "fluid", pts, [])], 0.01)

    def mean_nbrs(r):
        d.set_radius(r)
        d.update()
        return d.nhood.query(0, count_pairs=True) / n

    r = scenes.calibrate_radius(mean_nbrs, n, 40.0)
    d.set_radius(r)
    d.update()
    o = oracle_mod.Scene(np.float32)
    point_scene(o, [("p", "fluid", pts, [])], r)
    o.update()
    _grid_and_lists(d, o, {"p": n}, ["p"])
    mean = d.nhood.query(0, count_pairs=True) / n
    assert 39.9 <= mean <= 40.5, mean


def _fields(d, o, group, names):
    for name, nc in names:
        assert_bitwise(d.get_varying(group, name, nc), o.get_varying(group, name, nc), f"{group}.{name}")


def _step(d, o, p, t, permute, check):
    """One step of the reference driver on both models, comparing after
    every procedure when ``check``."""
    for m in (d, o):
        m.set_global("current_time", float(np.float32(t)))
        m.update()
        if permute:
            m.permute()
    if check:
        _grid_and_lists(d, o, {"b": 363_436, "f": 1_000_000}, ["b", "f"])
        _fields(d, o, "f", [("position", 3), ("velocity", 3), ("mass", 1)])
        _fields(d, o, "b", [("position", 3), ("volume", 1)])
    seq = [
        ("density", "compute_density", [("density", 1)]),
        ("gravity", "initialize_acceleration", [("acceleration", 3)]),
        ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
        ("iisph", "setup", [("iisph_helper_c", 3), ("iisph_source_term", 1), ("iisph_diagonal_element", 1),
                            ("pressure", 1)]),
        ("iisph", "solve_pressure", [("pressure", 1), ("acceleration", 3), ("iisph_right_hand_side", 1)]),
        ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
        ("wkbb18", "compute_diagonal", [("wkbb18_system_diagonal", 9)]),
        ("wkbb18", "accumulate_acceleration", [("wkbb18_velocity_delta", 3), ("acceleration", 3)]),
        ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
        ("symplectic_euler", "integrate_position", [("position", 3)]),
    ]
    counts = {}
    for scheme, proc, out in seq:
        for m in (d, o):
            m.run(scheme, proc)
        if proc == "setup":
            assert d.get_global("iisph_nprde") == o.get_global("iisph_nprde")
        if proc == "solve_pressure":
            it_d, it_o = int(d.get_global("iisph_iterations")), int(o.get_global("iisph_iterations"))
            assert it_d == it_o, (it_d, it_o)
            ad, ao = d.get_global("iisph_aprde"), o.get_global("iisph_aprde")
            assert abs(ad - ao) <= 1e-6 * max(1.0, abs(ao)), (ad, ao)
            counts["jacobi"] = it_d
        if proc == "accumulate_acceleration":
            pd, po = int(d.get_uniform("f", "wkbb18_iterations")), int(o.get_uniform("f", "wkbb18_iterations"))
            assert pd == po, (pd, po)
            counts["pcg"] = pd
        if check:
            _fields(d, o, "f", out)
    if check:
        assert d.get_global("maximum_speed") == np.float32(o.get_global("maximum_speed"))
    return counts


def test_dam_break_1m_steps_bitexact(oracle_mod):
    sc = scenes.dam_break_1m()
    p = driver.DAM_BREAK_1M
    assert len(sc["fluid"]) == 1_000_000 and len(sc["boundary"]) == 363_436
    d, o = both_scenes(sc, p, oracle_mod)
    _fields(d, o, "b", [("volume", 1)])
    dt = float(np.float32(p["time_step"]))
    t, since = 0.0, 0
    history = []
    for k in range(1, 9):
        since += 1
        permute = since >= p["permute_every"]
        if permute:
            since = 0
        history.append(_step(d, o, p, t, permute, check=k in (1, 8)))
        t += dt
    print("per-step iteration counts (Jacobi, PCG):", [(h["jacobi"], h["pcg"]) for h in history])
    assert all(h["jacobi"] >= 2 for h in history)
