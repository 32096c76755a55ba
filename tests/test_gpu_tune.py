"""The launch-shape knobs change speed only: a dam break (IISPH + WKBB18,
all tuned sweeps active) and a batch of scenes give bit-identical fields and
the same iteration counts under every knob setting; the autotuner runs
end to end on the device."""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes, tune

pytestmark = pytest.mark.gpu

SETTINGS = [
    {**{k: 1 for k in tune.SWEEP_KNOBS}, "jacobi_unroll": 2},
    {**{k: 2 for k in tune.SWEEP_KNOBS}, "jacobi_unroll": 4},
    {**{k: 3 for k in tune.SWEEP_KNOBS}, "jacobi_unroll": 1},
    {"pcg_q": 4},  # the cell-tile sweep
    {"staging": 1},  # staged lists and sweeps
    {"staging": 1, "jacobi_unroll": 2, "iisph_pressure": 2},
    {"grid_sort": 0},  # the grid sorted by the tiled launches (default: one cluster launch)
    {"grid_sort": 0, "staging": 1},
    {"list_split": 0},  # one thread per query builds the lists (default: four for small groups)
    {"list_split": 1, "staging": 1},  # staging takes precedence over the split build
]
FIELDS = (("position", 3), ("velocity", 3), ("density", 1), ("pressure", 1), ("acceleration", 3),
          ("wkbb18_velocity_delta", 3))


def _run(sc, p, knobs, steps):
    from prtcl_gb300.core import DeviceScene
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    for k, v in knobs.items():
        d.model.tune_set(k, v)
    loop = driver.StepLoop(d, p, device_loop=True)
    counts = [loop.step() for _ in range(steps)]
    return d, [(c["jacobi_iterations"], c["pcg_iterations"]) for c in counts]


@pytest.mark.parametrize("setting", range(len(SETTINGS)))
def test_knobs_keep_results_bitwise(gpu_lib, setting):
    sc = scenes.dam_break(fluid_cells=(16, 18, 12), spacing=0.025, box=(0.8, 0.7, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    ref, cref = _run(sc, p, {}, 10)
    d, c = _run(sc, p, SETTINGS[setting], 10)
    assert c == cref
    for name, nc in FIELDS:
        a, b = d.get_varying("f", name, nc), ref.get_varying("f", name, nc)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
    for k, v in SETTINGS[setting].items():
        assert d.model.tune_get(k) == v


def test_cell_tile_sweep_at_1m(gpu_lib):
    """The cell-tile PCG sweep on the 1M dam break (tiles along the walls,
    tiles that overflow the staging and take the lists): two steps equal
    the list sweep's bit for bit."""
    sc = scenes.dam_break_1m()
    p = driver.DAM_BREAK_1M
    ref, cref = _run(sc, p, {}, 2)
    d, c = _run(sc, p, {"pcg_q": 4}, 2)
    assert c == cref
    for name, nc in FIELDS:
        a, b = d.get_varying("f", name, nc), ref.get_varying("f", name, nc)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


def test_staged_sweeps_at_1m(gpu_lib):
    """Staged lists and sweeps on the 1M dam break: most tiles stage (the
    others take the global gathers) and two steps equal the unstaged run's
    bit for bit."""
    sc = scenes.dam_break_1m()
    p = driver.DAM_BREAK_1M
    ref, cref = _run(sc, p, {}, 2)
    d, c = _run(sc, p, {"staging": 1}, 2)
    assert c == cref
    for name, nc in FIELDS:
        a, b = d.get_varying("f", name, nc), ref.get_varying("f", name, nc)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
    fg = d.model.get_group("f").index
    staged, tiles = d.nhood.staged_tiles(fg)
    assert tiles == (len(sc["fluid"]) + 127) // 128
    assert staged >= 0.5 * tiles, (staged, tiles)
    assert ref.nhood.staged_tiles(fg) == (0, 0)


def test_staging_switches_off(gpu_lib):
    """Turning staging off after staged steps rebuilds plain lists; the run
    continues bit-identically to one that never staged."""
    sc = scenes.dam_break(fluid_cells=(16, 18, 12), spacing=0.025, box=(0.8, 0.7, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    from prtcl_gb300.core import DeviceScene
    runs = []
    for knobs in ((0, 0), (1, 0)):
        d = DeviceScene()
        driver.setup_dam_break(d, sc, p)
        loop = driver.StepLoop(d, p, device_loop=True)
        for k in knobs:
            d.model.tune_set("staging", k)
            for _ in range(4):
                loop.step()
        runs.append(d)
    fg = runs[1].model.get_group("f").index
    assert runs[1].nhood.staged_tiles(fg) == (0, 0)
    for name, nc in FIELDS:
        a, b = runs[1].get_varying("f", name, nc), runs[0].get_varying("f", name, nc)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


def test_knobs_keep_batched_results_bitwise(gpu_lib):
    from prtcl_gb300.batch import Batch
    p = dict(driver.DAM_BREAK_27K)
    sc = scenes.mixed_batch(count=6, lo=600, hi=6000, seed=11)
    out = []
    # the last setting: the persistent tiled sweeps taking tiles from a work counter
    for knobs in ({}, SETTINGS[0], SETTINGS[1], {"iisph_accel": 4, "iisph_pressure": 4, "jacobi_unroll": 2}):
        bt = Batch(p)
        for k, v in knobs.items():
            bt.tune_set(k, v)
        ids = [bt.add_scene(x["fluid"], x["boundary"]) for x in sc]
        bt.step(9)
        out.append([(bt.download(i, "position"), bt.info(i)["jacobi_iterations"]) for i in ids])
    for other in out[1:]:
        for (x, it), (xr, itr) in zip(other, out[0]):
            assert it == itr
            assert np.array_equal(x.view(np.uint32), xr.view(np.uint32))


def test_tuner_on_the_device(gpu_lib, tmp_path):
    sc = scenes.dam_break(fluid_cells=(14, 14, 10), spacing=0.025, box=(0.7, 0.6, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    t = tune.Autotuner(cache_path=str(tmp_path / "t.json"), device="test-device")
    choice, source, timings = tune.tune_plain(sc, p, tuner=t)
    assert source == "tuned" and set(choice) == set(tune.VALUES)
    assert all(f"{k}={v}" in timings for k in tune.SWEEP_KNOBS for v in tune.VALUES[k])
    assert tune.tune_plain(sc, p, tuner=t)[1] == "cache"
    d, c = _run(sc, p, choice, 4)
    ref, cref = _run(sc, p, {}, 4)
    assert c == cref
    assert np.array_equal(d.get_varying("f", "position", 3).view(np.uint32),
                          ref.get_varying("f", "position", 3).view(np.uint32))


def test_knob_errors(gpu_lib):
    from prtcl_gb300 import PrtclGpuError, PrtclNotFound
    from prtcl_gb300.core import Model
    m = Model()
    with pytest.raises(PrtclNotFound, match="unknown tuning knob"):
        m.tune_set("no_such_knob", 0)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("iisph_accel", 5)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("density", 4)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("pcg_q", 5)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("jacobi_unroll", 3)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("staging", 2)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("grid_sort", 2)
    with pytest.raises(PrtclGpuError, match="invalid argument"):
        m.tune_set("list_split", 2)
    assert m.tune_get("jacobi_unroll") == 1 and m.tune_get("pcg_q") == 0
    m.tune_set("pcg_q", 4)
    assert m.tune_get("pcg_q") == 4
