"""Long run of the 27,000-particle dam break (the reference's plain
configuration): 300 steps of the device step loop must stay finite, keep the
fluid inside its box (up to the integration's small overshoot at the walls),
meet the density-error bound in every step that did not hit the iteration
cap, and keep the kinetic energy of the same order as the potential energy
released (no blow-up; the compressed lattice start releases some pressure
energy on top of gravity's, so exact balance is not expected)."""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes

pytestmark = pytest.mark.gpu


def test_dam_break_300_steps():
    from prtcl_gb300.core import DeviceScene
    sc = scenes.dam_break()
    p = dict(driver.DAM_BREAK_27K)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    loop = driver.StepLoop(d, p, device_loop=True)
    y0 = d.get_varying("f", "position")[:, 1].astype(np.float64)
    stats = [loop.step() for _ in range(300)]
    x = d.get_varying("f", "position").astype(np.float64)
    v = d.get_varying("f", "velocity").astype(np.float64)
    for name in ("position", "velocity", "density", "pressure", "acceleration"):
        assert np.isfinite(d.get_varying("f", name)).all(), name
    box = np.array([2.0, 1.0, 1.0])
    margin = 0.5 * p["smoothing_scale"]
    assert (x > -margin).all() and (x < box + margin).all()
    for st in stats:
        if st["jacobi_iterations"] < p["max_iters"]:
            assert st["relative_aprde"] < p["eta"]
    capped = sum(st["jacobi_iterations"] >= p["max_iters"] for st in stats)
    assert capped <= 3  # only the first steps from the compressed lattice start
    # energy per unit mass: kinetic energy of the order of the potential
    # energy released
    ke = 0.5 * (v * v).sum(axis=1).mean()
    pe = 9.81 * (y0.mean() - x[:, 1].mean())
    assert pe > 0 and ke <= pe * 1.5
    # the fluid has moved (the dam collapses)
    assert x[:, 0].max() > sc["fluid"][:, 0].max() + 0.05


def test_batch_long_run_matches_constraints():
    from prtcl_gb300.batch import Batch
    p = dict(driver.DAM_BREAK_27K)
    bt = Batch(p)
    ids = [bt.add_scene(s["fluid"], s["boundary"]) for s in scenes.mixed_batch(count=8, lo=1500, hi=6000, seed=21)]
    bt.step(60)
    for sid in ids:
        i = bt.info(sid)
        assert i["steps"] == 60 and i["jacobi_solves"] == 60
        x = bt.download(sid, "position")
        assert np.isfinite(x).all() and np.isfinite(bt.download(sid, "velocity")).all()
        if i["jacobi_capped"] == 0:
            assert i["max_relative_density_error"] < p["eta"]
