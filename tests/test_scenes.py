"""Synthetic workloads: the search points and the radius calibration
(CPU, with the oracle's grid as the counter)."""
import numpy as np
import pytest

from prtcl_gb300 import scenes


@pytest.mark.parametrize("density", [1.0, 30.0, 0.001])
def test_calibration_brackets_from_below(density):
    """Mean count ~ r^3 at any density: the calibrated radius is the first
    to reach the target, and no trial radius sees more than about twice the
    target (the trial at the uniform radius of a clustered set would see
    `density` times it)."""
    ru = scenes.uniform_radius_for_mean_neighbours(4_000_000, 40.0)
    seen = []

    def mean_at(r):
        m = density * 40.0 * (r / ru) ** 3
        seen.append(m)
        return m

    r = scenes.calibrate_radius(mean_at, 4_000_000, 40.0)
    assert 40.0 <= mean_at(r) <= 40.02
    assert max(seen) <= 2.0 * 40.0 + 1e-9


def test_calibration_on_the_oracle_grid(oracle_mod):
    """A 40k-point blob set: the oracle's mean count at the calibrated radius
    is the target, and just below it is not."""
    from tests.helpers import point_scene
    n = 40_000
    pts = scenes.search_points(n, "blobs", seed=2)
    o = oracle_mod.Scene(np.float32)
    point_scene(o, [("p", "fluid", pts, [])], 0.05)

    def mean_at(r):
        o.set_radius(r)
        o.update()
        offs, _ = o.neighbor_lists(0, 0, n, cap=n * 200)
        return offs[-1] / n

    r = scenes.calibrate_radius(mean_at, n, 40.0, steps=10)
    assert mean_at(r) >= 40.0
    assert mean_at(r * (1 - 2e-3)) < 40.0
