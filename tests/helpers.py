"""Shared test helpers: build the same scene on the device and in the oracle."""
import numpy as np

from prtcl_gb300 import driver


def both_scenes(scene, params, oracle_mod):
    from prtcl_gb300.core import DeviceScene
    d = DeviceScene()
    o = oracle_mod.Scene(np.float32, fp64_reductions=True)
    driver.setup_dam_break(d, scene, params)
    driver.setup_dam_break(o, scene, params)
    return d, o


def point_scene(m, groups, radius):
    """groups: list of (name, type, points, tags)."""
    for name, type_, pts, tags in groups:
        m.add_group(name, type_)
        for t in tags:
            m.add_tag(name, t)
    for name, type_, pts, tags in groups:
        m.resize(name, len(pts))
        m.set_varying(name, "position", np.asarray(pts, np.float32))
    m.set_radius(radius)


def assert_bitwise(a, b, what=""):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    if not eq.all():
        bad = np.argwhere(~eq)[:5]
        raise AssertionError(f"{what}: {np.count_nonzero(~eq)} of {a.size} differ, e.g. at {bad.tolist()}: "
                             f"{a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}")
