"""Group configurations beyond one fluid and one boundary group: two fluid
and two boundary groups (every procedure, bit for bit against the oracle),
a model whose second fluid group is empty, and a model without boundary
groups.  The reference's procedures iterate `foreach fluid neighbor` over
every fluid group and `foreach _ neighbor` over the item's own group
(schemes/iisph.hpp:223-231, schemes/wkbb18.hpp:229-244)."""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise

pytestmark = pytest.mark.gpu

P = dict(driver.DAM_BREAK_27K, viscosity=True)


def setup(m, fluids, bounds, p):
    for name, pts in fluids.items():
        m.add_group(name, "fluid")
        m.add_tag(name, "dynamic")
    for name, pts in bounds.items():
        m.add_group(name, "boundary")
    for name, pts in {**fluids, **bounds}.items():
        m.resize(name, len(pts))
    h = np.float32(p["smoothing_scale"])
    rho0 = np.float32(p["rest_density"])
    for k, v in (("smoothing_scale", float(h)), ("time_step", float(np.float32(p["time_step"]))),
                 ("iisph_relaxation", float(np.float32(p["iisph_relaxation"]))), ("fade_duration", 0.0),
                 ("current_time", 0.0), ("maximum_speed", 0.0), ("iisph_iterations", 0),
                 ("iisph_maximum_iterations", int(p["max_iters"])),
                 ("iisph_maximum_density_error", float(np.float32(p["eta"])))):
        m.set_global(k, v)
    m.set_global("gravity", np.asarray(p["gravity"], np.float32).astype(np.float64))
    mass = np.float32(float(h) ** 3 * float(rho0))
    rng = np.random.default_rng(9)
    for name, pts in fluids.items():
        n = len(pts)
        m.set_uniform(name, "rest_density", float(rho0))
        m.set_uniform(name, "dynamic_viscosity", float(np.float32(p["dynamic_viscosity"])))
        m.set_uniform(name, "wkbb18_maximum_error", float(np.float32(p["wkbb18_maximum_error"])))
        m.set_uniform(name, "wkbb18_maximum_iterations", int(p["wkbb18_maximum_iterations"]))
        m.set_varying(name, "position", pts)
        m.set_varying(name, "velocity", (rng.standard_normal((n, 3)) * 0.2).astype(np.float32))
        m.set_varying(name, "acceleration", np.zeros((n, 3), np.float32))
        m.set_varying(name, "mass", np.full(n, mass, np.float32))
        m.set_varying(name, "time_of_birth", np.full(n, -1.0, np.float32))
    for name, pts in bounds.items():
        m.set_uniform(name, "dynamic_viscosity", float(np.float32(p["boundary_dynamic_viscosity"])))
        m.set_varying(name, "position", pts)
        m.set_varying(name, "volume", np.zeros(len(pts), np.float32))
    m.set_radius(2.0 * float(h))
    m.update()
    m.permute()
    m.run("aiast12", "compute_volume")


def pair(oracle_mod, fluids, bounds):
    from prtcl_gb300.core import DeviceScene
    d, o = DeviceScene(), oracle_mod.Scene(np.float32, fp64_reductions=True)
    setup(d, fluids, bounds, P)
    setup(o, fluids, bounds, P)
    return d, o


def compare(d, o, groups, fields, what):
    for g in groups:
        for name, nc in fields:
            assert_bitwise(d.get_varying(g, name, nc), o.get_varying(g, name, nc, d.model.get_group(g).item_count),
                           f"{what}: {g}.{name}")


def run_all(d, o, fl, bd):
    for m in (d, o):
        m.run("density", "compute_density")
    compare(d, o, fl, [("density", 1)], "density")
    for m in (d, o):
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("iisph", "setup")
    compare(d, o, fl, [("iisph_source_term", 1), ("iisph_diagonal_element", 1), ("iisph_helper_c", 3)], "setup")
    for it in range(3):
        for m in (d, o):
            m.set_global("iisph_aprde", 0.0)
            m.run("iisph", "iteration_pressure_acceleration")
            m.run("iisph", "iteration_pressure")
        compare(d, o, fl, [("acceleration", 3), ("pressure", 1)], f"jacobi {it}")
    for m in (d, o):
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("wkbb18", "compute_diagonal")
        m.run("wkbb18", "accumulate_acceleration")
    compare(d, o, fl, [("wkbb18_system_diagonal", 9), ("wkbb18_velocity_delta", 3), ("acceleration", 3)], "wkbb18")
    for g in fl:
        assert d.get_uniform(g, "wkbb18_iterations") == int(o.get_uniform(g, "wkbb18_iterations"))
    for m in (d, o):
        m.run("viscosity", "accumulate_acceleration")
        m.run("correction", "compute_gradient_correction")
        m.run("symplectic_euler", "integrate_position")
    compare(d, o, fl, [("acceleration", 3), ("gradient_correction", 9), ("position", 3)], "viscosity / L / x")
    compare(d, o, bd, [("volume", 1)], "volume")


def test_two_fluid_and_two_boundary_groups(oracle_mod):
    sc = scenes.dam_break(fluid_cells=(14, 12, 10), spacing=0.025, box=(0.7, 0.6, 0.5))
    f, b = sc["fluid"], sc["boundary"]
    fluids = {"fa": f[f[:, 0] < 0.17], "fb": f[f[:, 0] >= 0.17]}
    bounds = {"ba": b[b[:, 1] < 0.0], "bb": b[b[:, 1] >= 0.0]}
    d, o = pair(oracle_mod, fluids, bounds)
    run_all(d, o, list(fluids), list(bounds))


def test_empty_fluid_group(oracle_mod):
    sc = scenes.dam_break(fluid_cells=(10, 10, 10), spacing=0.025, box=(0.5, 0.5, 0.5))
    fluids = {"f": sc["fluid"], "g": np.zeros((0, 3), np.float32)}
    d, o = pair(oracle_mod, fluids, {"b": sc["boundary"]})
    run_all(d, o, ["f"], ["b"])
    assert d.get_uniform("g", "wkbb18_iterations") == 0


def test_no_boundary_group(oracle_mod):
    rng = np.random.default_rng(2)
    pts = ((np.stack(np.meshgrid(*[np.arange(10)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * 0.025
           + rng.standard_normal((1000, 3)) * 0.002).astype(np.float32)
    d, o = pair(oracle_mod, {"f": pts}, {})
    run_all(d, o, ["f"], [])
