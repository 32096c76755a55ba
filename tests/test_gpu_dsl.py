"""Schemes generated from the scheme language (prtcl_gb300.dsl) on the
device.  tests/dsl/sph_test_schemes.prtcl restates procedures of the
reference's schemes with the oracle's operation order; their generated
kernels must give the oracle's fields bit for bit.  FP64 reductions agree
to rounding; dimension loops, min / max / count reductions, slices, `_`
neighbour loops and group selectors are checked against numpy."""
import os

import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise, both_scenes

pytestmark = pytest.mark.gpu

SRC = os.path.join(os.path.dirname(__file__), "dsl", "sph_test_schemes.prtcl")


@pytest.fixture(scope="module")
def generated(gpu_lib):
    from prtcl_gb300.dsl.build import compile_file
    names = compile_file(SRC)
    assert len(names) == 11
    return names


def fld(m, g, name, nc):
    return m.get_varying(g, name, nc)


@pytest.fixture
def pair(oracle_mod, generated):
    sc = scenes.dam_break(fluid_cells=(12, 14, 10), spacing=0.025, box=(0.6, 0.5, 0.4))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    d, o = both_scenes(sc, p, oracle_mod)
    rng = np.random.default_rng(4)
    v = (rng.standard_normal((len(sc["fluid"]), 3)) * 0.3).astype(np.float32)
    for m in (d, o):
        m.set_varying("f", "velocity", v)
        m.update()
    return d, o, sc


def test_density_and_volume(pair):
    d, o, _ = pair
    d.run("t_density", "compute_density")
    o.run("density", "compute_density")
    assert_bitwise(fld(d, "f", "density", 1), fld(o, "f", "density", 1), "density")
    d.run("t_volume", "compute_volume")
    o.run("aiast12", "compute_volume")
    assert_bitwise(fld(d, "b", "volume", 1), fld(o, "b", "volume", 1), "volume")


def test_sesph(pair):
    d, o, _ = pair
    d.scheme("t_sesph")  # loaded: adds the compressibility uniform
    for m in (d, o):
        m.set_uniform("f", "compressibility", 1000.0)
        m.set_varying("f", "acceleration", np.full((len(fld(o, "f", "density", 1)), 3), 0.5, np.float32))
    d.run("t_sesph", "compute_density_and_pressure")
    o.run("sesph", "compute_density_and_pressure")
    assert_bitwise(fld(d, "f", "density", 1), fld(o, "f", "density", 1), "density")
    assert_bitwise(fld(d, "f", "pressure", 1), fld(o, "f", "pressure", 1), "pressure")
    assert (fld(d, "f", "pressure", 1) > 0).any()
    d.run("t_sesph", "accumulate_acceleration")
    o.run("sesph", "accumulate_acceleration")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "acceleration")


def test_iisph(pair):
    d, o, _ = pair
    for m in (d, o):
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
    d.run("t_iisph", "setup")
    o.run("iisph", "setup")
    for name, nc in (("iisph_helper_c", 3), ("iisph_source_term", 1), ("iisph_diagonal_element", 1),
                     ("pressure", 1)):
        assert_bitwise(fld(d, "f", name, nc), fld(o, "f", name, nc), name)
    assert int(d.get_global("iisph_nprde")) == int(o.get_global("iisph_nprde"))
    for it in range(3):
        for m in (d, o):
            m.set_global("iisph_aprde", 0.0)
        d.run("t_iisph", "iteration_pressure_acceleration")
        o.run("iisph", "iteration_pressure_acceleration")
        d.run("t_iisph", "iteration_pressure")
        o.run("iisph", "iteration_pressure")
        for name, nc in (("acceleration", 3), ("iisph_right_hand_side", 1), ("pressure", 1)):
            assert_bitwise(fld(d, "f", name, nc), fld(o, "f", name, nc), f"{name} {it}")
        ad, ao = float(d.get_global("iisph_aprde")), float(o.get_global("iisph_aprde"))
        # FP64 partial sums in block order against the oracle's sequential FP64 sum
        assert abs(ad - ao) <= 1e-6 * max(1.0, abs(ao)), (ad, ao)


def test_motion_and_viscosity(pair):
    d, o, _ = pair
    for m in (d, o):
        m.run("density", "compute_density")
        m.set_global("maximum_speed", 0.0)
    d.run("t_motion", "initialize_acceleration")
    o.run("gravity", "initialize_acceleration")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "gravity")
    d.run("t_viscosity", "accumulate_acceleration")
    o.run("viscosity", "accumulate_acceleration")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "viscosity")
    d.run("t_motion", "integrate_velocity_with_hard_fade")
    o.run("symplectic_euler", "integrate_velocity_with_hard_fade")
    assert_bitwise(fld(d, "f", "velocity", 3), fld(o, "f", "velocity", 3), "velocity")
    d.run("t_motion", "integrate_position")
    o.run("symplectic_euler", "integrate_position")
    assert_bitwise(fld(d, "f", "position", 3), fld(o, "f", "position", 3), "position")
    # max= reductions are exact
    assert np.float32(d.get_global("maximum_speed")) == np.float32(o.get_global("maximum_speed"))


def test_bounds_tally_and_own_group_loops(pair):
    d, o, sc = pair
    d.scheme("t_bounds")
    d.set_global("bounds_padding", 0.125)
    d.run("t_bounds", "update")
    x = fld(d, "f", "position", 3).astype(np.float32)
    pad = np.float32(0.125)
    np.testing.assert_array_equal(np.asarray(d.get_global("bounds_min"), np.float32), x.min(0) - pad)
    np.testing.assert_array_equal(np.asarray(d.get_global("bounds_max"), np.float32), x.max(0) + pad)

    d.run("t_tally", "tally")
    m = fld(d, "f", "mass", 1).astype(np.float64)
    assert int(d.get_global("fluid_items")) == len(m)
    assert abs(float(d.get_global("total_mass")) - m.sum()) <= 1e-6 * m.sum()

    d.run("t_tally", "count_neighbours")
    n = len(m)
    offs, _ = o.neighbor_lists(1, 1, n)  # fluid (group 1) towards fluid
    np.testing.assert_array_equal(fld(d, "f", "neighbour_count", 1).astype(np.int64), np.diff(offs))
    np.testing.assert_array_equal(fld(d, "f", "height", 1), x[:, 1])


def test_group_selectors(pair):
    d, _, _ = pair
    v0 = fld(d, "b", "volume", 1).copy()
    d.run("t_selectors", "mark")
    np.testing.assert_array_equal(fld(d, "b", "volume", 1), v0 * np.float32(2))
    assert (fld(d, "f", "marker", 1) == 1).all()
    # tagging the boundary group changes which groups the selectors take
    d.add_tag("b", "frozen")
    d.run("t_selectors", "mark")
    np.testing.assert_array_equal(fld(d, "b", "volume", 1), v0 * np.float32(2))
    assert (fld(d, "b", "marker", 1) == 1).all()


def test_wkbb18_pcg(pair):
    """A generated solve pcg: WKBB18's implicit viscosity against the
    oracle's FP64-mode solver, fields and iteration count exact."""
    d, o, _ = pair
    for m in (d, o):
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
    d.run("t_wkbb18", "compute_diagonal")
    o.run("wkbb18", "compute_diagonal")
    assert_bitwise(fld(d, "f", "wkbb18_system_diagonal", 9), fld(o, "f", "wkbb18_system_diagonal", 9), "sp")
    d.run("t_wkbb18", "accumulate_acceleration")
    o.run("wkbb18", "accumulate_acceleration")
    it = int(d.get_uniform("f", "wkbb18_iterations"))
    assert it == int(o.get_uniform("f", "wkbb18_iterations")) and it >= 1
    assert_bitwise(fld(d, "f", "wkbb18_velocity_delta", 3), fld(o, "f", "wkbb18_velocity_delta", 3), "vd")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "viscous accel")


def test_scalar_pcg(pair):
    d, _, sc = pair
    n = len(sc["fluid"])
    src = np.random.default_rng(2).standard_normal(n).astype(np.float32)
    d.scheme("t_scalar_pcg")
    d.set_varying("f", "scalar_source", src)
    d.set_uniform("f", "scalar_pcg_error", 1e-6)
    d.set_uniform("f", "scalar_pcg_iterations_max", 10)
    d.run("t_scalar_pcg", "solve")
    np.testing.assert_array_equal(fld(d, "f", "scalar_solution", 1), src * np.float32(0.5))
    assert int(d.get_uniform("f", "scalar_pcg_iterations")) == 1


def test_unknown_generated_procedure(generated, gpu_lib):
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300.core import DeviceScene
    d = DeviceScene()
    d.add_group("f", "fluid")
    d.resize("f", 4)
    d.set_varying("f", "position", np.zeros((4, 3), np.float32))
    with pytest.raises(PrtclGpuError, match="procedure does not exist"):
        d.run("t_density", "no_such_procedure")
