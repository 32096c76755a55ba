"""Device procedures vs the oracle on identical inputs: every per-particle
field must be bit-identical (same FP32 operation order, no FMA); the FP64
reductions agree to double rounding."""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise, both_scenes

pytestmark = pytest.mark.gpu

V3 = ["position", "velocity", "acceleration"]


def fld(m, g, name, ncomp):
    return m.get_varying(g, name, ncomp)


@pytest.fixture(scope="module")
def pair(oracle_mod):
    sc = scenes.dam_break(fluid_cells=(16, 20, 12), spacing=0.025, box=(0.8, 0.7, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    d, o = both_scenes(sc, p, oracle_mod)
    # non-trivial velocities so that every term is exercised
    rng = np.random.default_rng(4)
    v = (rng.standard_normal((len(sc["fluid"]), 3)) * 0.3).astype(np.float32)
    d.set_varying("f", "velocity", v)
    o.set_varying("f", "velocity", v)
    return d, o


def test_boundary_volume(pair):
    d, o = pair
    assert_bitwise(fld(d, "b", "volume", 1), fld(o, "b", "volume", 1), "aiast12 volume")


def test_step_procedures_bitwise(pair):
    d, o = pair
    for m in (d, o):
        m.update()
        m.run("density", "compute_density")
    assert_bitwise(fld(d, "f", "density", 1), fld(o, "f", "density", 1), "density")
    for m in (d, o):
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
    assert_bitwise(fld(d, "f", "velocity", 3), fld(o, "f", "velocity", 3), "velocity")
    for m in (d, o):
        m.run("iisph", "setup")
    for name, nc in [("iisph_helper_c", 3), ("iisph_source_term", 1), ("iisph_diagonal_element", 1), ("pressure", 1)]:
        assert_bitwise(fld(d, "f", name, nc), fld(o, "f", name, nc), name)
    assert d.get_global("iisph_nprde") == o.get_global("iisph_nprde")
    for it in range(4):
        for m in (d, o):
            m.set_global("iisph_aprde", 0.0)
            m.run("iisph", "iteration_pressure_acceleration")
            m.run("iisph", "iteration_pressure")
        assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), f"pressure accel {it}")
        assert_bitwise(fld(d, "f", "iisph_right_hand_side", 1), fld(o, "f", "iisph_right_hand_side", 1), f"Ap {it}")
        assert_bitwise(fld(d, "f", "pressure", 1), fld(o, "f", "pressure", 1), f"pressure {it}")
        ad, ao = d.get_global("iisph_aprde"), o.get_global("iisph_aprde")
        # device stores the FP64 sum rounded to f32; oracle keeps the double
        assert abs(ad - ao) <= 1e-6 * max(1.0, abs(ao)), (ad, ao)
    for m in (d, o):
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("wkbb18", "compute_diagonal")
    assert_bitwise(fld(d, "f", "wkbb18_system_diagonal", 9), fld(o, "f", "wkbb18_system_diagonal", 9), "sp")
    for m in (d, o):
        m.run("wkbb18", "accumulate_acceleration")
    assert d.get_uniform("f", "wkbb18_iterations") == int(o.get_uniform("f", "wkbb18_iterations"))
    assert_bitwise(fld(d, "f", "wkbb18_velocity_delta", 3), fld(o, "f", "wkbb18_velocity_delta", 3), "vd")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "viscous accel")
    for m in (d, o):
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("symplectic_euler", "integrate_position")
    assert_bitwise(fld(d, "f", "position", 3), fld(o, "f", "position", 3), "position")
    assert d.get_global("maximum_speed") == np.float32(o.get_global("maximum_speed"))
    # explicit viscosity (viscosity.accumulate_acceleration) on top of gravity
    for m in (d, o):
        m.update()
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("viscosity", "accumulate_acceleration")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "explicit viscosity")
    # gradient correction (pseudo-inverse) and the gradient-corrected WKBB18
    for m in (d, o):
        m.run("correction", "identity_gradient_correction")
    eye = np.tile(np.eye(3, dtype=np.float32).reshape(1, 9), (fld(d, "f", "density", 1).shape[0], 1))
    assert_bitwise(fld(d, "f", "gradient_correction", 9), eye, "identity L")
    for m in (d, o):
        m.run("correction", "compute_gradient_correction")
    assert_bitwise(fld(d, "f", "gradient_correction", 9), fld(o, "f", "gradient_correction", 9), "L")
    for m in (d, o):
        m.run("wkbb18_gc", "compute_diagonal")
    assert_bitwise(fld(d, "f", "wkbb18_system_diagonal", 9), fld(o, "f", "wkbb18_system_diagonal", 9), "sp gc")
    for m in (d, o):
        m.run("wkbb18_gc", "accumulate_acceleration")
    assert d.get_uniform("f", "wkbb18_iterations") == int(o.get_uniform("f", "wkbb18_iterations"))
    assert_bitwise(fld(d, "f", "wkbb18_velocity_delta", 3), fld(o, "f", "wkbb18_velocity_delta", 3), "vd gc")
    assert_bitwise(fld(d, "f", "acceleration", 3), fld(o, "f", "acceleration", 3), "viscous accel gc")


def test_procedures_on_unpermuted_fluid(oracle_mod):
    """The fluid shuffled after set-up and not permuted again: neighbour
    indices are scattered, so the lists are stored as 32-bit indices beside
    their gradient factors; the sweeps must give the oracle's fields bit for
    bit all the same."""
    sc = scenes.dam_break(fluid_cells=(12, 14, 10), spacing=0.025, box=(0.6, 0.5, 0.4))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    d, o = both_scenes(sc, p, oracle_mod)
    nf = len(sc["fluid"])
    perm = np.random.default_rng(8).permutation(nf)
    v = (np.random.default_rng(9).standard_normal((nf, 3)) * 0.3).astype(np.float32)
    for m in (d, o):
        for name, nc in (("position", 3), ("mass", 1), ("time_of_birth", 1)):
            a = fld(o, "f", name, nc)
            m.set_varying("f", name, a[perm])
        m.set_varying("f", "velocity", v)
        m.update()
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("iisph", "setup")
        for it in range(3):
            m.set_global("iisph_aprde", 0.0)
            m.run("iisph", "iteration_pressure_acceleration")
            m.run("iisph", "iteration_pressure")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("wkbb18", "compute_diagonal")
        m.run("wkbb18", "accumulate_acceleration")
    for name, nc in (("density", 1), ("iisph_diagonal_element", 1), ("pressure", 1),
                     ("wkbb18_system_diagonal", 9), ("wkbb18_velocity_delta", 3), ("acceleration", 3)):
        assert_bitwise(fld(d, "f", name, nc), fld(o, "f", name, nc), name)
    assert d.get_uniform("f", "wkbb18_iterations") == int(o.get_uniform("f", "wkbb18_iterations"))


def test_unknown_procedure_and_scheme(pair):
    from prtcl_gb300 import PrtclNotFound
    from prtcl_gb300.core import make_scheme
    d, _ = pair
    with pytest.raises(PrtclNotFound, match="procedure does not exist"):
        d.run("iisph", "no_such_procedure")
    with pytest.raises(PrtclNotFound, match="scheme is not registered"):
        make_scheme("prtcl::schemes::iisph[T=f64, N=3, K=Cubic Spline]")


def test_solve_pressure_matches_host_loop(oracle_mod):
    """iisph.solve_pressure (device loop in a CUDA graph) == the script's
    host loop of iteration_pressure_acceleration + iteration_pressure."""
    sc = scenes.dam_break(fluid_cells=(14, 18, 10), spacing=0.025, box=(0.7, 0.6, 0.5))
    p = dict(driver.DAM_BREAK_27K)
    d1, o = both_scenes(sc, p, oracle_mod)
    from tests.helpers import both_scenes as _b
    d2, _ = _b(sc, p, oracle_mod)
    for m in (d1, d2, o):
        m.update()
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("iisph", "setup")
    s1 = driver.StepLoop(d1, p, device_loop=True)
    d1.run("iisph", "solve_pressure")
    o.run("iisph", "solve_pressure")
    it = int(d1.get_global("iisph_iterations"))
    assert it == int(o.get_global("iisph_iterations")) and it >= 2
    # host loop with the same number of iterations
    for k in range(it):
        d2.set_global("iisph_aprde", 0.0)
        d2.run("iisph", "iteration_pressure_acceleration")
        d2.run("iisph", "iteration_pressure")
    for name, nc in [("pressure", 1), ("acceleration", 3), ("iisph_right_hand_side", 1)]:
        assert_bitwise(fld(d1, "f", name, nc), fld(d2, "f", name, nc), name + " (device vs host loop)")
        assert_bitwise(fld(d1, "f", name, nc), fld(o, "f", name, nc), name + " (device vs oracle)")
