"""The reference's own scheme sources, generated into CUDA and run on the
device, against the oracle and the hand-written schemes.

tests/golden/reference_schemes_plugin.cu is what prtcl_gb300.dsl emits for
the reference's share/schemes/{aiast12, density, gravity, iisph,
symplectic_euler, wkbb18}.prtcl, unmodified (schemes renamed ref_<name>;
tests/golden/make_reference_schemes.py, checked against the live sources by
tests/test_dsl.py).  Those texts are what the reference's generated
src/prtcl/schemes/*.hpp come from, and the oracle restates the generated
C++ (iisph.hpp:188-516, wkbb18.hpp:194-425, cg_openmp.hpp:35-215, ...).

A dam break of a few thousand particles with random velocities runs the
reference driver's step (share/scripts/prtcl-lua.example.lua:363-461, the
relaxed-Jacobi loop on the host) twice on three models: the generated
reference schemes, the hand-written schemes and the oracle (f32, FP64
convergence reductions).  After every procedure each field it writes must
be bit-identical across all three, and the Jacobi and PCG iteration counts
equal.
"""
import json
import os

import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def reference_schemes(gpu_lib):
    from prtcl_gb300.dsl.build import load_plugin_source
    with open(os.path.join(GOLDEN, "reference_schemes_plugin.json")) as f:
        names = json.load(f)["schemes"]
    with open(os.path.join(GOLDEN, "reference_schemes_plugin.cu")) as f:
        cu = f.read()
    return load_plugin_source(names, cu)


class Renamed:
    """The flat model API of a device scene whose procedures run through
    the schemes named ``prefix + name``."""

    def __init__(self, m, prefix):
        self._m, self._prefix = m, prefix

    def __getattr__(self, k):
        return getattr(self._m, k)

    def run(self, scheme, procedure):
        self._m.run(self._prefix + scheme, procedure)


STEP = [
    ("density", "compute_density", [("density", 1)]),
    ("gravity", "initialize_acceleration", [("acceleration", 3)]),
    ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
    ("iisph", "setup", [("iisph_helper_c", 3), ("iisph_source_term", 1), ("iisph_diagonal_element", 1),
                        ("pressure", 1)]),
    ("jacobi", None, [("acceleration", 3), ("iisph_right_hand_side", 1), ("pressure", 1)]),
    ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
    ("wkbb18", "compute_diagonal", [("wkbb18_system_diagonal", 9)]),
    ("wkbb18", "accumulate_acceleration", [("wkbb18_velocity_delta", 3), ("acceleration", 3)]),
    ("symplectic_euler", "integrate_velocity_with_hard_fade", [("velocity", 3)]),
    ("symplectic_euler", "integrate_position", [("position", 3)]),
]


def _same(models, group, fields, what):
    o = models[-1]
    for name, nc in fields:
        ref = o.get_varying(group, name, nc)
        for m, label in zip(models[:-1], ("generated reference scheme", "hand-written scheme")):
            assert_bitwise(m.get_varying(group, name, nc), ref, f"{what}: {group}.{name} ({label})")


def _jacobi(m, p):
    """The script's relaxed-Jacobi loop (prtcl-lua.example.lua:404-423)."""
    nprde = m.get_global("iisph_nprde")
    it, sums = 0, []
    if nprde >= 1:
        for it in range(1, p["max_iters"] + 1):
            m.set_global("iisph_aprde", 0.0)
            m.run("iisph", "iteration_pressure_acceleration")
            m.run("iisph", "iteration_pressure")
            sums.append(m.get_global("iisph_aprde"))
            if it >= 2 and sums[-1] / nprde < p["eta"]:
                break
    return it, sums


def test_reference_scheme_text_on_device(oracle_mod, reference_schemes):
    from prtcl_gb300.core import DeviceScene
    sc = scenes.dam_break(fluid_cells=(14, 16, 12), spacing=0.025, box=(0.7, 0.6, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    gen, hw = DeviceScene(), DeviceScene()
    o = oracle_mod.Scene(np.float32, fp64_reductions=True)
    models = [Renamed(gen, "ref_"), hw, o]
    for m in models:
        driver.setup_dam_break(m, sc, p)
    _same(models, "b", [("volume", 1)], "aiast12.compute_volume")
    v = (np.random.default_rng(6).standard_normal((len(sc["fluid"]), 3)) * 0.3).astype(np.float32)
    for m in models:
        m.set_varying("f", "velocity", v)
    dt = float(np.float32(p["time_step"]))
    for step in range(2):
        for m in models:
            m.set_global("current_time", float(np.float32(step * dt)))
            m.update()
            if step == 1:
                m.permute()
        for scheme, proc, fields in STEP:
            if scheme == "jacobi":
                res = [_jacobi(m, p) for m in models]
                its = [r[0] for r in res]
                assert its[0] == its[1] == its[2] and its[0] >= 2, its
                for a, b in zip(res[0][1], res[2][1]):
                    assert abs(a - b) <= 1e-6 * max(1.0, abs(b)), (a, b)
            else:
                for m in models:
                    m.run(scheme, proc)
            if proc == "setup":
                assert len({int(m.get_global("iisph_nprde")) for m in models}) == 1
            if proc == "accumulate_acceleration":
                its = [int(m.get_uniform("f", "wkbb18_iterations")) for m in models]
                assert its[0] == its[1] == its[2] and its[0] >= 1, its
            _same(models, "f", fields, f"step {step + 1} {scheme}.{proc or 'relaxed Jacobi loop'}")
        mx = [np.float32(m.get_global("maximum_speed")) for m in models]
        assert mx[0] == mx[1] == mx[2], mx
