"""Batched scenes (prtcl_gpu_batch_*): a scene's results are the same, bit
for bit, alone and in a mix of scenes that are added and removed around it;
a batch of one matches the plain single-scene path; every scene converges on
its own."""
import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import assert_bitwise

pytestmark = pytest.mark.gpu

P = dict(driver.DAM_BREAK_27K, viscosity=True)
FIELDS = ("position", "velocity", "density", "pressure", "acceleration")


def small(cells, box):
    return scenes.dam_break(fluid_cells=cells, spacing=0.025, box=box)


A = ((8, 9, 7), (0.4, 0.5, 0.35))
B = ((12, 6, 10), (0.6, 0.3, 0.5))
C = ((5, 5, 5), (0.25, 0.25, 0.25))
D = ((10, 10, 10), (0.5, 0.5, 0.5))


def run_alone(spec, steps):
    from prtcl_gb300.batch import Batch
    sc = small(*spec)
    bt = Batch(P)
    sid = bt.add_scene(sc["fluid"], sc["boundary"])
    bt.step(steps)
    return {f: bt.download(sid, f) for f in FIELDS}, bt.info(sid)


def test_same_alone_and_in_the_mix():
    from prtcl_gb300.batch import Batch
    K = 20
    alone, ia = run_alone(A, K)
    bt = Batch(P)
    sb = small(*B)
    idb = bt.add_scene(sb["fluid"], sb["boundary"])
    bt.step(3)
    sa, sc_, sd = small(*A), small(*C), small(*D)
    ida = bt.add_scene(sa["fluid"], sa["boundary"])
    idc = bt.add_scene(sc_["fluid"], sc_["boundary"])
    bt.step(9)                       # A: 9 steps, permuted at its 8th
    bt.remove_scene(idb)             # ranges below A's move
    idd = bt.add_scene(sd["fluid"], sd["boundary"])  # takes B's slot
    bt.step(K - 9)
    assert bt.scene_count == 3
    ib = bt.info(ida)
    assert ib["steps"] == K
    for f in FIELDS:
        assert_bitwise(bt.download(ida, f), alone[f], f"scene A {f}")
    for k in ("jacobi_solves", "jacobi_iterations", "jacobi_capped", "max_relative_density_error",
              "pcg_solves", "pcg_iterations", "last_jacobi_iterations", "last_pcg_iterations"):
        assert ib[k] == ia[k], k
    # the others advanced too, and converge on their own
    for sid, steps in ((idc, K), (idd, K - 9)):
        i = bt.info(sid)
        assert i["steps"] == steps and i["jacobi_solves"] == steps
        assert i["jacobi_capped"] == 0 or i["max_relative_density_error"] >= P["eta"]


def test_batch_of_one_matches_plain_path():
    from prtcl_gb300.core import DeviceScene
    K = 12
    sc = small(*A)
    alone, ia = run_alone(A, K)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, P)
    loop = driver.StepLoop(d, P, device_loop=True)
    its = [loop.step() for _ in range(K)]
    # the same neighbour order and arithmetic; only the FP64 reduction order
    # of the convergence sums differs (per tile instead of per grid block)
    assert ia["jacobi_iterations"] == sum(s["jacobi_iterations"] for s in its)
    assert ia["last_pcg_iterations"] == its[-1]["pcg_iterations"]
    for f, tol in (("position", 1e-6), ("velocity", 1e-4), ("density", 1e-5), ("pressure", 1e-3)):
        a, b = alone[f].astype(np.float64), d.get_varying("f", f).astype(np.float64).reshape(alone[f].shape)
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err <= tol, (f, err)


def test_every_scene_converges_on_its_own():
    from prtcl_gb300.batch import Batch
    bt = Batch(P)
    ids = []
    for k, sc in enumerate(scenes.mixed_batch(count=6, lo=300, hi=4000, seed=11)):
        ids.append(bt.add_scene(sc["fluid"], sc["boundary"]))
    bt.step(10)
    nf, nb = bt.particles()
    assert nf > 0 and nb > 0 and bt.device_bytes() > 0
    for sid in ids:
        i = bt.info(sid)
        assert i["jacobi_solves"] == 10 and i["pcg_solves"] == 10
        assert i["jacobi_iterations"] >= 2 * 10
        # each solve ends converged (rel < eta) unless it hit the cap
        if i["jacobi_capped"] == 0:
            assert i["max_relative_density_error"] < P["eta"]


def test_errors():
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300.batch import Batch
    bt = Batch(P)
    sc = small(*C)
    sid = bt.add_scene(sc["fluid"], sc["boundary"])
    with pytest.raises(PrtclGpuError, match="no scene"):
        bt.remove_scene(sid + 100)
    with pytest.raises(PrtclGpuError, match="does not exist"):
        bt.download(sid, "no_such_field")
    bt.remove_scene(sid)
    assert bt.scene_count == 0
    bt.step(2)  # an empty batch steps its clock only
    assert bt.particles() == (0, 0)
