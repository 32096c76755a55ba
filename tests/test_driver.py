"""The native driver prtcl_gb300/bin/prtcl_gpu_run (host C++ over the C++
facade include/prtcl_gpu.hpp): on the GPU it must reproduce the Python step
loop bit for bit, starting from a model archive; on the CPU its argument
handling and its failure without a device are checked."""
import os
import subprocess

import numpy as np
import pytest

from prtcl_gb300 import build, driver, scenes

DRIVER = os.path.join(os.path.dirname(build.__file__), "bin", "prtcl_gpu_run")


@pytest.fixture(scope="module")
def exe(gpu_lib):
    assert os.path.exists(DRIVER)
    return DRIVER


def test_usage(exe):
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_fails_cleanly_without_input(exe, tmp_path):
    r = subprocess.run([exe, str(tmp_path / "missing.bin"), "1", str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and r.stderr.startswith("prtcl_gpu_run:")


@pytest.mark.gpu
def test_native_driver_matches_python_loop(exe, tmp_path):
    from prtcl_gb300.core import DeviceScene, Model
    sc = scenes.dam_break(fluid_cells=(10, 12, 8), spacing=0.025, box=(0.5, 0.4, 0.4))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    start = tmp_path / "model.0.bin"
    d.model.save(start)
    steps = 10
    r = subprocess.run([exe, str(start), str(steps), str(tmp_path / "model.10.bin"), "--viscosity",
                        "--vtk-every", "5", "--vtk-prefix", str(tmp_path / "frame")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("step")]
    assert len(lines) == steps
    loop = driver.StepLoop(d, p, device_loop=True)
    stats = [loop.step() for _ in range(steps)]
    for line, st in zip(lines, stats):
        f = line.split()
        assert int(f[5]) == st["jacobi_iterations"] and int(f[7]) == st["pcg_iterations"]
    m = Model()
    m.load(tmp_path / "model.10.bin")
    for name in ("position", "velocity", "density", "pressure", "acceleration"):
        a = d.model.get_group("f").varying.get_field(name).download()
        b = m.get_group("f").varying.get_field(name).download()
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32)), name
    assert (tmp_path / "frame.f.10.vtk").exists() and (tmp_path / "frame.b.5.vtk").exists()
