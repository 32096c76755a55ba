"""Native binary model archives (prtcl_gpu_model_save / _load) against the
fixture tests/golden/model_small.bin, which the reference's own reader
(share/python/prtcl_archive.py) reads back exactly (tests/golden/
make_archive.py)."""
import os

import numpy as np
import pytest

from prtcl_gb300 import driver, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BIN = os.path.join(GOLDEN, "model_small.bin")


def expected():
    return dict(np.load(os.path.join(GOLDEN, "model_small.npz")))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_load_reference_format_archive():
    from prtcl_gb300.core import Model
    m = Model()
    m.load(BIN)
    assert m.group_names() == ["b", "f"]
    for key, v in expected().items():
        parts = key.split("/")
        if parts[0] == "global":
            got = np.asarray(m.global_.get_field(parts[1]).get())
            assert np.array_equal(got.reshape(np.shape(v)).astype(v.dtype), v), key
            continue
        g, kind, name = parts
        grp = m.get_group(g)
        if kind == "varying":
            got = grp.varying.get_field(name).download()
            assert np.array_equal(bits(got.reshape(v.shape)), bits(v)), key
        else:
            got = np.asarray(grp.uniform.get_field(name).get())
            assert np.array_equal(bits(got.reshape(np.shape(v)).astype(v.dtype)), bits(np.asarray(v))), key
    assert m.get_group("f").index == 1 and m.get_group("b").item_count == 5


def test_save_reproduces_the_archive_bytes(tmp_path):
    from prtcl_gb300.core import Model
    m = Model()
    m.load(BIN)
    out = tmp_path / "again.bin"
    m.save(out)
    assert out.read_bytes() == open(BIN, "rb").read()


def test_dam_break_state_round_trip(tmp_path):
    from prtcl_gb300.core import DeviceScene, Model
    sc = scenes.dam_break(fluid_cells=(10, 10, 10), spacing=0.025, box=(0.5, 0.5, 0.5))
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    loop = driver.StepLoop(d, p, device_loop=True)
    for _ in range(3):
        loop.step()
    path = tmp_path / "model.3.bin"
    d.model.save(path)
    m = Model()
    m.load(path)
    for g in ("b", "f"):
        src, dst = d.model.get_group(g), m.get_group(g)
        assert dst.item_count == src.item_count
        for name in ("position", "velocity", "density", "pressure", "volume", "mass"):
            if not src.varying.has_field(name):
                continue
            a = src.varying.get_field(name).download()
            b = dst.varying.get_field(name).download()
            assert np.array_equal(bits(a), bits(b)), (g, name)


def test_corrupt_and_unsupported_archives(tmp_path):
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300.core import Model
    data = open(BIN, "rb").read()
    short = tmp_path / "short.bin"
    short.write_bytes(data[: len(data) // 2])
    with pytest.raises(PrtclGpuError, match="truncated"):
        Model().load(short)
    f64 = tmp_path / "f64.bin"
    f64.write_bytes(data.replace(b"f32", b"f64", 1))
    with pytest.raises(PrtclGpuError, match="component type 'f64'"):
        Model().load(f64)
    with pytest.raises(PrtclGpuError, match="cannot read"):
        Model().load(tmp_path / "missing.bin")
