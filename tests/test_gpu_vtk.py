"""Frame output: a group as a legacy ASCII VTK file, the reference's SaveVTK
format (util/save_vtk.cpp:57-128), compared line by line with a rendering of
that format from the same values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def render(name, type_, n, f):
    out = ["# vtk DataFile Version 2.0", f"{name} {type_}", "ASCII", "DATASET POLYDATA", f"POINTS {n} float"]

    def rows(a):
        a = np.asarray(a, np.float32).reshape(n, -1)
        return [" ".join("%f" % float(v) for v in r) for r in a]

    out += rows(f["position"])
    out.append(f"POINT_DATA {n}")
    for k in ("velocity", "acceleration"):
        if k in f:
            out += [f"VECTORS {k} float"] + rows(f[k])
    out += ["SCALARS _index float 1", "LOOKUP_TABLE default"] + [str(i) for i in range(n)]
    for k in ("mass", "volume", "density", "pressure", "time_of_birth", "implicit_function"):
        if k in f:
            out += [f"SCALARS {k} float 1", "LOOKUP_TABLE default"] + rows(f[k])
    return "\n".join(out) + "\n"


def test_save_vtk_matches_reference_format(tmp_path):
    from prtcl_gb300.core import Model
    rng = np.random.default_rng(3)
    m = Model()
    g = m.add_group("f", "fluid")
    n = 11
    g.resize(n)
    vals = {"position": (rng.standard_normal((n, 3)) * 3).astype(np.float32),
            "velocity": rng.standard_normal((n, 3)).astype(np.float32),
            "density": (1000 + rng.standard_normal(n)).astype(np.float32),
            "mass": rng.random(n).astype(np.float32),
            "pressure": np.linspace(-1e-3, 1e4, n).astype(np.float32)}
    for k, v in vals.items():
        g.varying.add_field(k, "f32", (3,) if v.ndim == 2 else ())
        g.varying.get_field(k).upload(v)
    path = tmp_path / "f.0.vtk"
    g.save_vtk(path)
    assert path.read_text() == render("f", "fluid", n, vals)


def test_save_vtk_needs_positions(tmp_path):
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300.core import Model
    m = Model()
    g = m.add_group("b", "boundary")
    g.resize(2)
    with pytest.raises(PrtclGpuError, match="no position field"):
        g.save_vtk(tmp_path / "b.vtk")
