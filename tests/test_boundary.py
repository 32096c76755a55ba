"""The C-ABI boundary without a GPU: the library loads, exports every entry
point include/prtcl_gpu.h declares, answers registry queries, and reports
unknown names the way the reference does; the C++ facade compiles."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from prtcl_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "prtcl_gpu.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(prtcl_gpu_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = declared()
    assert len(names) > 30
    from prtcl_gb300 import _lib
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert not [n for n in names if n not in _lib.SIGNATURES]


def test_registry_and_errors_without_device(gpu_lib):
    from prtcl_gb300 import PrtclNotFound
    from prtcl_gb300.core import get_scheme_names, make_scheme
    names = get_scheme_names()
    for s in ("aiast12", "correction", "density", "gravity", "iisph", "symplectic_euler", "viscosity", "wkbb18",
              "wkbb18_gc"):
        assert f"prtcl::schemes::{s}[T=f32, N=3, K=Cubic Spline]" in names
    with pytest.raises(PrtclNotFound, match="scheme is not registered"):
        make_scheme("prtcl::schemes::sesph[T=f32, N=3, K=Cubic Spline]")
    sch = make_scheme("prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]")
    assert sch.get_full_name() == "prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]"
    assert sorted(sch.get_procedure_names()) == ["iteration_pressure", "iteration_pressure_acceleration",
                                                 "setup", "solve_pressure"]
    # running a procedure before Load is an error, not a crash
    from prtcl_gb300 import PrtclGpuError
    lib = gpu_lib
    h = C.c_void_p()
    assert lib.prtcl_gpu_scheme_new(b"prtcl::schemes::density[T=f32, N=3, K=Cubic Spline]", C.byref(h)) == 0
    assert lib.prtcl_gpu_scheme_run(h, b"no_such_procedure", C.c_void_p(1), None) == -2
    assert b"procedure does not exist" in lib.prtcl_gpu_last_error()
    assert lib.prtcl_gpu_scheme_run(h, b"compute_density", None, None) == -3  # null neighbourhood
    lib.prtcl_gpu_scheme_destroy(h)


def test_no_cpu_fallback(gpu_lib):
    """Without a device the product path fails loudly."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300.core import Model
    with pytest.raises(PrtclGpuError):
        Model()
    from prtcl_gb300 import driver
    from prtcl_gb300.batch import Batch
    with pytest.raises(PrtclGpuError):
        Batch(driver.DAM_BREAK_27K)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_facade_compiles(tmp_path, gpu_lib):
    """Driver code over the façade compiles and links against the library
    (not run: no device here)."""
    src = tmp_path / "use.cpp"
    src.write_text('#include "prtcl_gpu.hpp"\n'
                   'int main() { prtcl_gpu::Model m; auto f = m.AddGroup("f", "fluid"); f.AddTag("dynamic");\n'
                   '  prtcl_gpu::Neighborhood n; n.Load(m); n.SetRadius(0.05); n.Update();\n'
                   '  auto s = prtcl_gpu::SchemeRegistry::NewScheme("prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]");\n'
                   '  s->Load(m); s->RunProcedure("setup", n);\n'
                   '  prtcl_gpu_batch_params bp{}; prtcl_gpu_server_params sp{}; sp.max_scenes = 8;\n'
                   '  prtcl_gpu::Batch b(bp); auto id = b.AddScene({0, 0, 0}, {}); b.Step(); b.Positions(id);\n'
                   '  prtcl_gpu::Server srv(bp, sp); srv.Submit(1, 0.0, {0, 0, 0}, {}, 2);\n'
                   '  while (srv.Turn()) srv.TakeResults();\n'
                   '  return int(srv.Status().pending); }\n')
    lib_dir = os.path.dirname(gpu_lib._name)
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "use"), "-L", lib_dir, "-lprtcl_gpu", "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_dam_break_scene_sizes():
    sc = scenes.dam_break()
    assert len(sc["fluid"]) == 27000 and len(sc["boundary"]) == 34624
    assert sc["fluid"].dtype.name == "float32"
    # fluid inside the box, walls outside
    assert (sc["fluid"] > 0).all()
    b = sc["boundary"]
    inside = (b[:, 0] > 0) & (b[:, 0] < 2) & (b[:, 1] > 0) & (b[:, 1] < 1) & (b[:, 2] > 0) & (b[:, 2] < 1)
    assert not inside.any()
