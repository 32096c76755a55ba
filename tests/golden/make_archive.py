"""Generate model_small.bin, a model archive in the reference's native binary
format (util/archive.cpp:5-40; data/model.cpp:54-75), and model_small.npz
with its values.

The archive is written by the restatement below and then read back with the
reference's own reader (share/python/prtcl_archive.py, load_model), which
must return exactly the values written.  That module imports matplotlib for
its plotting helpers; a stand-in module is installed for the import.

Run:  python tests/golden/make_archive.py   (needs the reference checkout)
"""
import os
import struct
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def reference_python():
    """share/python of the reference checkout (located by oracle/Makefile,
    PRTCL_REFERENCE overrides); exits with a message where it is absent."""
    from oracle import ref_build
    root = ref_build.reference_root()
    if not root:
        raise SystemExit("the reference checkout is needed: set PRTCL_REFERENCE")
    return os.path.join(root, "share", "python")


def w_size(f, v):
    f.write(struct.pack("<Q", v))


def w_str(f, s):
    b = s.encode()
    w_size(f, len(b))
    f.write(b)


def w_type(f, ctype, shape):
    w_str(f, ctype)
    w_size(f, len(shape))
    for e in shape:
        w_size(f, e)


DT = {"f32": "<f4", "s32": "<i4"}


def model():
    rng = np.random.default_rng(17)
    g = {
        "globals": {"gravity": ("f32", [3], np.array([0.0, -9.81, 0.0], np.float32)),
                    "iisph_maximum_iterations": ("s32", [], np.array(100, np.int32)),
                    "smoothing_scale": ("f32", [], np.array(0.025, np.float32))},
        "groups": {
            "b": {"type": "boundary", "tags": [], "count": 5,
                  "varying": {"position": ("f32", [3], rng.standard_normal((5, 3)).astype(np.float32)),
                              "volume": ("f32", [], rng.random(5).astype(np.float32))},
                  "uniform": {"dynamic_viscosity": ("f32", [], np.array(10.0, np.float32))}},
            "f": {"type": "fluid", "tags": ["dynamic"], "count": 7,
                  "varying": {"mass": ("f32", [], rng.random(7).astype(np.float32)),
                              "position": ("f32", [3], rng.standard_normal((7, 3)).astype(np.float32)),
                              "velocity": ("f32", [3], rng.standard_normal((7, 3)).astype(np.float32)),
                              "wkbb18_iterations_item": ("s32", [], rng.integers(-5, 5, 7).astype(np.int32)),
                              "wkbb18_system_diagonal": ("f32", [3, 3],
                                                         rng.standard_normal((7, 3, 3)).astype(np.float32))},
                  "uniform": {"rest_density": ("f32", [], np.array(1000.0, np.float32)),
                              "wkbb18_maximum_iterations": ("s32", [], np.array(100, np.int32))}},
        },
    }
    return g


def values_bytes(ctype, arr, matrix_items=False):
    a = np.asarray(arr)
    if matrix_items:  # items of 3x3 matrices, column-major per item
        a = np.transpose(a, (0, 2, 1))
    return np.ascontiguousarray(a, DT[ctype]).tobytes()


def write(path, m):
    with open(path, "wb") as f:
        w_size(f, len(m["globals"]))
        for name, (ct, shape, v) in sorted(m["globals"].items()):
            w_str(f, name)
            w_type(f, ct, shape)
            f.write(values_bytes(ct, v))
        w_size(f, len(m["groups"]))
        for gname, g in sorted(m["groups"].items()):
            w_str(f, gname)
            w_str(f, g["type"])
            w_size(f, len(g["tags"]))
            for t in sorted(g["tags"]):
                w_str(f, t)
            w_size(f, g["count"])
            w_size(f, len(g["varying"]))
            for name, (ct, shape, v) in sorted(g["varying"].items()):
                w_str(f, name)
                w_type(f, ct, shape)
                w_size(f, g["count"])
                f.write(values_bytes(ct, v, matrix_items=(len(shape) == 2)))
            w_size(f, len(g["uniform"]))
            for name, (ct, shape, v) in sorted(g["uniform"].items()):
                w_str(f, name)
                w_type(f, ct, shape)
                f.write(values_bytes(ct, v))


def check_with_reference(path, m):
    sys.modules.setdefault("matplotlib", types.ModuleType("matplotlib"))
    sys.modules.setdefault("matplotlib.pyplot", types.ModuleType("matplotlib.pyplot"))
    sys.path.insert(0, reference_python())
    import prtcl_archive
    with open(path, "rb") as f:
        r = prtcl_archive.load_model(f)
    for name, (ct, shape, v) in m["globals"].items():
        np.testing.assert_array_equal(r["global_fields"][name]["data"].reshape(v.shape), v)
    for gname, g in m["groups"].items():
        rg = r["groups"][gname]
        assert rg["type"] == g["type"] and rg["tags"] == sorted(g["tags"])
        for name, (ct, shape, v) in g["varying"].items():
            got = rg["varying_fields"][name]["data"]
            if len(shape) == 2:  # the reader reshapes the column-major items row-major
                got = np.transpose(got.reshape(g["count"], 3, 3), (0, 2, 1))
            np.testing.assert_array_equal(got.reshape(v.shape), v)
        for name, (ct, shape, v) in g["uniform"].items():
            np.testing.assert_array_equal(rg["uniform_fields"][name]["data"].reshape(v.shape), v)


def main():
    m = model()
    path = os.path.join(HERE, "model_small.bin")
    write(path, m)
    check_with_reference(path, m)
    flat = {}
    for name, (ct, shape, v) in m["globals"].items():
        flat["global/" + name] = v
    for gname, g in m["groups"].items():
        for name, (ct, shape, v) in g["varying"].items():
            # host layout of the C ABI: items x components, matrices column-major
            flat[f"{gname}/varying/{name}"] = (np.transpose(v, (0, 2, 1)).reshape(g["count"], 9)
                                               if len(shape) == 2 else v)
        for name, (ct, shape, v) in g["uniform"].items():
            flat[f"{gname}/uniform/{name}"] = v
    np.savez(os.path.join(HERE, "model_small.npz"), **flat)
    print("wrote", path, os.path.getsize(path), "bytes; the reference's reader agrees")


if __name__ == "__main__":
    main()
