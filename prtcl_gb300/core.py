"""Host-side mirror of prtcl's model / neighbourhood / scheme API over the
C ABI of the CUDA library.

Names follow the reference's C++ API (data/model.hpp, util/neighborhood.hpp,
schemes/scheme_base.hpp) with the Lua binding's snake_case spellings
(src/prtcl-lua/module_data.cpp, module_schemes.cpp, module_util.cpp) as
aliases, so driver code reads like the reference's scripts:

    model = Model()
    f = model.add_group("f", "fluid"); f.add_tag("dynamic")
    iisph = make_scheme("prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]")
    iisph.load(model)
    nhood = Neighborhood(); nhood.load(model); nhood.set_radius(2 * h)
    nhood.update(); iisph.run_procedure("setup", nhood)

Errors raise ``PrtclGpuError``; unknown procedure / scheme / field names
raise ``PrtclNotFound`` ("procedure does not exist", "scheme is not
registered"), where the reference throws a string.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import PrtclGpuError, PrtclNotFound, b, check, load, read_str

REAL = np.float32
INTEGER = np.int32


def _type_of(ctype, rank, ext):
    dt = REAL if ctype == "f32" else INTEGER
    shape = tuple(int(e) for e in ext[:rank])
    return dt, shape


def _ext_arr(shape):
    a = (C.c_int32 * 2)(*(list(shape) + [1, 1])[:2])
    return a


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return C.c_void_p(s)
    h = getattr(s, "cuda_stream", None) or getattr(s, "handle", None)
    return C.c_void_p(int(h)) if h is not None else None


class _Value:
    """A uniform or global field reference (get / set of one value)."""

    def __init__(self, model, group, name):
        self._m, self._g, self._n = model, group, name
        self._type = None

    def _info(self):
        ct = C.create_string_buffer(8)
        rank = C.c_int32(0)
        ext = (C.c_int32 * 2)()
        L = load()
        if self._g is None:
            check(L.prtcl_gpu_global_info(self._m._h, b(self._n), ct, C.byref(rank), ext))
        else:
            check(L.prtcl_gpu_uniform_info(self._m._h, b(self._g), b(self._n), ct, C.byref(rank), ext))
        return _type_of(ct.value.decode(), rank.value, list(ext))

    def get(self):
        dt, shape = self._info()
        out = np.zeros(max(1, int(np.prod(shape))), dtype=dt)
        L = load()
        if self._g is None:
            check(L.prtcl_gpu_global_get(self._m._h, b(self._n), out.ctypes.data))
        else:
            check(L.prtcl_gpu_uniform_get(self._m._h, b(self._g), b(self._n), out.ctypes.data))
        if not shape:
            return out[0].item()
        return out.reshape(shape, order="F")

    def set(self, value, asynchronous=False, stream=None):
        dt, shape = self._info() if self._type is None else self._type
        self._type = (dt, shape)
        a = np.asarray(value, dtype=dt)
        if a.size != max(1, int(np.prod(shape))):
            raise PrtclGpuError(f"value of size {a.size} for field {self._n} of shape {shape}")
        a = np.ascontiguousarray(a.reshape(-1, order="F"))
        L = load()
        if self._g is None and asynchronous:
            check(L.prtcl_gpu_global_set_async(self._m._h, b(self._n), a.ctypes.data, _stream(stream)))
        elif self._g is None:
            check(L.prtcl_gpu_global_set(self._m._h, b(self._n), a.ctypes.data))
        else:
            check(L.prtcl_gpu_uniform_set(self._m._h, b(self._g), b(self._n), a.ctypes.data))


class _Manager:
    def __init__(self, model, group, kind):
        self._m, self._g, self._kind = model, group, kind

    def add_field(self, name, ctype="f32", shape=()):
        L, ext = load(), _ext_arr(shape)
        if self._kind == "global":
            check(L.prtcl_gpu_global_add(self._m._h, b(name), b(ctype), len(shape), ext))
        elif self._kind == "uniform":
            check(L.prtcl_gpu_uniform_add(self._m._h, b(self._g), b(name), b(ctype), len(shape), ext))
        else:
            check(L.prtcl_gpu_field_add(self._m._h, b(self._g), b(name), b(ctype), len(shape), ext))
            self._m._dirty = True
        return self.get_field(name)

    def get_field(self, name):
        if self._kind == "varying":
            return VaryingField(self._m, self._g, name)
        return _Value(self._m, None if self._kind == "global" else self._g, name)

    def has_field(self, name):
        try:
            if self._kind == "varying":
                self.get_field(name).info()
            else:
                self.get_field(name)._info()
            return True
        except PrtclNotFound:
            return False

    AddField = add_field
    GetField = get_field
    HasField = has_field


class VaryingField:
    """A varying field of a group: bulk upload / download in the reference's
    host layout (items x components, matrices column-major)."""

    def __init__(self, model, group, name):
        self._m, self._g, self._n = model, group, name

    def info(self):
        ct = C.create_string_buffer(8)
        rank = C.c_int32(0)
        ext = (C.c_int32 * 2)()
        check(load().prtcl_gpu_field_info(self._m._h, b(self._g), b(self._n), ct, C.byref(rank), ext))
        return _type_of(ct.value.decode(), rank.value, list(ext))

    def upload(self, array, stream=None, asynchronous=False):
        dt, shape = self.info()
        n = self._m.get_group(self._g).item_count
        a = np.ascontiguousarray(np.asarray(array, dtype=dt).reshape((n,) + ((int(np.prod(shape)),) if shape else ())))
        fn = load().prtcl_gpu_field_upload_async if asynchronous else load().prtcl_gpu_field_upload
        check(fn(self._m._h, b(self._g), b(self._n), a.ctypes.data, n, _stream(stream)))
        return a

    def download(self, out=None, stream=None):
        dt, shape = self.info()
        n = self._m.get_group(self._g).item_count
        comps = int(np.prod(shape)) if shape else 1
        if out is None:
            out = np.empty((n, comps) if shape else (n,), dtype=dt)
        check(load().prtcl_gpu_field_download(self._m._h, b(self._g), b(self._n), out.ctypes.data, n, _stream(stream)))
        return out

    set_all = upload
    get_all = download


class Group:
    def __init__(self, model, name):
        self._m, self.name = model, name
        self.varying = _Manager(model, name, "varying")
        self.uniform = _Manager(model, name, "uniform")

    @property
    def item_count(self):
        n = C.c_int64(0)
        check(load().prtcl_gpu_group_count(self._m._h, b(self.name), C.byref(n)))
        return int(n.value)

    @property
    def index(self):
        i = C.c_int32(0)
        check(load().prtcl_gpu_group_index(self._m._h, b(self.name), C.byref(i)))
        return int(i.value)

    def add_tag(self, tag):
        check(load().prtcl_gpu_group_add_tag(self._m._h, b(self.name), b(tag)))
        self._m._dirty = True

    def resize(self, n):
        check(load().prtcl_gpu_group_resize(self._m._h, b(self.name), int(n)))
        self._m._dirty = True

    def save_vtk(self, path):
        """SaveVTK: the group as a legacy ASCII VTK polydata file."""
        check(load().prtcl_gpu_group_save_vtk(self._m._h, b(self.name), b(str(path))))

    AddTag = add_tag
    Resize = resize
    GetItemCount = lambda self: self.item_count  # noqa: E731
    GetGroupIndex = lambda self: self.index  # noqa: E731


class Model:
    """prtcl::Model on the device (data/model.hpp)."""

    def __init__(self):
        L = load()
        h = C.c_void_p()
        check(L.prtcl_gpu_model_create(C.byref(h)))
        self._h = h
        self.global_ = _Manager(self, None, "global")
        self._groups = {}
        self._dirty = True

    def close(self):
        if getattr(self, "_h", None):
            load().prtcl_gpu_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def dirty(self):
        return self._dirty

    @dirty.setter
    def dirty(self, v):
        self._dirty = bool(v)

    def add_group(self, name, type_):
        check(load().prtcl_gpu_group_add(self._h, b(name), b(type_)))
        self._groups.setdefault(name, Group(self, name))
        self._dirty = True
        return self._groups[name]

    def get_group(self, name):
        if name not in self._groups:
            raise PrtclNotFound(f"group does not exist: {name}")
        return self._groups[name]

    def group_names(self):
        return sorted(self._groups)

    @property
    def group_count(self):
        return len(self._groups)

    def save(self, path):
        """Model::Save in the reference's native binary archive format."""
        check(load().prtcl_gpu_model_save(self._h, b(str(path))))

    def load(self, path):
        """Model::Load from a native binary archive (adds groups and fields)."""
        check(load().prtcl_gpu_model_load(self._h, b(str(path))))
        for name in read_str(load().prtcl_gpu_model_group_names, self._h).splitlines():
            self._groups.setdefault(name, Group(self, name))
        self._dirty = True

    Save = save
    Load = load

    def synchronize(self, stream=None):
        check(load().prtcl_gpu_model_synchronize(self._h, _stream(stream)))

    def stats(self, reset=False):
        """Device-loop statistics since the last reset (see
        prtcl_gpu_model_stats)."""
        out = (C.c_double * 7)()
        check(load().prtcl_gpu_model_stats(self._h, out, 7, 1 if reset else 0))
        keys = ["jacobi_solves", "jacobi_iterations", "jacobi_capped", "max_relative_aprde",
                "pcg_solves", "pcg_iterations", "pcg_capped"]
        return dict(zip(keys, list(out)))

    def stream_handle(self):
        """The model's own cudaStream_t as an integer."""
        h = C.c_void_p()
        check(load().prtcl_gpu_model_stream(self._h, C.byref(h)))
        return int(h.value or 0)

    def profile(self, enable=True):
        """Enable / disable per-kernel CUDA-event timing."""
        check(load().prtcl_gpu_profile_enable(self._h, 1 if enable else 0))

    def profile_read(self):
        """{kernel name: (launches, total ms)} since the last reset."""
        out = {}
        for line in read_str(load().prtcl_gpu_profile_read, self._h).splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def profile_reset(self):
        check(load().prtcl_gpu_profile_reset(self._h))

    def tune_set(self, knob, value):
        """Set a launch-shape knob (prtcl_gpu_model_tune_set): bit-identical
        results, different speed."""
        check(load().prtcl_gpu_model_tune_set(self._h, b(knob), int(value)))

    def tune_get(self, knob):
        v = C.c_int32(0)
        check(load().prtcl_gpu_model_tune_get(self._h, b(knob), C.byref(v)))
        return v.value

    AddGroup = add_group
    GetGroup = get_group
    GetGroupCount = lambda self: self.group_count  # noqa: E731


class Neighborhood:
    """prtcl::Neighborhood on the device (util/neighborhood.hpp:23-42)."""

    def __init__(self):
        h = C.c_void_p()
        check(load().prtcl_gpu_nhood_create(C.byref(h)))
        self._h = h
        self._model = None

    def close(self):
        if getattr(self, "_h", None):
            load().prtcl_gpu_nhood_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_radius(self, r):
        check(load().prtcl_gpu_nhood_set_radius(self._h, float(r)))

    def load(self, model):
        check(load().prtcl_gpu_nhood_load(self._h, model._h))
        self._model = model

    def update(self, model=None, stream=None):
        check(load().prtcl_gpu_nhood_update(self._h, _stream(stream)))

    def permute(self, model, stream=None):
        check(load().prtcl_gpu_nhood_permute(self._h, model._h, _stream(stream)))

    def query(self, group_index, count_pairs=False, stream=None):
        """Build the neighbour sets of every item of a group on the device;
        with count_pairs, return the number of (item, neighbour) pairs."""
        n = C.c_int64(0)
        check(load().prtcl_gpu_nhood_query(self._h, int(group_index), C.byref(n) if count_pairs else None,
                                           _stream(stream)))
        return n.value if count_pairs else None

    def staged_tiles(self, group_index):
        """(staged, tiles) of the group's last built lists: the tiles of 128
        items whose neighbours' records fit shared memory, and all tiles;
        (0, 0) when they were not built staged."""
        k, t = C.c_int64(0), C.c_int64(0)
        check(load().prtcl_gpu_nhood_staged_tiles(self._h, int(group_index), C.byref(k), C.byref(t)))
        return k.value, t.value

    def copy_neighbors(self, group_index, index):
        """Neighbours of (group, index): one int64 array per group."""
        G = self._model.group_count
        counts = np.zeros(G, np.int64)
        cap = 8192
        out = np.zeros(cap, np.int64)
        tot = C.c_int64(0)
        check(load().prtcl_gpu_nhood_copy_neighbors(
            self._h, int(group_index), int(index), counts.ctypes.data_as(C.POINTER(C.c_int64)),
            out.ctypes.data_as(C.POINTER(C.c_int64)), cap, C.byref(tot)))
        res, o = [], 0
        for g in range(G):
            res.append(out[o:o + counts[g]].copy())
            o += counts[g]
        return res

    def neighbor_lists(self, query_group, neighbor_group, count):
        """CSR (offsets, indices) of the neighbours in `neighbor_group` of
        every item of `query_group` (for parity checks)."""
        offs = np.zeros(count + 1, np.int64)
        cap = max(16, count * 48)
        for _ in range(2):
            idx = np.zeros(cap, np.uint32)
            rc = load().prtcl_gpu_nhood_copy_lists(self._h, int(query_group), int(neighbor_group),
                                                   offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                                   idx.ctypes.data_as(C.POINTER(C.c_uint32)), cap)
            if rc == 0:
                return offs, idx[: offs[-1]].copy()
            if offs[-1] <= cap:
                check(rc)
            cap = int(offs[-1])  # offsets are complete; retry with the exact size
        check(rc)

    def grid(self):
        ns, nc = C.c_int64(0), C.c_int64(0)
        L = load()
        check(L.prtcl_gpu_nhood_grid_size(self._h, C.byref(ns), C.byref(nc)))
        n, c = int(ns.value), int(nc.value)
        sorted_ = np.empty(n, np.uint32)
        gi = np.empty((c, 3), np.int32)
        rng = np.empty((c, 2), np.int32)
        adj = np.empty((c, 26), np.int32)
        check(L.prtcl_gpu_nhood_copy_grid(self._h, sorted_.ctypes.data_as(C.POINTER(C.c_uint32)),
                                          gi.ctypes.data_as(C.POINTER(C.c_int32)),
                                          rng.ctypes.data_as(C.POINTER(C.c_int32)),
                                          adj.ctypes.data_as(C.POINTER(C.c_int32))))
        return {"sorted": sorted_, "cell_gi": gi, "cell_range": rng, "cell_adj": adj}

    SetRadius = set_radius
    Load = load
    Update = update
    Permute = permute

    def CopyNeighbors(self, g, i, neighbors=None):
        res = self.copy_neighbors(g, i)
        if neighbors is not None:
            for k, r in enumerate(res):
                neighbors[k].extend(int(x) for x in r)
        return res


class Scheme:
    """prtcl::SchemeBase on the device (schemes/scheme_base.hpp:18-64)."""

    def __init__(self, full_name):
        h = C.c_void_p()
        check(load().prtcl_gpu_scheme_new(b(full_name), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().prtcl_gpu_scheme_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, model):
        check(load().prtcl_gpu_scheme_load(self._h, model._h))

    def run_procedure(self, name, nhood, stream=None):
        check(load().prtcl_gpu_scheme_run(self._h, b(name), nhood._h, _stream(stream)))

    def get_full_name(self):
        return read_str(load().prtcl_gpu_scheme_full_name, self._h)

    def get_procedure_names(self):
        return read_str(load().prtcl_gpu_scheme_procedure_names, self._h).split("\n")

    def get_prtcl_source_code(self):
        return read_str(load().prtcl_gpu_scheme_source, self._h)

    Load = load
    RunProcedure = run_procedure
    GetFullName = get_full_name
    GetProcedureNames = get_procedure_names
    GetPrtclSourceCode = get_prtcl_source_code


def full_name(short):
    return f"prtcl::schemes::{short}[T=f32, N=3, K=Cubic Spline]"


def make_scheme(name):
    """SchemeRegistry::NewScheme (schemes/scheme_base.hpp:87-92)."""
    return Scheme(name)


def get_scheme_names():
    return read_str(load().prtcl_gpu_registry_scheme_names).split("\n")


class SchemeRegistry:
    NewScheme = staticmethod(make_scheme)
    GetSchemeNames = staticmethod(get_scheme_names)


class DeviceScene:
    """The flat model API of ``driver.py`` over a device model, one
    neighbourhood and the schemes of the hot path (loaded on first use and
    re-loaded after groups or fields change, like the reference's scripts do
    when ``model.dirty`` is set)."""

    SCHEMES = ("aiast12", "density", "gravity", "iisph", "symplectic_euler", "wkbb18")

    def __init__(self, stream=None):
        self.model = Model()
        self.nhood = Neighborhood()
        self.schemes = {}
        self.stream = stream
        self._loaded_for = None
        self._counts = {}
        self._globals = {}

    # ---- model ----
    def add_group(self, name, type_):
        self.model.add_group(name, type_)

    def add_tag(self, group, tag):
        self.model.get_group(group).add_tag(tag)

    def resize(self, group, n):
        self.model.get_group(group).resize(n)
        self._counts[group] = int(n)

    def _ensure_varying(self, group, name, arr):
        g = self.model.get_group(group)
        a = np.asarray(arr)
        shape = a.shape[1:]
        if len(shape) == 1 and shape[0] == 9:
            shape = (3, 3)
        ctype = "i32" if np.issubdtype(a.dtype, np.integer) else "f32"
        g.varying.add_field(name, ctype, shape)
        return g.varying.get_field(name)

    def set_varying(self, group, name, arr, stream=None, asynchronous=False):
        f = self._ensure_varying(group, name, arr)
        return f.upload(arr, stream=stream if stream is not None else self.stream, asynchronous=asynchronous)

    def get_varying(self, group, name, ncomp=1, out=None):
        return self.model.get_group(group).varying.get_field(name).download(out=out, stream=self.stream)

    @staticmethod
    def _small_type(value):
        a = np.asarray(value)
        ctype = "i32" if (np.issubdtype(a.dtype, np.integer) or isinstance(value, (bool, int))) else "f32"
        return ctype, a.shape

    def set_uniform(self, group, name, value):
        g = self.model.get_group(group)
        if not g.uniform.has_field(name):
            ct, sh = self._small_type(value)
            g.uniform.add_field(name, ct, sh)
        g.uniform.get_field(name).set(value)

    def get_uniform(self, group, name, n=1):
        return self.model.get_group(group).uniform.get_field(name).get()

    def set_global(self, name, value, asynchronous=False):
        f = self._globals.get(name)
        if f is None:
            if not self.model.global_.has_field(name):
                ct, sh = self._small_type(value)
                self.model.global_.add_field(name, ct, sh)
            f = self._globals[name] = self.model.global_.get_field(name)
        f.set(value, asynchronous=asynchronous, stream=self.stream)

    def get_global(self, name, n=1):
        return self.model.global_.get_field(name).get()

    # ---- neighbourhood / schemes ----
    def _refresh(self):
        if self.model.dirty:
            self.nhood.load(self.model)
            for s in self.schemes.values():
                s.load(self.model)
            self.model.dirty = False

    def set_radius(self, r):
        self.nhood.set_radius(r)

    def update(self):
        self._refresh()
        self.nhood.update(stream=self.stream)

    def permute(self):
        self._refresh()
        self.nhood.permute(self.model, stream=self.stream)

    def scheme(self, name):
        s = self.schemes.get(name)
        if s is None:
            s = make_scheme(full_name(name))
            s.load(self.model)
            self.schemes[name] = s
            self.model.dirty = True  # the scheme may have added fields
        return s

    def run(self, scheme, procedure):
        s = self.scheme(scheme)
        self._refresh()
        s.run_procedure(procedure, self.nhood, stream=self.stream)

    def synchronize(self):
        self.model.synchronize(self.stream)
