"""ctypes wrapper around the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile liboracle.so with the Makefile next to this file."""
    srcs = [os.path.join(_HERE, f) for f in ("oracle.cpp", "oracle.hpp", "Makefile")]
    if not force and os.path.exists(_SO):
        if os.path.getmtime(_SO) >= max(os.path.getmtime(s) for s in srcs):
            return _SO
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            vp, cp, i64, dp = C.c_void_p, C.c_char_p, C.c_int64, C.POINTER(C.c_double)
            L.oracle_last_error.restype = cp
            L.oracle_scene_new.restype = vp
            L.oracle_scene_new.argtypes = [C.c_int, C.c_int]
            L.oracle_scene_free.argtypes = [vp]
            L.oracle_set_threads.argtypes = [C.c_int]
            L.oracle_morton_compare_many.argtypes = [vp, vp, C.c_int64, vp]
            L.oracle_pinv3_many.argtypes = [vp, C.c_int64, vp]
            L.oracle_pinv3_many.restype = None
            L.oracle_morton_compare_many.restype = None
            L.oracle_add_group.argtypes = [vp, cp, cp]
            L.oracle_add_tag.argtypes = [vp, cp, cp]
            L.oracle_resize.argtypes = [vp, cp, i64]
            L.oracle_group_index.argtypes = [vp, cp]
            L.oracle_set_varying.argtypes = [vp, cp, cp, C.c_int, vp, i64]
            L.oracle_get_varying.argtypes = [vp, cp, cp, C.c_int, vp, i64]
            L.oracle_set_uniform.argtypes = [vp, cp, cp, dp, C.c_int]
            L.oracle_get_uniform.argtypes = [vp, cp, cp, dp, C.c_int]
            L.oracle_set_global.argtypes = [vp, cp, dp, C.c_int]
            L.oracle_get_global.argtypes = [vp, cp, dp, C.c_int]
            L.oracle_set_radius.argtypes = [vp, C.c_double]
            L.oracle_nhood_update.argtypes = [vp]
            L.oracle_nhood_permute.argtypes = [vp]
            L.oracle_run.argtypes = [vp, cp, cp]
            L.oracle_grid_sorted_count.restype = i64
            L.oracle_grid_sorted_count.argtypes = [vp]
            L.oracle_grid_cell_count.restype = i64
            L.oracle_grid_cell_count.argtypes = [vp]
            L.oracle_grid_dump.argtypes = [vp, vp, vp, vp, vp]
            L.oracle_neighbors.restype = i64
            L.oracle_neighbors.argtypes = [vp, C.c_int, i64, vp, vp, i64]
            L.oracle_neighbor_lists.argtypes = [vp, C.c_int, C.c_int, vp, vp, i64]
            L.oracle_step.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, dp]
            _lib = L
    return _lib


def _b(s):
    return s.encode() if isinstance(s, str) else s


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())


def morton_compare(a, b):
    """Three-way Morton compare (-1, 0, 1) of int32 triples a[i] and b[i]."""
    a = np.ascontiguousarray(a, np.int32).reshape(-1, 3)
    b = np.ascontiguousarray(b, np.int32).reshape(-1, 3)
    assert a.shape == b.shape
    out = np.empty(len(a), np.int8)
    lib().oracle_morton_compare_many(a.ctypes.data, b.ctypes.data, len(a), out.ctypes.data)
    return out


def pinv3(a):
    """Pseudo-inverses (f32) of 3x3 matrices a[k] (row-major numpy input)."""
    a = np.asarray(a, np.float32).reshape(-1, 3, 3)
    cm = np.ascontiguousarray(np.transpose(a, (0, 2, 1)))  # column-major items
    out = np.empty_like(cm)
    lib().oracle_pinv3_many(cm.ctypes.data, len(cm), out.ctypes.data)
    return np.transpose(out, (0, 2, 1))


def set_threads(n=0):
    """Set (n > 0) and return the OpenMP thread count of the oracle."""
    return lib().oracle_set_threads(int(n))


class Scene:
    """A CPU model + neighbourhood with the flat API the step driver uses."""

    def __init__(self, real=np.float32, fp64_reductions=True):
        self.real = np.dtype(real)
        self._h = lib().oracle_scene_new(self.real.itemsize, 1 if fp64_reductions else 0)
        self._counts = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_scene_free(h)
            self._h = None

    # ---- model ----
    def add_group(self, name, type_):
        _check(lib().oracle_add_group(self._h, _b(name), _b(type_)))

    def add_tag(self, group, tag):
        _check(lib().oracle_add_tag(self._h, _b(group), _b(tag)))

    def resize(self, group, n):
        _check(lib().oracle_resize(self._h, _b(group), int(n)))
        self._counts[group] = int(n)

    def group_index(self, group):
        return lib().oracle_group_index(self._h, _b(group))

    def set_varying(self, group, field, arr):
        a = np.ascontiguousarray(arr, dtype=self.real)
        n = a.shape[0]
        ncomp = int(np.prod(a.shape[1:])) if a.ndim > 1 else 1
        _check(lib().oracle_set_varying(self._h, _b(group), _b(field), ncomp, a.ctypes.data, n))

    def get_varying(self, group, field, ncomp=1, count=None):
        if count is None:
            count = self._count(group)
        out = np.empty((count, ncomp) if ncomp > 1 else (count,), dtype=self.real)
        _check(lib().oracle_get_varying(self._h, _b(group), _b(field), ncomp, out.ctypes.data, count))
        return out

    def _count(self, group):
        return self._counts[group]

    def set_uniform(self, group, name, value):
        v = np.atleast_1d(np.asarray(value, dtype=np.float64))
        _check(lib().oracle_set_uniform(self._h, _b(group), _b(name), v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def get_uniform(self, group, name, n=1):
        v = np.zeros(n, dtype=np.float64)
        _check(lib().oracle_get_uniform(self._h, _b(group), _b(name), v.ctypes.data_as(C.POINTER(C.c_double)), n))
        return v if n > 1 else float(v[0])

    def set_global(self, name, value, asynchronous=False):
        v = np.atleast_1d(np.asarray(value, dtype=np.float64))
        _check(lib().oracle_set_global(self._h, _b(name), v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def get_global(self, name, n=1):
        v = np.zeros(n, dtype=np.float64)
        _check(lib().oracle_get_global(self._h, _b(name), v.ctypes.data_as(C.POINTER(C.c_double)), n))
        return v if n > 1 else float(v[0])

    # ---- neighbourhood ----
    def set_radius(self, r):
        _check(lib().oracle_set_radius(self._h, float(r)))

    def update(self):
        _check(lib().oracle_nhood_update(self._h))

    def permute(self):
        _check(lib().oracle_nhood_permute(self._h))

    def run(self, scheme, procedure):
        _check(lib().oracle_run(self._h, _b(scheme), _b(procedure)))

    def step(self, permute=False, max_iters=100, eta=1e-3, viscosity=False):
        st = np.zeros(3, dtype=np.float64)
        _check(lib().oracle_step(self._h, 1 if permute else 0, int(max_iters), float(eta),
                                 1 if viscosity else 0, st.ctypes.data_as(C.POINTER(C.c_double))))
        return {"jacobi_iterations": int(st[0]), "relative_aprde": float(st[1])}

    # ---- grid introspection ----
    def grid(self):
        n = lib().oracle_grid_sorted_count(self._h)
        c = lib().oracle_grid_cell_count(self._h)
        sorted_ = np.empty(n, np.uint32)
        gi = np.empty((c, 3), np.int32)
        rng = np.empty((c, 2), np.int32)
        adj = np.empty((c, 26), np.int32)
        _check(lib().oracle_grid_dump(self._h, sorted_.ctypes.data, gi.ctypes.data, rng.ctypes.data, adj.ctypes.data))
        return {"sorted": sorted_, "cell_gi": gi, "cell_range": rng, "cell_adj": adj}

    def neighbors(self, group_index, i, ngroups):
        counts = np.zeros(ngroups, np.int64)
        cap = 4096
        out = np.zeros(cap, np.int64)
        k = lib().oracle_neighbors(self._h, int(group_index), int(i), counts.ctypes.data, out.ctypes.data, cap)
        if k < 0:
            raise OracleError(lib().oracle_last_error().decode())
        res, o = [], 0
        for g in range(ngroups):
            res.append(out[o:o + counts[g]].copy())
            o += counts[g]
        return res

    def neighbor_lists(self, qgroup, ngroup, count, cap=None):
        if cap is None:
            cap = count * 200 + 16
        offs = np.zeros(count + 1, np.int64)
        idx = np.zeros(cap, np.uint32)
        _check(lib().oracle_neighbor_lists(self._h, int(qgroup), int(ngroup), offs.ctypes.data, idx.ctypes.data, cap))
        return offs, idx[: offs[-1]].copy()
