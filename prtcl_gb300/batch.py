"""Batched scenes over the C ABI (prtcl_gpu_batch_*).

Many dam-break scenes resident on the device, stepped together; every scene
converges on its own and gets the same results as when it runs alone.
Parameters are the step-loop dictionaries of ``prtcl_gb300.driver``
(``DAM_BREAK_27K``, ``DAM_BREAK_1M``); the batch requires the hard fade to be
open (``fade_duration`` 0): particles are born one second before their scene
is added.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import BatchParams, SceneInfo, b, check, load, read_str

VEC3 = {"position", "velocity", "acceleration", "iisph_helper_c", "wkbb18_velocity_delta"}
MAT3 = {"wkbb18_system_diagonal"}


def params_struct(p):
    if float(p.get("fade_duration", 0.0)) != 0.0:
        raise ValueError("batched scenes need fade_duration == 0")
    s = BatchParams()
    s.smoothing_scale = float(np.float32(p["smoothing_scale"]))
    s.time_step = float(np.float32(p["time_step"]))
    s.rest_density = float(np.float32(p["rest_density"]))
    for k in range(3):
        s.gravity[k] = float(np.float32(p["gravity"][k]))
    s.relaxation = float(np.float32(p["iisph_relaxation"]))
    s.max_density_error = float(np.float32(p["eta"]))
    s.max_iterations = int(p["max_iters"])
    s.viscosity = 1 if p.get("viscosity") else 0
    s.dynamic_viscosity = float(np.float32(p["dynamic_viscosity"]))
    s.boundary_dynamic_viscosity = float(np.float32(p["boundary_dynamic_viscosity"]))
    s.pcg_max_error = float(np.float32(p["wkbb18_maximum_error"]))
    s.pcg_max_iterations = int(p["wkbb18_maximum_iterations"])
    s.permute_every = int(p["permute_every"])
    return s


class Batch:
    def __init__(self, params):
        self.params = dict(params)
        h = C.c_void_p()
        check(load().prtcl_gpu_batch_create(C.byref(params_struct(params)), C.byref(h)))
        self._h = h
        self._nf = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            load().prtcl_gpu_batch_destroy(h)
            self._h = None

    def add_scene(self, fluid, boundary):
        f = np.ascontiguousarray(fluid, np.float32).reshape(-1, 3)
        bd = np.ascontiguousarray(boundary, np.float32).reshape(-1, 3)
        sid = C.c_int64(0)
        check(load().prtcl_gpu_batch_add_scene(self._h, f.ctypes.data, len(f), bd.ctypes.data, len(bd),
                                               C.byref(sid)))
        self._nf[sid.value] = len(f)
        return sid.value

    def remove_scene(self, sid):
        check(load().prtcl_gpu_batch_remove_scene(self._h, int(sid)))
        self._nf.pop(int(sid), None)

    def step(self, steps=1):
        check(load().prtcl_gpu_batch_step(self._h, int(steps)))

    def synchronize(self):
        check(load().prtcl_gpu_batch_synchronize(self._h))

    def info(self, sid):
        out = SceneInfo()
        check(load().prtcl_gpu_batch_scene_info(self._h, int(sid), C.byref(out)))
        return {k: getattr(out, k) for k, _ in SceneInfo._fields_ if k != "pad"}

    def download(self, sid, field):
        n = self._nf[int(sid)]
        if field in VEC3:
            out = np.empty((n, 3), np.float32)
        elif field in MAT3:
            out = np.empty((n, 9), np.float32)
        else:
            out = np.empty(n, np.float32)
        check(load().prtcl_gpu_batch_download(self._h, int(sid), b(field), out.ctypes.data, n))
        return out

    @property
    def scene_count(self):
        n = C.c_int32(0)
        check(load().prtcl_gpu_batch_scene_count(self._h, C.byref(n)))
        return n.value

    def particles(self):
        nf, nb = C.c_int64(0), C.c_int64(0)
        check(load().prtcl_gpu_batch_particles(self._h, C.byref(nf), C.byref(nb)))
        return nf.value, nb.value

    def device_bytes(self):
        v = C.c_int64(0)
        check(load().prtcl_gpu_batch_device_bytes(self._h, C.byref(v)))
        return v.value

    def profile(self, enable=True):
        check(load().prtcl_gpu_batch_profile_enable(self._h, 1 if enable else 0))

    def tune_set(self, knob, value):
        """Set a launch-shape knob of the batch's model (bit-identical)."""
        check(load().prtcl_gpu_batch_tune_set(self._h, b(knob), int(value)))

    def tune_get(self, knob):
        v = C.c_int32(0)
        check(load().prtcl_gpu_batch_tune_get(self._h, b(knob), C.byref(v)))
        return v.value

    def profile_read(self):
        out = {}
        for line in read_str(load().prtcl_gpu_batch_profile_read, self._h).splitlines():
            name, count, ms = line.split()
            out[name] = (int(count), float(ms))
        return out
