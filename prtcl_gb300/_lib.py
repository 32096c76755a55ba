"""ctypes binding of the C ABI declared in include/prtcl_gpu.h.

The library is built in-tree (prtcl_gb300/libprtcl_gpu.so) by
``prtcl_gb300.build.build()``.  There is no CPU fallback: if the library is
missing, cannot be loaded or no CUDA device is present, the first call
raises ``PrtclGpuUnavailable``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libprtcl_gpu.so")

OK, ERROR, NOT_FOUND, INVALID = 0, -1, -2, -3


class PrtclGpuError(RuntimeError):
    """A failed call of the C ABI (the message of prtcl_gpu_last_error)."""


class PrtclNotFound(PrtclGpuError, LookupError):
    """Unknown group, field, procedure or scheme ("procedure does not exist",
    "scheme is not registered" in the reference)."""


class PrtclGpuUnavailable(ImportError):
    """The CUDA library is missing or could not be loaded."""


vp, cp, i32, i64, u32p, i64p, i32p, dbl = (C.c_void_p, C.c_char_p, C.c_int32, C.c_int64, C.POINTER(C.c_uint32),
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_double)
pp = C.POINTER(C.c_void_p)

# name -> argtypes (all entry points return int unless listed in _RESTYPE)
SIGNATURES = {
    "prtcl_gpu_last_error": [],
    "prtcl_gpu_version": [],
    "prtcl_gpu_launch_count": [],
    "prtcl_gpu_model_create": [pp],
    "prtcl_gpu_model_destroy": [vp],
    "prtcl_gpu_group_add": [vp, cp, cp],
    "prtcl_gpu_group_add_tag": [vp, cp, cp],
    "prtcl_gpu_group_resize": [vp, cp, i64],
    "prtcl_gpu_group_count": [vp, cp, i64p],
    "prtcl_gpu_group_index": [vp, cp, i32p],
    "prtcl_gpu_model_group_count": [vp, i32p],
    "prtcl_gpu_field_add": [vp, cp, cp, cp, i32, i32p],
    "prtcl_gpu_field_upload": [vp, cp, cp, vp, i64, vp],
    "prtcl_gpu_field_upload_async": [vp, cp, cp, vp, i64, vp],
    "prtcl_gpu_field_upload_noalloc": [vp, cp, cp, vp, i64, vp],
    "prtcl_gpu_field_download": [vp, cp, cp, vp, i64, vp],
    "prtcl_gpu_field_info": [vp, cp, cp, C.c_char_p, i32p, i32p],
    "prtcl_gpu_uniform_add": [vp, cp, cp, cp, i32, i32p],
    "prtcl_gpu_uniform_set": [vp, cp, cp, vp],
    "prtcl_gpu_uniform_get": [vp, cp, cp, vp],
    "prtcl_gpu_global_add": [vp, cp, cp, i32, i32p],
    "prtcl_gpu_global_set": [vp, cp, vp],
    "prtcl_gpu_global_get": [vp, cp, vp],
    "prtcl_gpu_global_set_async": [vp, cp, vp, vp],
    "prtcl_gpu_model_stats": [vp, C.POINTER(C.c_double), i32, i32],
    "prtcl_gpu_uniform_info": [vp, cp, cp, C.c_char_p, i32p, i32p],
    "prtcl_gpu_global_info": [vp, cp, C.c_char_p, i32p, i32p],
    "prtcl_gpu_model_stream": [vp, pp],
    "prtcl_gpu_model_synchronize": [vp, vp],
    "prtcl_gpu_profile_enable": [vp, i32],
    "prtcl_gpu_profile_read": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_profile_reset": [vp],
    "prtcl_gpu_tune_knobs": [C.c_char_p, i64, i64p],
    "prtcl_gpu_model_tune_set": [vp, cp, i32],
    "prtcl_gpu_model_tune_get": [vp, cp, i32p],
    "prtcl_gpu_nhood_create": [pp],
    "prtcl_gpu_nhood_destroy": [vp],
    "prtcl_gpu_nhood_set_radius": [vp, dbl],
    "prtcl_gpu_nhood_load": [vp, vp],
    "prtcl_gpu_nhood_update": [vp, vp],
    "prtcl_gpu_nhood_permute": [vp, vp, vp],
    "prtcl_gpu_nhood_copy_neighbors": [vp, i32, i64, i64p, i64p, i64, i64p],
    "prtcl_gpu_nhood_copy_lists": [vp, i32, i32, i64p, u32p, i64],
    "prtcl_gpu_nhood_staged_tiles": [vp, i32, i64p, i64p],
    "prtcl_gpu_nhood_grid_size": [vp, i64p, i64p],
    "prtcl_gpu_nhood_copy_grid": [vp, u32p, i32p, i32p, i32p],
    "prtcl_gpu_scheme_new": [cp, pp],
    "prtcl_gpu_scheme_destroy": [vp],
    "prtcl_gpu_scheme_load": [vp, vp],
    "prtcl_gpu_scheme_run": [vp, cp, vp, vp],
    "prtcl_gpu_scheme_full_name": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_scheme_procedure_names": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_scheme_source": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_registry_scheme_names": [C.c_char_p, i64, i64p],
    "prtcl_gpu_scheme_load_plugin": [C.c_char_p],
    "prtcl_gpu_nhood_query": [vp, i32, i64p, vp],
    "prtcl_gpu_model_group_names": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_model_save": [vp, cp],
    "prtcl_gpu_group_save_vtk": [vp, cp, cp],
    "prtcl_gpu_model_load": [vp, cp],
    "prtcl_gpu_batch_create": [vp, pp],
    "prtcl_gpu_batch_destroy": [vp],
    "prtcl_gpu_batch_add_scene": [vp, vp, i64, vp, i64, i64p],
    "prtcl_gpu_batch_remove_scene": [vp, i64],
    "prtcl_gpu_batch_step": [vp, i32],
    "prtcl_gpu_batch_synchronize": [vp],
    "prtcl_gpu_batch_scene_info": [vp, i64, vp],
    "prtcl_gpu_batch_download": [vp, i64, cp, vp, i64],
    "prtcl_gpu_batch_scene_count": [vp, i32p],
    "prtcl_gpu_batch_particles": [vp, i64p, i64p],
    "prtcl_gpu_batch_device_bytes": [vp, i64p],
    "prtcl_gpu_batch_profile_enable": [vp, i32],
    "prtcl_gpu_batch_profile_read": [vp, C.c_char_p, i64, i64p],
    "prtcl_gpu_batch_tune_set": [vp, cp, i32],
    "prtcl_gpu_batch_tune_get": [vp, cp, i32p],
    "prtcl_gpu_server_create": [vp, vp, pp],
    "prtcl_gpu_server_create_custom": [vp, vp, vp, pp],
    "prtcl_gpu_server_destroy": [vp],
    "prtcl_gpu_server_submit": [vp, i64, dbl, vp, i64, vp, i64, i64],
    "prtcl_gpu_server_turn": [vp, i32p],
    "prtcl_gpu_server_status_get": [vp, vp],
    "prtcl_gpu_server_cancel": [vp, i64, i32p],
    "prtcl_gpu_server_next_result": [vp, vp, vp, i64, i32p],
}


class BatchParams(C.Structure):
    """prtcl_gpu_batch_params"""
    _fields_ = [("smoothing_scale", C.c_double), ("time_step", C.c_double), ("rest_density", C.c_double),
                ("gravity", C.c_double * 3), ("relaxation", C.c_double), ("max_density_error", C.c_double),
                ("max_iterations", C.c_int32), ("viscosity", C.c_int32), ("dynamic_viscosity", C.c_double),
                ("boundary_dynamic_viscosity", C.c_double), ("pcg_max_error", C.c_double),
                ("pcg_max_iterations", C.c_int32), ("permute_every", C.c_int32)]


class SceneInfo(C.Structure):
    """prtcl_gpu_scene_info"""
    _fields_ = [("fluid", C.c_int64), ("boundary", C.c_int64), ("steps", C.c_int64), ("slot", C.c_int32),
                ("last_jacobi_iterations", C.c_int32), ("last_pcg_iterations", C.c_int32), ("pad", C.c_int32),
                ("last_relative_density_error", C.c_double), ("max_relative_density_error", C.c_double),
                ("jacobi_solves", C.c_double), ("jacobi_iterations", C.c_double), ("jacobi_capped", C.c_double),
                ("pcg_solves", C.c_double), ("pcg_iterations", C.c_double), ("pcg_capped", C.c_double)]


CLOCK_FN = C.CFUNCTYPE(C.c_double, C.c_void_p)


class ServerParams(C.Structure):
    """prtcl_gpu_server_params"""
    _fields_ = [("budget_bytes", C.c_double), ("max_scenes", C.c_int32), ("keep_results", C.c_int32),
                ("bytes_per_particle", C.c_double), ("clock", CLOCK_FN), ("clock_user", C.c_void_p)]


class ServerBatchOps(C.Structure):
    """prtcl_gpu_server_batch_ops"""
    _fields_ = [
        ("add_scene", C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                  C.c_int64, C.POINTER(C.c_int64))),
        ("remove_scene", C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64)),
        ("step", C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32)),
        ("synchronize", C.CFUNCTYPE(C.c_int, C.c_void_p)),
        ("device_bytes", C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_int64))),
        ("scene_info", C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(SceneInfo))),
        ("download_positions", C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_int64)),
    ]


class RequestResult(C.Structure):
    """prtcl_gpu_request_result"""
    _fields_ = [("request_id", C.c_int64), ("fluid", C.c_int64), ("boundary", C.c_int64), ("steps", C.c_int64),
                ("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double), ("info", SceneInfo),
                ("status", C.c_int32), ("pad", C.c_int32)]


# prtcl_gpu_request_result.status
REQUEST_STATUS = {0: "done", 1: "cancelled", 2: "rejected", 3: "failed"}


class ServerStatus(C.Structure):
    """prtcl_gpu_server_status"""
    _fields_ = [("pending", C.c_int64), ("running", C.c_int64), ("results", C.c_int64), ("steps_run", C.c_int64),
                ("particle_steps", C.c_int64), ("held_bytes", C.c_int64), ("next_arrival", C.c_double)]


_RESTYPE = {"prtcl_gpu_last_error": cp, "prtcl_gpu_version": cp, "prtcl_gpu_launch_count": C.c_uint64}

_lock = threading.Lock()
_lib = None


def load(path=LIB_PATH):
    """Load (once) and return the ctypes library with all signatures set."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise PrtclGpuUnavailable(
                f"{path} is missing: build it with `python -m prtcl_gb300.build` "
                "(there is no CPU fallback)")
        try:
            L = C.CDLL(path)
        except OSError as e:
            raise PrtclGpuUnavailable(f"cannot load {path}: {e}") from e
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
        return L


def check(rc):
    if rc == OK:
        return
    msg = load().prtcl_gpu_last_error().decode()
    if rc == NOT_FOUND:
        raise PrtclNotFound(msg)
    raise PrtclGpuError(msg)


def b(s):
    return s.encode() if isinstance(s, str) else s


def read_str(fn, *args):
    need = C.c_int64(0)
    check(fn(*args, None, 0, C.byref(need)))
    buf = C.create_string_buffer(int(need.value))
    check(fn(*args, buf, need.value, C.byref(need)))
    return buf.value.decode()
