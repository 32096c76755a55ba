"""GB300-native (CUDA sm_103a) implementation of prtcl's SPH hot path:
uniform-grid neighbourhood, IISPH pressure solve, WKBB18 implicit viscosity
PCG, behind the reference's model / neighbourhood / scheme API; batched
scenes (Batch) and a serving loop (Server) beside it.

The CUDA library is loaded on first use; there is no CPU fallback.
"""
from ._lib import PrtclGpuError, PrtclGpuUnavailable, PrtclNotFound  # noqa: F401


def __getattr__(name):
    # the device API is imported lazily so that the pure-Python parts
    # (scenes, driver) import on machines without the library
    if name in ("Model", "Neighborhood", "Scheme", "SchemeRegistry", "DeviceScene", "make_scheme",
                "get_scheme_names", "full_name", "VaryingField", "Group"):
        from . import core
        return getattr(core, name)
    if name == "Batch":
        from . import batch
        return batch.Batch
    if name == "Server":
        from . import serve
        return serve.Server
    raise AttributeError(name)
