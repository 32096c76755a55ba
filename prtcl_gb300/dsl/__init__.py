"""The scheme language (``.prtcl``) and its CUDA backend.

``compile_scheme(text)`` / ``compile_file(path)`` turn the schemes of a
``.prtcl`` source into a plugin of device kernels and register them by full
name, after which they are created, loaded and run like the built-in
schemes (``prtcl_gb300.core.Scheme``, ``DeviceScene.run``).  Counterpart of
the reference's generator (lua/prtcl/generate/cxx_openmp_impl_hpp.lua).
"""
from .build import compile_file, compile_scheme, plugin_source  # noqa: F401
from .parser import DslError, parse, parse_one  # noqa: F401
