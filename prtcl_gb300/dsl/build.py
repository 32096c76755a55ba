"""Compile schemes of the scheme language into loadable plugins.

``compile_scheme(source)`` parses a ``.prtcl`` text, generates the CUDA
plugin of each scheme (``prtcl_gb300.dsl.cuda``), compiles it for sm_103a
with the flags of the library itself (no FMA contraction, IEEE division and
square root), links it against ``libprtcl_gpu.so`` and loads it through
``prtcl_gpu_scheme_load_plugin``.  The schemes are then created by full name
like the built-in ones (``prtcl_gb300.core.Scheme``).

Plugins are cached in-tree under ``prtcl_gb300/_dsl_cache/<hash>/`` (keyed
on the generated source and the library build), so a scheme compiles once.
A ``prefix`` renames the schemes (``prefix + name``), e.g. to run a
generated ``density`` beside the built-in one.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import threading

from .. import build as libbuild
from .cuda import full_name, generate_all
from .parser import parse

CACHE = os.path.join(libbuild.HERE, "_dsl_cache")
_loaded = {}
_lib_lock = threading.Lock()  # one library build at a time


def plugin_source(source: str, prefix: str = "", embed_source: bool = True):
    """(full names, CUDA source) of the plugin of a ``.prtcl`` text: every
    scheme of the text in one translation unit."""
    schemes = parse(source)
    return [full_name(s, prefix) for s in schemes], generate_all(schemes, prefix, embed_source)


def _compile(name: str, cu: str) -> str:
    with _lib_lock:
        lib = libbuild.build()
    key = hashlib.sha1((cu + str(os.path.getmtime(lib))).encode()).hexdigest()[:16]
    d = os.path.join(CACHE, key)
    so = os.path.join(d, "plugin.so")
    if os.path.exists(so):
        return so
    os.makedirs(d, exist_ok=True)
    src = os.path.join(d, "plugin.cu")
    with open(src, "w") as f:
        f.write(cu)
    tmp = so + f".{os.getpid()}.tmp"
    cmd = [libbuild.nvcc(), *libbuild.ARCH, *libbuild.FLAGS, "-I", libbuild.CSRC, "-shared", "-cudart", "static",
           src, "-o", tmp, "-L", libbuild.HERE, "-lprtcl_gpu", "-Xlinker", "-rpath=" + libbuild.HERE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for the generated scheme {name}:\n{r.stderr[-4000:]}")
    os.replace(tmp, so)
    return so


def compile_scheme(source: str, prefix: str = ""):
    """Generate, compile and load every scheme of a ``.prtcl`` text (one
    plugin); returns their full names."""
    names, cu = plugin_source(source, prefix)
    return load_plugin_source(names, cu)


def load_plugin_source(names, cu: str):
    """Compile and load an already generated plugin source (e.g. one
    generated elsewhere and kept as a file) whose schemes are ``names``."""
    from .._lib import check, load
    done = [n for n in names if n in _loaded]
    if done:
        if all(_loaded.get(n) == cu for n in names):
            return names
        raise RuntimeError(f"schemes already loaded from another source: {', '.join(done)}")
    so = _compile(", ".join(names), cu)
    check(load().prtcl_gpu_scheme_load_plugin(so.encode()))
    for n in names:
        _loaded[n] = cu
    return names


def compile_file(path: str, prefix: str = ""):
    with open(path) as f:
        return compile_scheme(f.read(), prefix)
