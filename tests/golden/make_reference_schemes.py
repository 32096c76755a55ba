"""Generate tests/golden/reference_schemes_plugin.cu: the CUDA plugin that
this package's scheme-language generator (prtcl_gb300.dsl) emits for the
reference's own scheme sources on the simulation path,

    share/schemes/{aiast12, density, gravity, iisph, symplectic_euler,
                   wkbb18}.prtcl

with every scheme renamed ``ref_<name>`` so that it loads beside the
hand-written schemes.  The plugin does not embed the ``.prtcl`` texts (its
GetPrtclSourceCode returns a fixed note).  The fixture is committed so that
the GPU parity test (tests/test_gpu_reference_schemes.py) runs where the
reference checkout is absent; tests/test_dsl.py checks, where the checkout
is present, that the committed file is still what the generator emits.

Run:  PRTCL_REFERENCE=<reference checkout> python tests/golden/make_reference_schemes.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SCHEMES = ("aiast12", "density", "gravity", "iisph", "symplectic_euler", "wkbb18")
PREFIX = "ref_"
OUT = os.path.join(HERE, "reference_schemes_plugin.cu")
META = os.path.join(HERE, "reference_schemes_plugin.json")


def reference_texts(root):
    texts = []
    for s in SCHEMES:
        with open(os.path.join(root, "share", "schemes", s + ".prtcl")) as f:
            texts.append((s, f.read()))
    return texts


def generate(root):
    """(names, CUDA source, metadata) of the plugin for the checkout at root."""
    from prtcl_gb300.dsl.build import plugin_source
    texts = reference_texts(root)
    names, cu = plugin_source("\n".join(t for _, t in texts), prefix=PREFIX, embed_source=False)
    header = ("// Generated by tests/golden/make_reference_schemes.py with prtcl_gb300.dsl from the\n"
              "// reference's share/schemes/{" + ", ".join(SCHEMES) + "}.prtcl (schemes renamed\n"
              "// ref_<name>).  Test fixture: do not edit.\n")
    meta = {"schemes": names, "sources": {s: hashlib.sha256(t.encode()).hexdigest() for s, t in texts}}
    return names, header + cu, meta


def main():
    root = os.environ.get("PRTCL_REFERENCE")
    if not root:
        sys.exit("set PRTCL_REFERENCE to the reference checkout")
    names, cu, meta = generate(root)
    with open(OUT, "w") as f:
        f.write(cu)
    with open(META, "w") as f:
        json.dump(meta, f, indent=1)
        f.write("\n")
    print(OUT, len(cu), "bytes;", ", ".join(names))


if __name__ == "__main__":
    main()
