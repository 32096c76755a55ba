"""bench.py's measurement helpers on the CPU: the roofline block of a
single-scene profile, the knob overrides and the leg selection of its
command line."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _NoScene:
    """A scene the roofline never touches (no list-build kernel in the
    profile)."""


def test_roofline_takes_the_top_kernel_with_a_formula():
    prof = {"grid_cells": (3, 0.9), "iisph_pressure": (6, 0.8), "density": (3, 0.1)}
    nf, nb = 1000, 500
    roof = bench.plain_roofline(_NoScene(), prof, nf, nb, 6800.0, "measured", "test")
    assert roof["kernel"] == "iisph_pressure"
    per_launch = bench.ALGO_BYTES["iisph_pressure"][0] * nf + bench.ALGO_BYTES["iisph_pressure"][1] * nb
    assert roof["algorithmic_bytes_per_launch"] == per_launch
    assert abs(roof["avg_launch_us"] - 0.8e3 / 6) < 0.01
    assert abs(roof["achieved"] - round(per_launch / (0.8e-3 / 6) / 1e9, 1)) < 0.05
    assert roof["top_kernel_without_formula"] == {"kernel": "grid_cells", "ms": 0.9}
    assert abs(roof["share_of_kernel_time"] - 0.8 / 1.8) < 1e-4


def test_roofline_without_any_formula():
    roof = bench.plain_roofline(_NoScene(), {"grid_sort": (1, 1.0)}, 10, 10, 6800.0, "measured", "test")
    assert roof["frac"] is None and roof["kernel"] == "grid_sort"


def test_roofline_of_the_top_kernel_has_no_extra_key():
    prof = {"pcg_q": (4, 0.6), "grid_cells": (3, 0.1)}
    roof = bench.plain_roofline(_NoScene(), prof, 1000, 0, 6800.0, "measured", "test")
    assert roof["kernel"] == "pcg_q" and "top_kernel_without_formula" not in roof


def _usage_error(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 2, r.stderr
    return r.stderr


def test_knob_and_leg_arguments_are_checked():
    assert "knobs are" in _usage_error("--knob", "staging=3")
    assert "knobs are" in _usage_error("--knob", "nosuchknob=1")
    assert "knobs are" in _usage_error("--knob", "grid_sort")
    assert "legs are" in _usage_error("--extras", "search,nosuchleg")
