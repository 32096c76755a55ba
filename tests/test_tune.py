"""The autotuner's search and cache (prtcl_gb300.tune) against a stand-in
target with fixed per-variant costs, and the knob table of the C ABI (no
device needed)."""
import json

import pytest

from prtcl_gb300 import tune


class FakeTarget:
    """Per-kernel seconds per launch by variant; whole-step seconds by
    Jacobi repeat count (plus the staging knob's cost, when given).  Counts
    the measurements."""

    def __init__(self, costs, unroll_cost, knobs=None, staging_cost=None):
        self.costs, self.unroll_cost, self.staging_cost = costs, unroll_cost, staging_cost or {0: 0.0, 1: 0.0}
        self.v = dict(tune.DEFAULTS)
        self.calls = 0
        self._knobs = knobs or list(costs) + ["jacobi_unroll"]

    def knobs(self):
        return self._knobs

    def set(self, k, v):
        assert v in tune.VALUES[k]
        self.v[k] = v

    def measure_kernels(self, names):
        self.calls += 1
        return {k: self.costs[k][self.v[k]] for k in names}

    def measure_steps(self):
        self.calls += 1
        return self.unroll_cost[self.v["jacobi_unroll"]] + self.staging_cost[self.v["staging"]]


COSTS = {"iisph_accel": [1.0e-4, 0.9e-4, 1.2e-4, 0.8e-4, 0.85e-4],
         "iisph_pressure": [1.4e-4, 1.5e-4, 1.1e-4, 2.0e-4, 1.6e-4],
         "density": [1.0e-4, 1.0e-4, 1.0e-4, 1.0e-4]}
UNROLL = {1: 3.0e-3, 2: 2.9e-3, 4: 2.95e-3}


def test_search_picks_the_fastest_variant_per_knob(tmp_path):
    t = tune.Autotuner(cache_path=str(tmp_path / "c.json"), device="GB300-test")
    tgt = FakeTarget(COSTS, UNROLL)
    choice, source, timings = t.tune(tgt, "plain:f2^20")
    assert source == "tuned"
    assert choice == {"iisph_accel": 3, "iisph_pressure": 2, "density": 0, "jacobi_unroll": 2}
    assert tgt.v["iisph_accel"] == 3 and tgt.v["jacobi_unroll"] == 2  # applied
    # each shape index (0..4: some knobs have a fifth form) twice, rising and
    # falling, and each repeat count twice; a knob without the index keeps
    # its default in that run
    assert tgt.calls == 2 * 5 + 2 * 3
    assert "density=4" not in timings and "iisph_accel=4" in timings
    assert timings["iisph_pressure=2"] == pytest.approx(110.0)


def test_step_knobs_are_timed_over_steps_in_turn(tmp_path):
    t = tune.Autotuner(cache_path=str(tmp_path / "c.json"), device="d")
    tgt = FakeTarget(COSTS, UNROLL, knobs=list(COSTS) + ["staging", "jacobi_unroll"],
                     staging_cost={0: 1.0e-3, 1: 0.4e-3})
    choice, _, timings = t.tune(tgt, "w")
    assert choice["staging"] == 1 and choice["jacobi_unroll"] == 2
    assert tgt.v["staging"] == 1
    # staging is decided first (at the default repeat count), then the
    # repeat count with staging on
    assert timings["staging=0"] == pytest.approx(4000.0) and timings["staging=1"] == pytest.approx(3400.0)
    assert timings["jacobi_unroll=2"] == pytest.approx(3300.0)
    assert tgt.calls == 2 * 5 + 2 * 2 + 2 * 3


def test_ties_keep_the_default(tmp_path):
    t = tune.Autotuner(cache_path=str(tmp_path / "c.json"), device="d")
    choice, _, _ = t.tune(FakeTarget({"density": [1e-4] * 4}, {1: 1e-3, 2: 1e-3, 4: 1e-3}), "w")
    assert choice == {"density": 0, "jacobi_unroll": 1}


def test_cache_is_keyed_by_device_and_workload(tmp_path):
    path = str(tmp_path / "sub" / "c.json")
    a = tune.Autotuner(cache_path=path, device="GB300")
    choice, _, _ = a.tune(FakeTarget(COSTS, UNROLL), "plain:f2^20")
    data = json.load(open(path))
    assert list(data) == ["GB300|plain:f2^20"] and data["GB300|plain:f2^20"]["choice"] == choice
    # a second tune of the same workload reads the cache: no measurement
    tgt = FakeTarget(COSTS, UNROLL)
    again, source, _ = a.tune(tgt, "plain:f2^20")
    assert (again, source, tgt.calls) == (choice, "cache", 0)
    assert tgt.v["iisph_accel"] == 3  # the cached choice is applied
    # another device or workload is tuned afresh; `force` re-tunes
    tgt = FakeTarget(COSTS, UNROLL)
    assert tune.Autotuner(cache_path=path, device="other").tune(tgt, "plain:f2^20")[1] == "tuned"
    assert a.tune(FakeTarget(COSTS, UNROLL), "plain:f2^15")[1] == "tuned"
    assert a.tune(FakeTarget(COSTS, UNROLL), "plain:f2^20", force=True)[1] == "tuned"
    assert len(json.load(open(path))) == 3


def test_stale_cache_entries_are_ignored(tmp_path):
    path = tmp_path / "c.json"
    path.write_text(json.dumps({"d|w": {"choice": {"iisph_accel": 9}}}))
    t = tune.Autotuner(cache_path=str(path), device="d")
    assert t.lookup("w") is None
    path.write_text("not json")
    assert t.lookup("w") is None


def test_knobs_outside_the_workload_are_not_measured(tmp_path):
    t = tune.Autotuner(cache_path=str(tmp_path / "c.json"), device="d")
    tgt = FakeTarget(COSTS, UNROLL, knobs=["iisph_accel"])
    choice, _, _ = t.tune(tgt, "w")
    assert choice == {"iisph_accel": 3}


def test_workload_classes():
    assert tune.workload_class("plain", 1_000_000) == "plain:f2^20"
    assert tune.workload_class("plain", 27_000) == "plain:f2^15"
    assert tune.workload_class("batched", 11_400_000, 256) == "batched:f2^23:s2^8"


def test_library_knob_table(gpu_lib):
    from prtcl_gb300._lib import INVALID
    table = tune.knob_table()
    assert set(table) == set(tune.VALUES)
    for k in tune.SWEEP_KNOBS:
        assert table[k].startswith("0 0=128x8/"), table[k]
    assert "batched:" in table["iisph_accel"]
    assert table["jacobi_unroll"].split()[0] == "1"
    assert gpu_lib.prtcl_gpu_model_tune_set(None, b"iisph_accel", 1) == INVALID
    assert gpu_lib.prtcl_gpu_batch_tune_get(None, b"iisph_accel", None) == INVALID
