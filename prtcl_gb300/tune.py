"""Autotuner for the launch-shape knobs of the neighbour sweeps and the
relaxed-Jacobi loop (prtcl_gpu_model_tune_set / prtcl_gpu_batch_tune_set).

Every knob value gives bit-identical results (see include/prtcl_gpu.h), so
the tuner is free to pick the fastest per workload:

* the sweep knobs (density, iisph_setup, iisph_accel, iisph_pressure,
  wkbb18_diag, pcg_init, pcg_q) select a launch shape: threads per block,
  blocks resident per SM (the register cap) and neighbour-walk batch;
* jacobi_unroll is the number of relaxed-Jacobi iterations per iteration of
  the device loop's graph (1, 2 or 4);
* staging (single-scene models) builds staged neighbour lists and runs the
  staged relaxed-Jacobi and PCG sweeps, which read their neighbours'
  records from shared memory (0 or 1);
* grid_sort (single-scene models whose grid holds at most 128k items)
  sorts the grid in one launch of a thread-block cluster instead of the
  tiled radix-sort launches (0 or 1);
* list_split (query groups of at most 64k items) builds each query's lists
  with four threads, each walking a quarter of its cells (0 or 1).

The cell size is not a knob: it equals the search radius, as in the
reference's grid (util/grouped_uniform_grid.hpp:621-632), because the
neighbour order, and with it every sum, depends on it.

Search.  The sweeps are independent kernels, so one profiled run per shape
index times every sweep knob at once (each kernel with its own variant);
each (knob, value) is measured twice, in rising and falling order, and the
smaller time counts.  The step knobs (grid_sort, list_split, staging,
then jacobi_unroll) are timed over whole steps, one after the other, the
same way.  Workloads
run on their own copy of the scene, so a tuned run starts from the same
state as an untuned one.

Cache.  Choices persist in a JSON file keyed by the device name and a
workload class (plain or batched, with the fluid count and scene count in
powers of two): ``$PRTCL_GB300_TUNE_CACHE``, else
``~/.cache/prtcl_gb300/tuning.json``.
"""
from __future__ import annotations

import json
import math
import os
import time

SWEEP_KNOBS = ("density", "iisph_setup", "iisph_accel", "iisph_pressure", "wkbb18_diag", "pcg_init", "pcg_q")
VALUES = {**{k: (0, 1, 2, 3) for k in SWEEP_KNOBS}, "pcg_q": (0, 1, 2, 3, 4), "iisph_accel": (0, 1, 2, 3, 4),
          "iisph_pressure": (0, 1, 2, 3, 4), "jacobi_unroll": (1, 2, 4), "staging": (0, 1), "grid_sort": (0, 1),
          "list_split": (0, 1)}
DEFAULTS = {**{k: 0 for k in SWEEP_KNOBS}, "jacobi_unroll": 1, "staging": 0, "grid_sort": 1, "list_split": 1}
# knobs timed over whole steps, in this order
STEP_KNOBS = ("grid_sort", "list_split", "staging", "jacobi_unroll")


def knob_table():
    """{knob: text} of the library's knob table (prtcl_gpu_tune_knobs)."""
    from ._lib import load, read_str
    out = {}
    for line in read_str(load().prtcl_gpu_tune_knobs).splitlines():
        name, _, rest = line.partition(" ")
        out[name] = rest
    return out


def default_cache_path():
    p = os.environ.get("PRTCL_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "prtcl_gb300", "tuning.json")


def device_name():
    """Name of CUDA device 0 (NVML through nvidia-smi; 'unknown' if absent)."""
    import subprocess
    try:
        r = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                           capture_output=True, text=True, timeout=20)
        name = r.stdout.strip().splitlines()[0] if r.returncode == 0 and r.stdout.strip() else ""
    except (OSError, subprocess.TimeoutExpired, IndexError):
        name = ""
    return name or "unknown"


def workload_class(kind, fluid, scenes=1):
    """plain:f2^k or batched:f2^k:s2^m (fluid particles, scenes; powers of
    two rounded to the nearest)."""
    f = int(round(math.log2(max(fluid, 1))))
    if kind == "plain":
        return f"plain:f2^{f}"
    return f"{kind}:f2^{f}:s2^{int(round(math.log2(max(scenes, 1))))}"


class Autotuner:
    """Search and cache of knob choices.  ``timer`` (seconds, monotonic) is
    injectable for tests."""

    def __init__(self, cache_path=None, device=None, timer=time.perf_counter):
        self.path = cache_path or default_cache_path()
        self.device = device or device_name()
        self.timer = timer

    def _load(self):
        try:
            with open(self.path) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}

    def key(self, workload):
        return f"{self.device}|{workload}"

    def lookup(self, workload):
        rec = self._load().get(self.key(workload))
        if not rec:
            return None
        choice = rec.get("choice", {})
        if any(k not in VALUES or v not in VALUES[k] for k, v in choice.items()):
            return None
        return choice

    def store(self, workload, choice, timings):
        data = self._load()
        data[self.key(workload)] = {"choice": choice, "timings_us": timings, "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        tmp = self.path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    def tune(self, target, workload, force=False):
        """The choice for ``workload`` (from the cache unless ``force``),
        applied to ``target``.  Returns (choice, source, timings)."""
        if not force:
            cached = self.lookup(workload)
            if cached is not None:
                for k, v in cached.items():
                    target.set(k, v)
                return cached, "cache", None
        timings = {}
        sweeps = [k for k in SWEEP_KNOBS if k in target.knobs()]
        best = {}
        shapes = sorted({v for k in sweeps for v in VALUES[k]})
        for order in (shapes, tuple(reversed(shapes))):
            for v in order:
                for k in sweeps:
                    target.set(k, v if v in VALUES[k] else DEFAULTS[k])
                per = target.measure_kernels(sweeps)
                for k in sweeps:
                    if k in per and v in VALUES[k]:
                        t = per[k]
                        key = f"{k}={v}"
                        timings[key] = min(timings.get(key, math.inf), t * 1e6)
        for k in sweeps:
            cand = [(timings[f"{k}={v}"], v) for v in VALUES[k] if f"{k}={v}" in timings]
            best[k] = min(cand)[1] if cand else DEFAULTS[k]
            target.set(k, best[k])
        for k in STEP_KNOBS:
            if k not in target.knobs():
                continue
            for order in (VALUES[k], tuple(reversed(VALUES[k]))):
                for v in order:
                    target.set(k, v)
                    t = target.measure_steps()
                    key = f"{k}={v}"
                    timings[key] = min(timings.get(key, math.inf), t * 1e6)
            best[k] = min((timings[f"{k}={v}"], v) for v in VALUES[k])[1]
            target.set(k, best[k])
        self.store(workload, best, {k: round(v, 2) for k, v in timings.items()})
        return best, "tuned", timings


class PlainTarget:
    """A single-scene model stepped by the reference driver loop
    (prtcl_gb300.driver.StepLoop with the device Jacobi loop)."""

    def __init__(self, scene, loop, probe_steps=3, grid_items=None, fluid_items=None):
        self.d, self.loop, self.n = scene, loop, probe_steps
        self.viscosity = bool(loop.p.get("viscosity"))
        # items of the grid (fluid and boundary) and of the fluid group, where
        # known: grid_sort and list_split are knobs only for the sizes they take
        self.grid_items = float("inf") if grid_items is None else grid_items
        self.fluid_items = float("inf") if fluid_items is None else fluid_items

    def knobs(self):
        k = ["density", "iisph_setup", "iisph_accel", "iisph_pressure", "jacobi_unroll", "staging"]
        if self.grid_items <= 128_000:
            k.append("grid_sort")
        if self.fluid_items <= 65_536:
            k.append("list_split")
        if self.viscosity:
            k += ["wkbb18_diag", "pcg_init", "pcg_q"]
        return k

    def set(self, knob, value):
        self.d.model.tune_set(knob, value)

    def get(self, knob):
        return self.d.model.tune_get(knob)

    def measure_kernels(self, names):
        """Mean seconds per launch of each kernel over the probe steps
        (CUDA events around each launch)."""
        m = self.d.model
        m.profile(True)
        m.profile_reset()
        for _ in range(self.n):
            self.loop.step(quiet=True)
        self.d.synchronize()
        prof = m.profile_read()
        m.profile(False)
        return {k: prof[k][1] / 1e3 / prof[k][0] for k in names if k in prof and prof[k][0]}

    def measure_steps(self):
        """Seconds per step (device loops in their graphs), host clock
        around synchronised steps, after one untimed step (a changed knob
        rebuilds the loops' graphs on their next launch)."""
        self.loop.step(quiet=True)
        self.d.synchronize()
        t0 = time.perf_counter()
        for _ in range(self.n):
            self.loop.step(quiet=True)
        self.d.synchronize()
        return (time.perf_counter() - t0) / self.n


class BatchTarget:
    """A batch of scenes (prtcl_gb300.batch.Batch)."""

    def __init__(self, batch, viscosity=False, probe_steps=2):
        self.b, self.n, self.viscosity = batch, probe_steps, viscosity

    def knobs(self):
        k = ["density", "iisph_setup", "iisph_accel", "iisph_pressure", "jacobi_unroll"]
        if self.viscosity:
            k += ["wkbb18_diag", "pcg_init", "pcg_q"]
        return k

    def set(self, knob, value):
        self.b.tune_set(knob, value)

    def get(self, knob):
        return self.b.tune_get(knob)

    def measure_kernels(self, names):
        self.b.profile(True)
        self.b.profile_read()
        self.b.step(self.n)
        self.b.synchronize()
        prof = self.b.profile_read()
        self.b.profile(False)
        return {k: prof[k][1] / 1e3 / prof[k][0] for k in names if k in prof and prof[k][0]}

    def measure_steps(self):
        self.b.step(1)  # untimed: a changed knob rebuilds the loops' graphs
        self.b.synchronize()
        t0 = time.perf_counter()
        self.b.step(self.n)
        self.b.synchronize()
        return (time.perf_counter() - t0) / self.n


def tune_plain(scene, params, tuner=None, warmup=3, force=False):
    """Tune the knobs for a single-scene workload on a copy of the scene
    (set up and stepped `warmup` steps); returns (choice, source, timings)."""
    from . import driver
    from .core import DeviceScene
    tuner = tuner or Autotuner()
    workload = workload_class("plain", len(scene["fluid"]))
    cached = None if force else tuner.lookup(workload)
    if cached is not None:
        return cached, "cache", None
    d = DeviceScene()
    driver.setup_dam_break(d, scene, params)
    loop = driver.StepLoop(d, params, device_loop=True)
    for _ in range(warmup):
        loop.step(quiet=True)
    return tuner.tune(PlainTarget(d, loop, grid_items=len(scene["fluid"]) + len(scene.get("boundary", ())),
                                  fluid_items=len(scene["fluid"])),
                      workload, force=True)


def tune_batched(scene_list, params, tuner=None, warmup=2, force=False):
    """Tune the knobs for a batch of scenes on a copy of the batch."""
    from .batch import Batch
    tuner = tuner or Autotuner()
    workload = workload_class("batched", sum(len(x["fluid"]) for x in scene_list), len(scene_list))
    cached = None if force else tuner.lookup(workload)
    if cached is not None:
        return cached, "cache", None
    bt = Batch(params)
    for x in scene_list:
        bt.add_scene(x["fluid"], x["boundary"])
    bt.step(warmup)
    return tuner.tune(BatchTarget(bt, viscosity=bool(params.get("viscosity"))), workload, force=True)


def apply(target_model, choice):
    """Set every knob of ``choice`` on a Model or Batch (anything with
    tune_set)."""
    for k, v in choice.items():
        target_model.tune_set(k, v)
