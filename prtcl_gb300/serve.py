"""Serving loop: continuous batching of simulation requests.

Requests (dam-break scenes with a fluid count and a step count) arrive over
time.  The server keeps every admitted scene resident on the device in one
batch (``prtcl_gb300.batch.Batch``) and steps all of them together, one step
per loop turn.  Between turns it admits the requests that have arrived, in
arrival order, while the batch's device bytes stay within the HBM budget and
a slot is free, and retires the requests that have taken all their steps
(their final fluid positions are downloaded as the result).  Because every
scene converges on its own and its neighbour order does not depend on the
other scenes, a request's result is the same alone and in the mix.

The batch is injected (``batch_factory``), so the scheduling logic runs on
the CPU against a stand-in in the tests.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import scenes


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    fluid_cells: tuple      # fluid block in lattice cells
    steps: int
    seed: int = 0
    # filled in by the server
    admitted: float = math.nan
    finished: float = math.nan
    done_steps: int = 0
    fluid: int = 0
    boundary: int = 0
    info: dict = field(default_factory=dict)
    result: np.ndarray | None = None
    _scene: dict | None = field(default=None, repr=False)

    @property
    def latency(self):
        return self.finished - self.arrival

    def scene(self, spacing=0.025):
        """The request's particles (generated once; a client brings them
        with the request, so generate them before a timed run)."""
        if self._scene is None:
            box = tuple(2.0 * c * spacing for c in self.fluid_cells)
            self._scene = scenes.dam_break(fluid_cells=self.fluid_cells, spacing=spacing, box=box)
        return self._scene

    def release(self):
        self._scene = None


def poisson_requests(count, rate, seed=4, lo=5000, hi=500000, steps=(100, 1000)):
    """``count`` requests with exponential inter-arrival times of mean
    1 / ``rate`` s, fluid counts log-uniform in [lo, hi], block aspect ratios
    uniform in [0.5, 2] and step counts uniform in [steps[0], steps[1]]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        nf = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        ax, az = rng.uniform(0.5, 2.0, size=2)
        c = (nf / (ax * az)) ** (1.0 / 3.0)
        cells = (max(1, int(round(ax * c))), max(1, int(round(c))), max(1, int(round(az * c))))
        out.append(Request(rid=k, arrival=t, fluid_cells=cells, steps=int(rng.integers(steps[0], steps[1] + 1)),
                           seed=k))
    return out


class Server:
    """``budget_bytes``: device bytes the batch may hold (admission limit);
    ``bytes_per_particle``: estimate for a request not yet admitted, replaced
    by the batch's measured bytes per particle once it holds scenes."""

    def __init__(self, batch_factory, params, budget_bytes=120e9, max_scenes=4096, bytes_per_particle=1000.0,
                 clock=time.perf_counter, sleep=time.sleep, keep_results=True):
        self.batch = batch_factory(params)
        self.budget = float(budget_bytes)
        self.max_scenes = int(max_scenes)
        self.bpp = float(bytes_per_particle)
        self.clock, self.sleep = clock, sleep
        self.keep_results = keep_results
        self.steps_run = 0
        self.particle_steps = 0

    def _estimate(self, req, scene):
        return (len(scene["fluid"]) + len(scene["boundary"])) * self.bpp

    def run(self, requests):
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        running = {}
        done = []
        held = 0.0
        t0 = self.clock()
        while pending or running:
            now = self.clock() - t0
            # admit in arrival order while the budget and the slots allow
            while pending and pending[0].arrival <= now and len(running) < self.max_scenes:
                req = pending[0]
                sc = req.scene()
                need = self._estimate(req, sc)
                # (a request alone is always admitted, even above the budget)
                if running and held + need > self.budget:
                    break
                pending.popleft()
                sid = self.batch.add_scene(sc["fluid"], sc["boundary"])
                req.release()
                req.admitted = now
                req.fluid, req.boundary = len(sc["fluid"]), len(sc["boundary"])
                running[sid] = req
                held = float(self.batch.device_bytes())
                nparts = sum(r.fluid + r.boundary for r in running.values())
                if nparts:
                    self.bpp = max(self.bpp, held / nparts)
            if not running:
                if pending:
                    self.sleep(max(0.0, pending[0].arrival - (self.clock() - t0)))
                continue
            self.batch.step(1)
            self.steps_run += 1
            self.particle_steps += sum(r.fluid for r in running.values())
            finished = []
            for sid, req in running.items():
                req.done_steps += 1
                if req.done_steps >= req.steps:
                    finished.append(sid)
            for sid in finished:
                req = running.pop(sid)
                req.info = self.batch.info(sid)
                if self.keep_results:
                    req.result = self.batch.download(sid, "position")
                else:
                    self.batch.synchronize()
                req.finished = self.clock() - t0
                self.batch.remove_scene(sid)
                done.append(req)
            if finished:
                held = float(self.batch.device_bytes()) if running else 0.0
        self.makespan = self.clock() - t0
        return done


def report(done, makespan, particle_steps, eta=1e-3):
    """Throughput, latency percentiles and density-error compliance."""
    lat = np.array([r.latency for r in done]) if done else np.zeros(1)
    solves = sum(r.info.get("jacobi_solves", 0.0) for r in done)
    capped = sum(r.info.get("jacobi_capped", 0.0) for r in done)
    return {
        "requests": len(done),
        "particle_steps": int(particle_steps),
        "makespan_s": makespan,
        "particle_steps_per_s": particle_steps / makespan if makespan > 0 else 0.0,
        "latency_p50_s": float(np.percentile(lat, 50)),
        "latency_p99_s": float(np.percentile(lat, 99)),
        # steps whose Jacobi loop ended below the density-error bound (the
        # others stopped at the iteration cap)
        "converged_step_fraction": (solves - capped) / solves if solves else 1.0,
        "density_error_bound": eta,
    }
