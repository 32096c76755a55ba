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

The loop itself is native (``prtcl_gpu_server_*``, csrc/server.cu); this
module submits requests as they arrive, turns the server and collects the
results.  The batch is injected (``batch_factory``), so the scheduling logic
runs on the CPU against a stand-in in the tests.
"""
from __future__ import annotations

import ctypes as C
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
    cancel_at: float = math.inf  # the client cancels the request at this time
    # filled in by the server
    admitted: float = math.nan
    finished: float = math.nan
    done_steps: int = 0
    fluid: int = 0
    boundary: int = 0
    info: dict = field(default_factory=dict)
    result: np.ndarray | None = None
    status: str = ""        # done, cancelled, rejected or failed
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
    """The native serving loop (``prtcl_gpu_server_*``) driven from Python.

    ``batch_factory``: ``prtcl_gb300.batch.Batch`` (or None) serves on the
    device through the server's own batch; any other factory's object (the
    batch interface: add_scene, remove_scene, step, synchronize,
    device_bytes, info, download) is driven through callbacks, so the
    scheduling runs on the CPU against a stand-in in the tests.
    ``budget_bytes``: device bytes the batch may hold (admission limit);
    ``bytes_per_particle``: estimate for a request not yet admitted,
    replaced by the batch's measured bytes per particle once it holds
    scenes.  ``clock`` / ``sleep`` give the server its time (seconds)."""

    def __init__(self, batch_factory, params, budget_bytes=120e9, max_scenes=4096, bytes_per_particle=1000.0,
                 clock=time.perf_counter, sleep=time.sleep, keep_results=True):
        from ._lib import CLOCK_FN, ServerParams, check, load
        from .batch import Batch, params_struct
        self.clock, self.sleep = clock, sleep
        self.keep_results = keep_results
        self.steps_run = 0
        self.particle_steps = 0
        self.makespan = 0.0
        self._t0 = clock()
        self._error = None
        self._clock_fn = CLOCK_FN(lambda _user: self.clock() - self._t0)
        sp = ServerParams()
        sp.budget_bytes = float(budget_bytes)
        sp.max_scenes = int(max_scenes)
        sp.keep_results = 1 if keep_results else 0
        sp.bytes_per_particle = float(bytes_per_particle)
        sp.clock = self._clock_fn
        sp.clock_user = None
        h = C.c_void_p()
        if batch_factory is None or batch_factory is Batch:
            self.batch = None
            check(load().prtcl_gpu_server_create(C.byref(params_struct(params)), C.byref(sp), C.byref(h)))
        else:
            self.batch = batch_factory(params)
            self._ops = self._callback_ops(self.batch)
            check(load().prtcl_gpu_server_create_custom(C.byref(self._ops), None, C.byref(sp), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            from ._lib import load
            load().prtcl_gpu_server_destroy(h)
            self._h = None

    def _callback_ops(self, bt):
        """prtcl_gpu_server_batch_ops over a Python batch object; an exception
        in a callback fails the operation and, if the server call then fails,
        is raised after the call."""
        from ._lib import SceneInfo, ServerBatchOps

        def guarded(fn):
            def call(*a):
                try:
                    fn(*a)
                    return 0
                except BaseException as e:  # re-raised by _call
                    self._error = e
                    return 1
            return call

        def xyz(ptr, n):
            return np.ctypeslib.as_array(ptr, shape=(n, 3)).copy() if n else np.zeros((0, 3), np.float32)

        def add_scene(_u, f, nf, b, nb, out):
            out[0] = int(bt.add_scene(xyz(f, nf), xyz(b, nb)))

        def scene_info(_u, sid, out):
            d = bt.info(sid)
            for k, t in SceneInfo._fields_:
                if k in d:
                    setattr(out.contents, k, int(d[k]) if t in (C.c_int32, C.c_int64) else float(d[k]))

        def download(_u, sid, host, n):
            if n:
                np.ctypeslib.as_array(host, shape=(n, 3))[:] = bt.download(sid, "position")

        def device_bytes(_u, out):
            out[0] = int(bt.device_bytes())

        T = dict(ServerBatchOps._fields_)
        return ServerBatchOps(
            add_scene=T["add_scene"](guarded(add_scene)),
            remove_scene=T["remove_scene"](guarded(lambda _u, sid: bt.remove_scene(sid))),
            step=T["step"](guarded(lambda _u, k: bt.step(k))),
            synchronize=T["synchronize"](guarded(lambda _u: bt.synchronize())),
            device_bytes=T["device_bytes"](guarded(device_bytes)),
            scene_info=T["scene_info"](guarded(scene_info)),
            download_positions=T["download_positions"](guarded(download)))

    def _call(self, fn, *args):
        from ._lib import check
        self._error = None
        rc = fn(self._h, *args)
        err, self._error = self._error, None
        # a callback error the server handled itself (a failed retirement)
        # leaves the call successful: it shows in that request's status
        if rc != 0 and err is not None:
            raise err
        check(rc)

    def cancel(self, key):
        """Cancel the submitted request ``key`` (queued or resident): it is
        retired with status ``cancelled``.  False if no queued or resident
        request has that key."""
        from ._lib import load
        found = C.c_int32(0)
        self._call(load().prtcl_gpu_server_cancel, int(key), C.byref(found))
        return bool(found.value)

    def _status(self):
        from ._lib import ServerStatus, load
        st = ServerStatus()
        self._call(load().prtcl_gpu_server_status_get, C.byref(st))
        return st

    def run(self, requests):
        """Serve ``requests`` (each submitted when its arrival time has come,
        and cancelled at its ``cancel_at``) until all are retired; returns
        them in retirement order, each with its ``status``.  If a turn
        raises (a failed batch step), the requests retired so far, the
        failed ones included, are in ``self.done``."""
        from ._lib import load
        L = load()
        self._t0 = self.clock()
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        inflight = {}
        done = self.done = []  # also readable when a turn raised
        buf = np.empty((0, 3), np.float32)
        stepped = C.c_int32(0)
        cancelled = set()
        while True:
            now = self.clock() - self._t0
            while pending and pending[0].arrival <= now:
                req = pending.popleft()
                sc = req.scene()
                f = np.ascontiguousarray(sc["fluid"], np.float32).reshape(-1, 3)
                bd = np.ascontiguousarray(sc["boundary"], np.float32).reshape(-1, 3)
                key = len(done) + len(inflight)
                while key in inflight:
                    key += 1
                self._call(L.prtcl_gpu_server_submit, key, float(req.arrival), f.ctypes.data, len(f),
                           bd.ctypes.data, len(bd), int(req.steps))
                req.fluid, req.boundary = len(f), len(bd)
                req.release()
                inflight[key] = req
            for key, req in list(inflight.items()):
                if req.cancel_at <= now and key not in cancelled:
                    cancelled.add(key)
                    self.cancel(key)
            st = self._status()
            if not pending and st.pending == 0 and st.running == 0 and st.results == 0:
                break
            try:
                self._call(L.prtcl_gpu_server_turn, C.byref(stepped))
            finally:
                # results retired by the turn, also those of a failed step
                buf = self._collect(inflight, done, buf)
            if not stepped.value:
                # nothing resident: wait for the next arrival
                st = self._status()
                nxt = min([st.next_arrival, pending[0].arrival if pending else math.inf]
                          + [r.cancel_at for k, r in inflight.items() if k not in cancelled])
                if math.isfinite(nxt):
                    self.sleep(max(0.0, nxt - (self.clock() - self._t0)))
        st = self._status()
        self.steps_run, self.particle_steps = int(st.steps_run), int(st.particle_steps)
        self.makespan = self.clock() - self._t0
        return done

    def _collect(self, inflight, done, buf):
        """Move the server's unread results onto their requests."""
        from ._lib import REQUEST_STATUS, RequestResult, load
        L = load()
        res, has = RequestResult(), C.c_int32(0)
        if self.keep_results and inflight:
            need = max(r.fluid for r in inflight.values())
            if len(buf) < need:
                buf = np.empty((need, 3), np.float32)
        while True:
            self._call(L.prtcl_gpu_server_next_result, C.byref(res),
                       buf.ctypes.data if self.keep_results else None, len(buf), C.byref(has))
            if not has.value:
                return buf
            req = inflight.pop(res.request_id)
            req.admitted, req.finished = res.admitted, res.finished
            req.done_steps = int(res.steps)
            req.status = REQUEST_STATUS.get(int(res.status), str(res.status))
            req.info = {k: getattr(res.info, k) for k, _ in res.info._fields_ if k != "pad"}
            if self.keep_results and req.status == "done":
                req.result = buf[:req.fluid].copy()
            done.append(req)


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
