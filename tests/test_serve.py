"""Serving loop (the native ``prtcl_gpu_server_*``): scheduling on the CPU
against a stand-in batch driven through callbacks (arrival order, HBM
budget, scene slots, completion, errors); on the GPU, every served request's
result is the same as the request run alone."""
import ctypes as C

import numpy as np
import pytest

from prtcl_gb300 import driver
from prtcl_gb300.serve import Request, Server, poisson_requests, report


@pytest.fixture(autouse=True)
def _library(gpu_lib):
    """The server is native: build / load the library (no GPU needed)."""
    return gpu_lib


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-6)


class FakeBatch:
    """Stand-in with the batch interface: 1 KB per particle, 10 ms a step."""

    def __init__(self, clock):
        self.clock = clock
        self.scenes = {}
        self.next = 1
        self.max_held = 0
        self.log = []

    def add_scene(self, f, b):
        sid = self.next
        self.next += 1
        self.scenes[sid] = [len(f), len(b), 0]
        self.log.append(("add", sid, len(f)))
        self.max_resident = max(getattr(self, "max_resident", 0), len(self.scenes))
        return sid

    def remove_scene(self, sid):
        del self.scenes[sid]

    def device_bytes(self):
        held = 1000 * sum(v[0] + v[1] for v in self.scenes.values())
        self.max_held = max(self.max_held, held)
        return held

    def step(self, k):
        for v in self.scenes.values():
            v[2] += k
        self.clock.t += 0.01 * k

    def info(self, sid):
        return {"jacobi_solves": float(self.scenes[sid][2]), "jacobi_capped": 0.0, "steps": self.scenes[sid][2]}

    def download(self, sid, field):
        return np.zeros((self.scenes[sid][0], 3), np.float32)

    def synchronize(self):
        pass


def serve(reqs, budget, batch=FakeBatch, **kw):
    clock = Clock()
    holder = {}

    def factory(p):
        holder["b"] = batch(clock)
        return holder["b"]

    srv = Server(factory, driver.DAM_BREAK_27K, budget_bytes=budget, clock=clock, sleep=clock.sleep,
                 bytes_per_particle=1000.0, **kw)
    done = srv.run(reqs)
    return srv, done, holder["b"]


def test_requests_are_seeded_and_shaped():
    a = poisson_requests(50, rate=5.0, seed=4, lo=5000, hi=500000, steps=(100, 1000))
    b = poisson_requests(50, rate=5.0, seed=4, lo=5000, hi=500000, steps=(100, 1000))
    assert [(r.arrival, r.fluid_cells, r.steps) for r in a] == [(r.arrival, r.fluid_cells, r.steps) for r in b]
    assert all(100 <= r.steps <= 1000 for r in a)
    arr = np.array([r.arrival for r in a])
    assert (np.diff(arr) > 0).all()
    assert 2.5 < len(arr) / arr[-1] < 10.0  # mean rate 5 / s
    n = np.array([np.prod(r.fluid_cells) for r in a])
    assert n.min() >= 2500 and n.max() <= 800000


def test_every_request_completes_in_arrival_order_of_admission():
    reqs = poisson_requests(12, rate=20.0, seed=5, lo=200, hi=2000, steps=(3, 12))
    srv, done, fb = serve(reqs, budget=1e12)
    assert len(done) == 12
    for r in done:
        assert r.info["steps"] == r.steps
        assert r.admitted >= r.arrival - 1e-12 and r.finished > r.admitted
        # at least one 10 ms step per requested step
        assert r.latency >= 0.01 * r.steps - 1e-9
    order = [e[1] for e in fb.log if e[0] == "add"]
    assert order == sorted(order)
    rep = report(done, srv.makespan, srv.particle_steps)
    assert rep["requests"] == 12 and rep["latency_p99_s"] >= rep["latency_p50_s"] > 0
    assert rep["particle_steps"] == sum(r.fluid * r.steps for r in done)


def test_budget_limits_resident_bytes():
    reqs = poisson_requests(10, rate=1000.0, seed=6, lo=1000, hi=3000, steps=(5, 10))
    one = max((np.prod(r.fluid_cells) * 12) for r in reqs) * 1000  # generous single-request bound
    budget = 3 * one
    srv, done, fb = serve(reqs, budget=budget)
    assert len(done) == 10
    assert fb.max_held <= budget


def test_scene_slots_limit_resident_requests():
    reqs = poisson_requests(9, rate=1000.0, seed=8, lo=200, hi=800, steps=(4, 9))
    srv, done, fb = serve(reqs, budget=1e12, max_scenes=2)
    assert len(done) == 9 and fb.max_resident == 2
    assert sum(r.fluid * r.steps for r in done) == srv.particle_steps


def test_ties_in_arrival_keep_submission_order_and_results():
    reqs = [Request(rid=k, arrival=0.5, fluid_cells=(2 + k, 2, 2), steps=3) for k in range(4)]
    srv, done, fb = serve(reqs, budget=1e12)
    assert [e[2] for e in fb.log if e[0] == "add"] == [8 * (2 + k) // 2 for k in range(4)]
    assert [r.rid for r in done] == [0, 1, 2, 3]  # same step count: retired in admission order
    for r in done:
        assert r.result.shape == (r.fluid, 3) and r.admitted == 0.5
    _, done, _ = serve([Request(rid=0, arrival=0.0, fluid_cells=(2, 2, 2), steps=2)], budget=1e12,
                       keep_results=False)
    assert done[0].result is None


class FailingBatch(FakeBatch):
    def step(self, k):
        if sum(v[2] for v in self.scenes.values()) > 5:
            raise RuntimeError("stand-in step failed")
        super().step(k)


def test_batch_errors_reach_the_caller():
    reqs = poisson_requests(3, rate=1000.0, seed=9, lo=200, hi=400, steps=(10, 12))
    with pytest.raises(RuntimeError, match="stand-in step failed"):
        serve(reqs, budget=1e12, batch=FailingBatch)


def test_failed_step_retires_the_resident_requests():
    """A failed batch step leaves the resident scenes' state undefined: each
    resident request is retired as failed, with the steps it completed, and
    its scene removed; queued requests stay queued; the server serves on."""
    clock = Clock()
    holder = {}

    def factory(p):
        holder["b"] = FailingBatch(clock)
        return holder["b"]

    srv = Server(factory, driver.DAM_BREAK_27K, budget_bytes=1e12, clock=clock, sleep=clock.sleep,
                 bytes_per_particle=1000.0, max_scenes=2)
    reqs = [Request(rid=k, arrival=0.0, fluid_cells=(2, 2, 2), steps=20) for k in range(3)]
    with pytest.raises(RuntimeError, match="stand-in step failed"):
        srv.run(reqs)
    assert sorted(r.rid for r in srv.done) == [0, 1]
    assert all(r.status == "failed" and r.result is None and 0 < r.done_steps < 20 for r in srv.done)
    st = srv._status()
    assert (st.pending, st.running, st.results) == (1, 0, 0)
    assert holder["b"].scenes == {}


def test_oversized_request_is_refused_at_submit():
    """A request whose own estimate exceeds the budget is refused even when
    nothing is resident: it never reaches the device allocator."""
    from prtcl_gb300 import PrtclGpuError
    with pytest.raises(PrtclGpuError, match="more than the budget"):
        serve([Request(rid=0, arrival=0.0, fluid_cells=(4, 4, 4), steps=2)], budget=1000.0 * 100)


def test_request_rejected_when_its_estimate_outgrows_the_budget():
    """The estimate per particle is learnt from the batch: a request that
    fitted the first estimate at submit but not the learnt one is retired
    unrun as rejected, and the others are served."""
    clock = Clock()
    srv = Server(lambda p: FakeBatch(clock), driver.DAM_BREAK_27K, budget_bytes=1000.0 * 800, clock=clock,
                 sleep=clock.sleep, bytes_per_particle=10.0)
    small = Request(rid=0, arrival=0.0, fluid_cells=(2, 2, 2), steps=3)
    large = Request(rid=1, arrival=0.0, fluid_cells=(6, 6, 6), steps=3)   # 216 fluid + its walls
    done = srv.run([small, large])
    st = {r.rid: r for r in done}
    assert st[0].status == "done" and st[0].done_steps == 3
    assert st[1].status == "rejected" and st[1].done_steps == 0 and st[1].admitted == -1.0


def test_cancel_queued_and_resident_requests():
    clock = Clock()
    holder = {}

    def factory(p):
        holder["b"] = FakeBatch(clock)
        return holder["b"]

    srv = Server(factory, driver.DAM_BREAK_27K, budget_bytes=1e12, clock=clock, sleep=clock.sleep,
                 bytes_per_particle=1000.0, max_scenes=1)
    reqs = [Request(rid=0, arrival=0.0, fluid_cells=(2, 2, 2), steps=10, cancel_at=0.055),   # resident
            Request(rid=1, arrival=0.0, fluid_cells=(2, 2, 2), steps=10, cancel_at=0.025),   # queued
            Request(rid=2, arrival=0.0, fluid_cells=(2, 2, 2), steps=4)]
    done = srv.run(reqs)
    st = {r.rid: r for r in done}
    assert st[1].status == "cancelled" and st[1].done_steps == 0 and st[1].admitted == -1.0
    assert st[0].status == "cancelled" and 0 < st[0].done_steps < 10 and st[0].result is None
    assert st[2].status == "done" and st[2].done_steps == 4
    assert [r.rid for r in done] == [1, 0, 2]
    assert holder["b"].scenes == {}
    assert srv.cancel(2) is False  # already retired


class FlakyReadBatch(FakeBatch):
    """Stand-in whose download fails once and whose remove fails once."""

    def __init__(self, clock):
        super().__init__(clock)
        self.download_failures = 1
        self.remove_failures = 1

    def download(self, sid, field):
        if self.download_failures:
            self.download_failures -= 1
            raise RuntimeError("stand-in download failed")
        return super().download(sid, field)

    def remove_scene(self, sid):
        if self.remove_failures:
            self.remove_failures -= 1
            raise RuntimeError("stand-in remove failed")
        super().remove_scene(sid)


def test_failed_retirement_fails_that_request_alone():
    """A request whose results cannot be read is retired as failed with the
    steps it asked for (never stepped again); a scene whose removal failed
    is removed at a later turn."""
    clock = Clock()
    holder = {}

    def factory(p):
        holder["b"] = FlakyReadBatch(clock)
        return holder["b"]

    srv = Server(factory, driver.DAM_BREAK_27K, budget_bytes=1e12, clock=clock, sleep=clock.sleep,
                 bytes_per_particle=1000.0)
    reqs = [Request(rid=0, arrival=0.0, fluid_cells=(2, 2, 2), steps=3),
            Request(rid=1, arrival=0.0, fluid_cells=(2, 2, 2), steps=6)]
    done = srv.run(reqs)
    st = {r.rid: r for r in done}
    assert st[0].status == "failed" and st[0].done_steps == 3 and st[0].result is None
    assert st[1].status == "done" and st[1].done_steps == 6 and st[1].result.shape == (8, 3)
    assert holder["b"].scenes == {}
    assert srv.particle_steps == 8 * 3 + 8 * 6


class RefusingBatch(FakeBatch):
    def add_scene(self, f, b):
        raise MemoryError("stand-in batch is full")


def test_a_refused_admission_keeps_the_request_queued():
    clock = Clock()
    srv = Server(lambda p: RefusingBatch(clock), driver.DAM_BREAK_27K, budget_bytes=1e12, clock=clock,
                 sleep=clock.sleep)
    with pytest.raises(MemoryError):
        srv.run([Request(rid=0, arrival=0.0, fluid_cells=(2, 2, 2), steps=2)])
    st = srv._status()
    assert (st.pending, st.running, st.results) == (1, 0, 0)


def test_server_rejects_invalid_requests(gpu_lib):
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300._lib import ServerParams, check
    srv = Server(lambda p: FakeBatch(Clock()), driver.DAM_BREAK_27K, budget_bytes=1e9)
    x = np.zeros((4, 3), np.float32)
    with pytest.raises(PrtclGpuError, match="at least one step"):
        check(gpu_lib.prtcl_gpu_server_submit(srv._h, 0, 0.0, x.ctypes.data, 4, x.ctypes.data, 4, 0))
    with pytest.raises(PrtclGpuError, match="not finite"):
        check(gpu_lib.prtcl_gpu_server_submit(srv._h, 0, float("nan"), x.ctypes.data, 4, x.ctypes.data, 4, 1))
    sp = ServerParams()
    sp.max_scenes = 0
    h = C.c_void_p()
    with pytest.raises(PrtclGpuError, match="max_scenes"):
        check(gpu_lib.prtcl_gpu_server_create_custom(C.byref(srv._ops), None, C.byref(sp), C.byref(h)))


def test_server_abi_argument_checks(gpu_lib):
    from prtcl_gb300 import PrtclGpuError
    from prtcl_gb300._lib import INVALID, RequestResult, ServerStatus, check
    assert gpu_lib.prtcl_gpu_server_turn(None, None) == INVALID
    assert gpu_lib.prtcl_gpu_server_status_get(None, None) == INVALID
    assert gpu_lib.prtcl_gpu_server_create(None, None, None) == INVALID
    assert gpu_lib.prtcl_gpu_server_destroy(None) == 0
    clock = Clock()
    srv = Server(lambda p: FakeBatch(clock), driver.DAM_BREAK_27K, budget_bytes=1e12, clock=clock, sleep=clock.sleep)
    x = np.zeros((8, 3), np.float32)
    assert gpu_lib.prtcl_gpu_server_submit(srv._h, 0, 0.0, x.ctypes.data, -1, x.ctypes.data, 8, 2) == INVALID
    check(gpu_lib.prtcl_gpu_server_submit(srv._h, 7, 0.0, x.ctypes.data, 8, x.ctypes.data, 8, 2))
    stepped = C.c_int32(0)
    for _ in range(2):
        check(gpu_lib.prtcl_gpu_server_turn(srv._h, C.byref(stepped)))
        assert stepped.value == 1
    st = ServerStatus()
    check(gpu_lib.prtcl_gpu_server_status_get(srv._h, C.byref(st)))
    assert (st.pending, st.running, st.results, st.steps_run, st.particle_steps) == (0, 0, 1, 2, 16)
    res, has = RequestResult(), C.c_int32(0)
    small = np.zeros((4, 3), np.float32)
    with pytest.raises(PrtclGpuError, match="smaller than"):
        check(gpu_lib.prtcl_gpu_server_next_result(srv._h, C.byref(res), small.ctypes.data, 4, C.byref(has)))
    out = np.ones((8, 3), np.float32)
    check(gpu_lib.prtcl_gpu_server_next_result(srv._h, C.byref(res), out.ctypes.data, 8, C.byref(has)))
    assert has.value == 1 and res.request_id == 7 and res.steps == 2 and (out == 0).all()
    check(gpu_lib.prtcl_gpu_server_next_result(srv._h, C.byref(res), None, 0, C.byref(has)))
    assert has.value == 0
    check(gpu_lib.prtcl_gpu_server_turn(srv._h, C.byref(stepped)))
    assert stepped.value == 0


@pytest.mark.gpu
def test_served_results_match_alone():
    from prtcl_gb300.batch import Batch
    p = dict(driver.DAM_BREAK_27K)
    reqs = poisson_requests(6, rate=200.0, seed=7, lo=600, hi=2500, steps=(6, 18))
    srv = Server(Batch, p, budget_bytes=120e9)
    done = srv.run(reqs)
    assert len(done) == 6
    for r in done:
        bt = Batch(p)
        sc = r.scene()
        sid = bt.add_scene(sc["fluid"], sc["boundary"])
        bt.step(r.steps)
        alone = bt.download(sid, "position")
        assert np.array_equal(alone.view(np.uint32), r.result.view(np.uint32)), r.rid
        assert bt.info(sid)["jacobi_iterations"] == r.info["jacobi_iterations"]
