"""Serving loop: scheduling on the CPU against a stand-in batch (arrival
order, HBM budget, completion); on the GPU, every served request's result is
the same as the request run alone."""
import numpy as np
import pytest

from prtcl_gb300 import driver
from prtcl_gb300.serve import Server, poisson_requests, report


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
        self.log.append(("add", sid))
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


def serve(reqs, budget):
    clock = Clock()
    holder = {}

    def factory(p):
        holder["b"] = FakeBatch(clock)
        return holder["b"]

    srv = Server(factory, driver.DAM_BREAK_27K, budget_bytes=budget, clock=clock, sleep=clock.sleep,
                 bytes_per_particle=1000.0)
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
    order = [sid for op, sid in fb.log if op == "add"]
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
