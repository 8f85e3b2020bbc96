"""Host logic of the serving loop (fullrmc_gb300/serve.py), on the CPU.

The engine set is replaced by a fake with the same methods that checks the
move-ring protocol (moves pushed contiguously, never over moves not yet
consumed, never stepped past what was pushed) and makes each fit's chi2 a
function of the moves it consumed, so that a fit's trace shows exactly which
moves it saw.  Failures are injected on the host: a footprint that raises (bad
shape), an engine creation that raises MemoryError (out of memory on
admission) and cancellations of queued and live fits.
"""
import types

import numpy as np
import pytest

from fullrmc_gb300 import serve


class FakeEngines:
    def __init__(self, move_cap=64):
        self.move_cap = move_cap
        self.next_id = 0
        self.eng = {}
        self.steps_calls = []

    def add(self, system):
        if getattr(system, "fail_add", False):
            raise MemoryError("out of device memory")
        e = self.next_id
        self.next_id += 1
        self.eng[e] = dict(n=system.box_coords.shape[0], ring={}, pushed=0, step=0, chi2=1.0, acc=0, results={})
        return e

    def remove(self, e):
        del self.eng[e]

    def push_moves(self, e, atoms, vecs, u, first):
        g = self.eng[e]
        assert first == g["pushed"], "moves must be pushed contiguously"
        assert first + len(atoms) <= g["step"] + self.move_cap, "push would overwrite unconsumed moves"
        assert np.all((atoms >= 0) & (atoms < g["n"]))
        for k in range(len(atoms)):
            g["ring"][(first + k) % self.move_cap] = (int(atoms[k]), tuple(map(float, vecs[k])), float(u[k]))
        g["pushed"] = first + len(atoms)

    def step(self, steps, engine=-1, graph=True, sync=True):
        assert engine == -1 and steps >= 1
        self.steps_calls.append((steps, len(self.eng)))
        for g in self.eng.values():
            for _ in range(steps):
                s = g["step"]
                assert s < g["pushed"], "stepped past the pushed moves"
                atom, v, u = g["ring"][s % self.move_cap]
                new = g["chi2"] * (1.0 + 0.01 * (v[0] - v[1])) + 1e-3 * atom / g["n"]
                accept = new < g["chi2"] or u < 0.1
                if accept:
                    g["chi2"] = new
                    g["acc"] += 1
                g["results"][s % self.move_cap] = (new, int(accept), atom)
                g["step"] = s + 1

    def state(self, e):
        g = self.eng[e]
        return g["chi2"], g["step"], g["acc"]

    def results(self, e, first, count):
        g = self.eng[e]
        r = [g["results"][(first + k) % self.move_cap] for k in range(count)]
        return (np.array([x[0] for x in r]), np.array([x[1] for x in r], np.int32), np.array([x[2] for x in r]))

    def counts(self, e):
        return np.zeros((1, 1, 4), np.int32), np.full((1, 1, 4), self.eng[e]["step"], np.int32)


def system(n, fail_add=False, bad=False):
    s = types.SimpleNamespace(box_coords=np.zeros((n, 3), np.float32), fail_add=fail_add, bad=bad)
    return s


def footprint(s):
    if s.bad:
        raise ValueError("box_coords must have shape (n, 3)")
    return 1000 + s.box_coords.shape[0]


def make_server(budget=10 ** 9, move_cap=64, **kw):
    return serve.Server(FakeEngines(move_cap), footprint, budget, record=True, keep_counts=True, **kw)


def run_alone(req, move_cap=64):
    s = make_server(move_cap=move_cap)
    s.submit(serve.FitRequest(req.rid, req.system, req.steps, req.seed, req.amplitude))
    s.drain()
    return s.results[req.rid]


def requests():
    return [serve.FitRequest(i, system(100 + 37 * i), steps, seed=1000 + i)
            for i, steps in enumerate([300, 45, 128, 1, 77, 500])]


def test_each_fit_runs_exactly_its_budget_and_matches_its_solo_run():
    reqs = requests()
    s = make_server()
    # staggered arrival: two now, the rest after some iterations
    s.submit(reqs[0])
    s.submit(reqs[1])
    s.iterate()
    s.iterate()
    for r in reqs[2:]:
        s.submit(r)
        s.iterate()
    s.drain()
    assert not s.live and not s.queue
    for r in reqs:
        got = s.results[r.rid]
        assert got.status == "done" and got.steps == r.steps
        assert len(got.trace[0]) == r.steps
        solo = run_alone(r)
        assert np.array_equal(got.trace[0], solo.trace[0])
        assert np.array_equal(got.trace[1], solo.trace[1])
        assert got.chi2 == solo.chi2 and got.accepted == solo.accepted == int(got.trace[1].sum())
    assert s.steps_done == sum(r.steps for r in reqs)
    # k never exceeds half the ring, so refills always stay ahead of the steps
    assert max(k for k, _ in s.es.steps_calls) <= 32


def test_admission_by_footprint_keeps_order_and_budget():
    reqs = [serve.FitRequest(i, system(500), 40, seed=i) for i in range(5)]
    budget = 2 * (1000 + 500) + 10  # two fits at a time
    s = make_server(budget=budget)
    for r in reqs:
        s.submit(r)
    s.iterate()
    assert sorted(s.live) == [0, 1] and [q.rid for q in s.queue] == [2, 3, 4]
    s.drain()
    assert s.peak_used <= budget and s.peak_live == 2
    assert all(s.results[r.rid].status == "done" for r in reqs)
    # admitted in arrival order
    order = sorted(reqs, key=lambda r: s.results[r.rid].admitted_at)
    assert [r.rid for r in order] == [0, 1, 2, 3, 4]


def test_oversized_request_fails_without_blocking_the_queue():
    s = make_server(budget=5000)
    s.submit(serve.FitRequest(0, system(10 ** 6), 10, seed=0))
    s.submit(serve.FitRequest(1, system(100), 10, seed=1))
    s.drain()
    assert s.results[0].status == "failed" and "exceeds the HBM budget" in s.results[0].error
    assert s.results[1].status == "done" and s.results[1].steps == 10


def test_failures_are_isolated():
    good = [serve.FitRequest(i, system(200 + i), 90, seed=7 + i) for i in range(3)]
    bad_shape = serve.FitRequest(10, system(50, bad=True), 90, seed=1)
    oom = serve.FitRequest(11, system(50, fail_add=True), 90, seed=2)
    zero = serve.FitRequest(12, system(50), 0, seed=3)
    s = make_server()
    for r in [good[0], bad_shape, good[1], oom, zero, good[2]]:
        s.submit(r)
    s.drain()
    assert s.results[10].status == "failed" and "ValueError" in s.results[10].error
    assert s.results[11].status == "failed" and "MemoryError" in s.results[11].error
    assert s.results[12].status == "failed"
    for r in good:
        got = s.results[r.rid]
        assert got.status == "done"
        assert np.array_equal(got.trace[0], run_alone(r).trace[0])
    assert s.used == 0 and not s.es.eng  # every engine was removed


def test_cancellation_of_queued_and_live_fits():
    reqs = [serve.FitRequest(i, system(300), 400, seed=i) for i in range(4)]
    s = make_server(budget=2 * 1300 + 1)
    for r in reqs:
        s.submit(r)
    s.iterate()                      # 0 and 1 live, 2 and 3 queued
    s.cancel(1)                      # live
    s.cancel(3)                      # queued
    s.drain()
    assert s.results[1].status == "cancelled" and 0 < s.results[1].steps < 400
    assert s.results[3].status == "cancelled" and s.results[3].steps == 0
    for rid in (0, 2):
        got = s.results[rid]
        assert got.status == "done" and got.steps == 400
        assert np.array_equal(got.trace[0], run_alone(reqs[rid]).trace[0])
    # the cancelled live fit's partial trace is a prefix of its solo run
    part = s.results[1]
    assert np.array_equal(part.trace[0], run_alone(reqs[1]).trace[0][:part.steps])


def test_weighted_percentile():
    v = [1.0, 2.0, 3.0]
    w = [1, 1, 98]
    assert serve.weighted_percentile(v, w, 50) == 3.0
    assert serve.weighted_percentile(v, w, 1) == 1.0
    assert serve.weighted_percentile(v, [1, 1, 1], 50) == 2.0
    assert serve.weighted_percentile([], [], 50) is None


def test_poisson_arrivals_rate():
    t = serve.poisson_arrivals(np.random.default_rng(0), 20.0, 500.0)
    assert abs(len(t) / 500.0 - 20.0) < 1.0
    assert all(a < b for a, b in zip(t, t[1:]))


def test_run_stream_with_a_fake_clock():
    now = [0.0]

    def clock():
        return now[0]

    def sleep(dt):
        now[0] += max(dt, 1e-4)

    fe = FakeEngines(64)
    orig = fe.step

    def timed_step(*a, **k):
        now[0] += 0.002  # every iteration takes 2 ms
        return orig(*a, **k)

    fe.step = timed_step
    s = serve.Server(fe, footprint, 10 ** 9, clock=clock, max_k=8)
    arr = serve.poisson_arrivals(np.random.default_rng(1), 20.0, 2.0)
    reqs = [serve.FitRequest(i, system(100), 50 + 10 * i, seed=i, arrival=a) for i, a in enumerate(arr)]
    elapsed = serve.run_stream(s, reqs, wall_limit=60.0, clock=clock, sleep=sleep)
    assert all(s.results[r.rid].status == "done" for r in reqs)
    assert elapsed < 60.0
    p50, p99 = s.step_latency(50), s.step_latency(99)
    assert p50 == pytest.approx(0.002 / 8) and p99 >= p50
    assert s.fit_latency(50) > 0


def test_close_cancels_queued_and_live_fits():
    s = make_server(budget=1300 + 1)
    reqs = [serve.FitRequest(i, system(300), 100, seed=i) for i in range(3)]
    for r in reqs:
        s.submit(r)
    s.iterate()
    s.close()
    assert [s.results[i].status for i in range(3)] == ["cancelled"] * 3
    assert 0 < s.results[0].steps < 100 and s.used == 0 and not s.es.eng
