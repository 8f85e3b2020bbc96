"""Serving loop: continuous batching of RMC fits resident on one GPU.

A request is one RMC fit: a system (``engine.EngineSystem``: coordinates,
box, elements, experimental curve(s)), a step budget and the seed of its
translation-move stream.  The server keeps every admitted fit's whole state on
the device (one engine of an ``engine.EngineSet``) and advances all live fits
together: an iteration is k batched Metropolis steps of every live fit, with
k no larger than the smallest remaining budget, so each fit stops exactly at
its budget.  Between iterations it

* retires fits that finished or were cancelled and hands back their results
  (chi2, accepted count, optionally the final histograms),
* admits waiting requests in arrival order while their device footprint fits
  the HBM budget and a slot is free (admission by footprint; a request larger
  than the whole budget fails at once instead of blocking the queue),
* isolates failures: a request whose footprint or engine creation raises
  fails alone, and the live fits carry on.

A fit's chain depends only on its own data and move stream, and the engines'
arithmetic is the same solo and batched, so a fit gives the same accept
sequence and chi2 alone as in any mix.

Per-step latency: an iteration of k steps that took t seconds gives every live
fit k steps of latency t / k each; percentiles are taken over fit-steps.  Fit
latency is the time from arrival to retirement.
"""
from __future__ import annotations

import collections
import dataclasses
import time
from typing import Callable

import numpy as np

from .engine import translation_moves


@dataclasses.dataclass
class FitRequest:
    """One RMC fit: `system` (engine.EngineSystem), `steps` to run, the seed of
    its translation-move stream and the move amplitude in A; `arrival` is the
    submission time in seconds from the start of the stream."""
    rid: int
    system: object
    steps: int
    seed: int
    amplitude: float = 0.1
    arrival: float = 0.0


@dataclasses.dataclass
class FitResult:
    rid: int
    status: str                    # "done", "failed" or "cancelled"
    steps: int = 0
    accepted: int = 0
    chi2: float = float("nan")
    counts: tuple | None = None    # (intra, inter) int32 histograms when requested
    trace: tuple | None = None     # (chi2_new, accepted) of every step when recorded
    error: str = ""
    arrival: float = 0.0
    admitted_at: float = float("nan")
    finished_at: float = float("nan")


class _Live:
    __slots__ = ("req", "eid", "need", "done", "pushed", "moves", "admitted_at", "trace")

    def __init__(self, req, eid, need, admitted_at):
        self.req = req
        self.eid = eid
        self.need = need
        self.done = 0
        self.pushed = 0
        self.moves = None
        self.admitted_at = admitted_at
        self.trace = []


def weighted_percentile(values, weights, pct):
    """Percentile `pct` (0-100) of samples `values` with integer `weights`
    (the lower of the two neighbouring samples, like numpy's 'inverted_cdf')."""
    v = np.asarray(values, np.float64)
    w = np.asarray(weights, np.float64)
    if v.size == 0:
        return None
    o = np.argsort(v, kind="stable")
    c = np.cumsum(w[o])
    k = int(np.searchsorted(c, pct / 100.0 * c[-1], side="left"))
    return float(v[o][min(k, v.size - 1)])


class Server:
    """Continuous-batching server over an engine set.

    `engines` is an engine.EngineSet (or an object with the same add / remove
    / push_moves / step / state / counts / results methods and `move_cap`);
    `footprint(system)` gives a fit's device bytes; `hbm_budget` bounds the sum
    of the live fits' footprints."""

    def __init__(self, engines, footprint: Callable, hbm_budget: int, max_live: int = 1024, max_k: int = 32,
                 keep_counts: bool = False, record: bool = False, graph: bool = True, clock=time.perf_counter):
        self.es = engines
        self.footprint = footprint
        self.hbm_budget = int(hbm_budget)
        self.max_live = int(max_live)
        self.ring = int(engines.move_cap)
        self.max_k = max(1, min(int(max_k), self.ring // 2))
        self.keep_counts = keep_counts
        self.record = record
        self.graph = graph
        self.clock = clock
        self.queue = collections.deque()
        self.live = {}             # rid -> _Live, in admission order
        self.used = 0              # bytes of the live fits
        self.results = {}          # rid -> FitResult
        self._cancel = set()
        self.lat_values = []       # per-iteration step latency t / k (seconds)
        self.lat_weights = []      # fit-steps it covers (live fits * k)
        self.steps_done = 0
        self.iterations = 0
        self.busy_time = 0.0
        self.peak_live = 0
        self.peak_used = 0

    # ------------------------------------------------------------ requests
    def submit(self, req: FitRequest):
        self.queue.append(req)

    def cancel(self, rid: int):
        """Cancel a queued or live fit; it is retired before the next iteration."""
        self._cancel.add(rid)

    # ------------------------------------------------------------ internals
    def _fail(self, req, error):
        self.results[req.rid] = FitResult(req.rid, "failed", error=error, arrival=req.arrival)

    def _refill(self, lv):
        """Top the fit's move ring up to a full ring ahead of its step."""
        ahead = lv.pushed - lv.done
        if lv.pushed >= lv.req.steps or ahead > self.ring // 2:
            return
        count = min(self.ring - ahead, lv.req.steps - lv.pushed)
        a, v, u = lv.moves
        s = slice(lv.pushed, lv.pushed + count)
        self.es.push_moves(lv.eid, a[s], v[s], u[s], lv.pushed)
        lv.pushed += count

    def _admit(self, now):
        while self.queue and len(self.live) < self.max_live:
            req = self.queue[0]
            if req.rid in self._cancel:
                self.queue.popleft()
                self._cancel.discard(req.rid)
                self.results[req.rid] = FitResult(req.rid, "cancelled", arrival=req.arrival)
                continue
            try:
                need = int(self.footprint(req.system))
                if req.steps < 1:
                    raise ValueError("a fit needs at least one step")
            except Exception as exc:  # a malformed request fails alone
                self.queue.popleft()
                self._fail(req, "%s: %s" % (type(exc).__name__, exc))
                continue
            if need > self.hbm_budget:
                self.queue.popleft()
                self._fail(req, "footprint of %d bytes exceeds the HBM budget of %d" % (need, self.hbm_budget))
                continue
            if self.used + need > self.hbm_budget:
                break  # wait for live fits to finish; arrival order is kept
            self.queue.popleft()
            try:
                eid = self.es.add(req.system)
            except Exception as exc:  # e.g. the device ran out of memory
                self._fail(req, "%s: %s" % (type(exc).__name__, exc))
                continue
            lv = _Live(req, eid, need, now)
            self.live[req.rid] = lv
            self.used += need
            try:
                n = req.system.box_coords.shape[0]
                lv.moves = translation_moves(np.random.default_rng(req.seed), n, req.steps, req.amplitude)
                self._refill(lv)
            except Exception as exc:
                self._retire(req.rid, "failed", now, "%s: %s" % (type(exc).__name__, exc))
        self.peak_live = max(self.peak_live, len(self.live))
        self.peak_used = max(self.peak_used, self.used)

    def _retire(self, rid, status, now, error=""):
        lv = self.live.pop(rid)
        res = FitResult(rid, status, steps=lv.done, error=error, arrival=lv.req.arrival, admitted_at=lv.admitted_at,
                        finished_at=now)
        try:
            if status != "failed":
                res.chi2, _step, res.accepted = self.es.state(lv.eid)
                if self.keep_counts:
                    res.counts = self.es.counts(lv.eid)
                if self.record:
                    res.trace = (np.concatenate([t[0] for t in lv.trace]) if lv.trace else np.empty(0),
                                 np.concatenate([t[1] for t in lv.trace]) if lv.trace else np.empty(0, np.int32))
        finally:
            self.es.remove(lv.eid)
            self.used -= lv.need
        self.results[rid] = res

    # ------------------------------------------------------------ iteration
    def iterate(self):
        """Retire cancelled fits, admit, step every live fit k times, retire
        the finished ones.  Returns the number of fit-steps done."""
        now = self.clock()
        for rid in [r for r in self.live if r in self._cancel]:
            self._cancel.discard(rid)
            self._retire(rid, "cancelled", now)
        self._admit(now)
        if not self.live:
            return 0
        lives = list(self.live.values())
        k = min(self.max_k, min(lv.req.steps - lv.done for lv in lives), min(lv.pushed - lv.done for lv in lives))
        t0 = self.clock()
        self.es.step(k, engine=-1, graph=self.graph and k == self.max_k, sync=True)
        t1 = self.clock()
        self.busy_time += t1 - t0
        nlive = len(lives)
        self.lat_values.append((t1 - t0) / k)
        self.lat_weights.append(nlive * k)
        self.steps_done += nlive * k
        self.iterations += 1
        for lv in lives:
            if self.record:
                c2, acc, _atoms = self.es.results(lv.eid, lv.done, k)
                lv.trace.append((c2, acc))
            lv.done += k
            if lv.done >= lv.req.steps:
                self._retire(lv.req.rid, "done", t1)
            else:
                self._refill(lv)
        return nlive * k

    def drain(self, max_iterations=None):
        """Iterate until no fit is live or queued (or `max_iterations`)."""
        it = 0
        while (self.live or self.queue) and (max_iterations is None or it < max_iterations):
            if self.iterate() == 0 and not self.live and self.queue:
                break  # the head of the queue can never be admitted
            it += 1

    def close(self):
        """Cancel every queued and live fit (live ones keep their partial results)."""
        now = self.clock()
        while self.queue:
            req = self.queue.popleft()
            self.results[req.rid] = FitResult(req.rid, "cancelled", arrival=req.arrival)
        for rid in list(self.live):
            self._retire(rid, "cancelled", now)

    # ------------------------------------------------------------ reporting
    def step_latency(self, pct):
        return weighted_percentile(self.lat_values, self.lat_weights, pct)

    def fit_latency(self, pct):
        t = [r.finished_at - r.arrival for r in self.results.values() if r.status == "done"]
        return float(np.percentile(t, pct)) if t else None


def poisson_arrivals(rng: np.random.Generator, rate: float, duration: float):
    """Arrival times (seconds) of a Poisson process of `rate` per second over
    `duration` seconds."""
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        out.append(t)


def run_stream(server: Server, requests, wall_limit: float, clock=time.perf_counter, sleep=time.sleep):
    """Submit `requests` (their `arrival` in seconds from now) to `server` in
    real time and iterate until every request is finished or `wall_limit`
    seconds have passed.  Arrival times are rebased onto `server.clock`.
    Returns the elapsed wall time."""
    start = clock()
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    while True:
        now = clock() - start
        while pending and pending[0].arrival <= now:
            req = pending.popleft()
            req.arrival = start + req.arrival
            server.submit(req)
        if now >= wall_limit or (not pending and not server.live and not server.queue):
            break
        if server.live or server.queue:
            before = len(server.live) + len(server.queue)
            server.iterate()
            if not server.live and len(server.queue) == before and pending:
                sleep(min(0.001, max(0.0, pending[0].arrival - now)))
        else:
            sleep(min(0.001, max(0.0, pending[0].arrival - now)))
    return clock() - start


def benchmark_stream(seconds, wall_limit, seed=0, rate=20.0, budget_gib=16, plain_fits=6, plain_steps=100):
    """The serving loop on a Poisson stream of fit requests: `rate` requests
    per second for `seconds` (sizes log-uniform in 2,000-200,000 atoms, 1-3
    species, G(r) on r 0-12 A plus S(Q) on Q 0.5-25 A^-1 with dQ 0.01, 2,000-
    50,000 steps each), run in real time until every fit is done or
    `wall_limit` seconds pass.  Reports total fit-steps/s, p50/p99 per-step
    latency, fit latency, and the same kind of fits stepped one at a time (the
    plain path) for comparison.  Needs the GPU library."""
    from . import synthetic
    from .engine import EngineSet, footprint
    cap = 4096
    arr = poisson_arrivals(np.random.default_rng([seed, 99]), rate, seconds)
    reqs = []
    for i, t in enumerate(arr):
        system, steps = synthetic.serving_fit(seed * 100000 + i)
        reqs.append(FitRequest(i, system, steps, seed=seed * 100000 + i, arrival=t))
    # fits average 44,000 atoms (up to 200,000): 512-thread CTAs, one per SM
    # (two 256-thread CTAs per SM pay off for the smaller engines of the
    # batching workload)
    es = EngineSet([], move_cap=cap, tune=(1024, 512, 1))
    srv = Server(es, lambda s: footprint(s, cap), budget_gib << 30, max_k=32)
    # warm the kernels and the shared S(Q) table outside the timed stream
    warm = Server(es, lambda s: footprint(s, cap), budget_gib << 30, max_k=32)
    w_sys, _ = synthetic.serving_fit(seed * 100000 + 99999, nmax=3000)
    warm.submit(FitRequest(-1, w_sys, 64, seed=1))
    warm.drain()
    elapsed = run_stream(srv, reqs, wall_limit)
    done = [r for r in srv.results.values() if r.status == "done"]
    failed = [r for r in srv.results.values() if r.status == "failed"]
    atoms = [r.system.box_coords.shape[0] for r in reqs]
    out = {
        "steps_per_s": srv.steps_done / elapsed,
        "fit_steps": srv.steps_done,
        "elapsed_s": elapsed,
        "busy_s": srv.busy_time,
        "p50_step_latency_ms": 1e3 * srv.step_latency(50) if srv.lat_values else None,
        "p99_step_latency_ms": 1e3 * srv.step_latency(99) if srv.lat_values else None,
        "p50_fit_latency_s": srv.fit_latency(50),
        "p99_fit_latency_s": srv.fit_latency(99),
        "requests": len(reqs), "fits_done": len(done), "fits_failed": len(failed),
        "fits_unfinished": sum(1 for r in reqs if r.rid not in srv.results),
        "peak_live": srv.peak_live, "peak_device_bytes": srv.peak_used, "hbm_budget_bytes": budget_gib << 30,
        "iterations": srv.iterations,
        "stream": {"rate_per_s": rate, "arrivals_s": seconds, "wall_limit_s": wall_limit,
                   "atoms": "log-uniform 2000-200000 (mean of this stream %.0f)" % (np.mean(atoms) if atoms else 0),
                   "species": "1-3", "G(r)": "r 0-12 A, dr 0.01", "S(Q)": "Q 0.5-25, dQ 0.01 (2451 points)",
                   "steps_per_fit": "uniform 2000-50000"},
    }
    srv.close()
    # plain: a sample of the stream's fits stepped one at a time
    sample = reqs[:plain_fits]
    ids = []
    for r in sample:
        e = es.add(r.system)
        a, v, u = translation_moves(np.random.default_rng(r.seed), r.system.box_coords.shape[0], plain_steps + 1,
                                    r.amplitude)
        es.push_moves(e, a, v, u, 0)
        ids.append(e)
    for e in ids:
        es.step(1, engine=e, graph=False)
    t0 = time.perf_counter()
    for e in ids:
        es.step(plain_steps, engine=e, graph=False, sync=False)
    es.sync()
    t_plain = time.perf_counter() - t0
    out["plain"] = {"steps_per_s": len(ids) * plain_steps / t_plain, "fits_sampled": len(ids),
                    "atoms": [r.system.box_coords.shape[0] for r in sample]}
    out["served_over_plain"] = out["steps_per_s"] / out["plain"]["steps_per_s"]
    es.close()
    return out
