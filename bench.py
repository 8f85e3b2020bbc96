"""Benchmark: RMC steps/s of 256 mixed-size engines on one GB300.

Workload (seeded synthetic data, shapes of the batching configuration):
256 independent engines, atom counts log-uniform in [1,000, 20,000], 1-4
species, cubic or triclinic boxes at 0.08-0.10 atoms/A^3, a seeded synthetic
G(r) per engine (r 0-12 A, dr 0.01 A), single-atom translation moves of up
to 0.1 A.  One step = one Metropolis step of every engine, executed as one
launch of the batched step kernel.

Reported beside the headline:
* ``plain``: the same engines stepped one at a time on the GPU (the plain
  path) -- steps/s and the batched/plain ratio;
* ``e2e``: the batched step driven through the public API with host
  buffers: each step uploads its moves from pinned host memory and reads
  every engine's chi2 and decision back;
* ``allpairs``: the all-pairs histogram of 100,000 atoms (three species,
  triclinic a = b = c = 103 A, gamma = 120, r 0-20 A): time, pair
  distances/s and its fraction of the SM issue roofline;
* ``roofline``: the batched step kernel against the issue roofline
  (46 algorithmic operations per pair distance, SMs x clock x 128 / 46);
* ``cpu_baseline``: fullrmc's own Cython path (compiled from its sources)
  running the same kind of steps on the host cores, on a bounded sample;
* ``configs``: single-engine step rates of the other configurations (the
  5,000-atom alloy; the 100,000-atom triclinic system and its FP64 S(Q)
  transform; the 52,000-atom molecular system with 13-atom group moves),
  beside fullrmc's Cython path on a few steps of the same systems;
* ``dropins``: per-call times of the atomic_distances and
  atomic_coordination drop-ins (the constraints' per-move call on a moved
  13-atom ring and their full recomputations, 52,000-atom molecular system)
  and of the ShapeFunction (100,000-atom finite cluster, every pair binned)
  beside fullrmc's Cython on the same calls;
* ``serving``: the serving loop on a Poisson stream of fit requests (20 per
  second; 2,000-200,000 atoms log-uniform, 1-3 species, G(r) on r 0-12 A
  plus S(Q) on Q 0.5-25 A^-1 with dQ 0.01, 2,000-50,000 steps each), admitted
  by device footprint and batched across the live fits: total fit-steps/s,
  p50/p99 per-step latency, fit latency, and the same fits stepped one at a
  time (plain) for comparison.

Timing: CUDA events on the stepping stream, W untimed warm-up steps, then K
timed steps each bracketed by its own events, with a write of a buffer larger
than L2 between steps (outside the events).  ``--impl reference`` times the
reference CPU path alone.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RMC steps/s (batched/served vs plain GPU, same accepts)"
UNIT = "steps/s"
WORKLOAD = "batched_256_mixed_engines"
OPS_PER_PAIR = 46


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    except Exception:
        return {"sm_max_mhz": 2070.0, "hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _host_cpu():
    """The host CPU as /proc/cpuinfo names it (x86 "model name"; Arm
    implementer/part codes), with the logical core count."""
    name = None
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read()
        for key in ("model name", "Model", "CPU part"):
            for line in info.splitlines():
                if line.split(":")[0].strip() == key:
                    name = "%s %s" % ("CPU part" if key == "CPU part" else "", line.split(":", 1)[1].strip())
                    break
            if name:
                break
    except OSError:
        pass
    import platform
    return "%s (%s), %d logical cores" % ((name or "unknown").strip(), platform.machine(), os.cpu_count() or 1)


def workload_config(ws, engines=256, amp=0.1, seed=0):
    """The `config` object of both arms: the batching workload as generated
    (the same dict whichever arm prints it)."""
    from fullrmc_gb300 import synthetic
    systems = synthetic.mixed_engines(seed=seed, count=engines)
    return {"workload": WORKLOAD, "engines": engines, "engines_total": ws * engines,
            "atoms_total": int(sum(s.box_coords.shape[0] for s in systems)),
            "atoms": "log-uniform 1000-20000", "species": "1-4", "rmax": 12.0, "dr": 0.01,
            "move": "single-atom translation <= %.1f A" % amp,
            "l2": "256 MiB buffer written between timed steps",
            "parallelism": "engines sharded per GPU" if ws > 1 else "single GPU"}


def stratified(systems, count):
    """`count` engine indexes spread evenly over the engines sorted by atom
    count (the sample's size distribution follows the population's)."""
    order = np.argsort([s.box_coords.shape[0] for s in systems], kind="stable")
    if count >= len(order):
        return sorted(int(e) for e in order)
    pick = np.floor((np.arange(count) + 0.5) * len(order) / count).astype(int)
    return sorted(int(order[k]) for k in pick)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


# ------------------------------------------------------------- reference arm
def _ref_worker(args):
    """Reference Cython host chains for engines `idxs`: one "step" moves every
    engine of this worker once; returns the duration of each step."""
    idxs, steps, seed, amp = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import translation_moves
    from fullrmc_gb300.hostloop import HostPDFChain
    R = build_ref.import_reference()
    systems = synthetic.mixed_engines(seed=seed, count=max(idxs) + 1)
    chains, mv = [], []
    for e in idxs:
        s = systems[e]
        chain = HostPDFChain(s, R["pairs_histograms"], R["boundary_conditions_collection"])
        chain.compute_data()
        chains.append(chain)
        mv.append(translation_moves(np.random.default_rng([seed, 1000 + e]), s.box_coords.shape[0], steps, amp))
    times = []
    for k in range(steps):
        t0 = time.perf_counter()
        for chain, (a, v, u) in zip(chains, mv):
            chain.step(a[k], v[k][None, :], u[k])
        times.append(time.perf_counter() - t0)
    return len(idxs), times


def reference_rate(engines, steps, warmup, processes, seed=0, amp=0.1):
    """Aggregate steps/s of the reference CPU path over the engine indexes
    `engines`: `processes` host processes each step their own engines (the
    engines are independent; engines are dealt largest first to the least
    loaded process); a timed step lasts as long as the slowest process."""
    import multiprocessing as mp
    from fullrmc_gb300 import synthetic
    sizes = [s.box_coords.shape[0] for s in synthetic.mixed_engines(seed=seed, count=max(engines) + 1)]
    chunks = [[] for _ in range(max(1, min(processes, len(engines))))]
    load = [0] * len(chunks)
    for e in sorted(engines, key=lambda e: -sizes[e]):
        k = load.index(min(load))
        chunks[k].append(e)
        load[k] += sizes[e]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(chunks)) as pool:
        out = pool.map(_ref_worker, [(c, warmup + steps, seed, amp) for c in chunks])
    total = sum(max(o[1][k] for o in out) for k in range(warmup, warmup + steps))
    done = len(engines) * steps
    return done / total, len(chunks)


def _engine_rate(torch, system, steps, seed, group=False):
    """Steps/s of one engine stepped alone (the plain GPU path, one CUDA
    graph of `steps` steps), and the engine's initial counts."""
    from fullrmc_gb300.engine import EngineSet, group_moves, translation_moves
    es = EngineSet([system], move_cap=steps + 16)
    es.init()
    rng = np.random.default_rng(seed)
    if group:
        mv = group_moves(rng, system.groups, steps + 16, 0.1, 10.0)
        es.push_group_moves(0, *mv, 0)
    else:
        mv = translation_moves(rng, system.box_coords.shape[0], steps + 16, 0.1)
        es.push_moves(0, *mv, 0)
    counts0 = es.counts(0)
    es.step(8, engine=0, graph=False)
    es.step(steps, engine=0, graph=True, sync=True)  # capture
    es.step(8, engine=0, graph=False)
    # time `steps` further steps (moves: the ring holds steps + 16; re-push)
    if group:
        es.push_group_moves(0, *[x[:steps] for x in group_moves(np.random.default_rng(seed + 1), system.groups,
                                                                  steps, 0.1, 10.0)], es.state(0)[1])
    else:
        es.push_moves(0, *[x[:steps] for x in translation_moves(np.random.default_rng(seed + 1),
                                                                system.box_coords.shape[0], steps, 0.1)],
                      es.state(0)[1])
    t0 = time.perf_counter()
    es.step(steps, engine=0, graph=True, sync=True)
    dt = time.perf_counter() - t0
    st = es.state(0)
    es.close()
    return steps / dt, counts0, st[2] / max(1, st[1]), mv


def _reference_config_rate(system, counts0, mv, steps, group=False):
    """Steps/s of fullrmc's Cython path (reference-style host loop, ncores=1)
    on the same system, started from the same initial counts."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    from fullrmc_gb300.engine import group_new_real
    from fullrmc_gb300.hostloop import HostPDFChain
    R = build_ref.import_reference()
    chain = HostPDFChain(system, R["pairs_histograms"], R["boundary_conditions_collection"])
    chain.data = (counts0[0].astype(np.float32), counts0[1].astype(np.float32))
    chain.error = chain.standard_error(*chain.data)
    t0 = time.perf_counter()
    for k in range(steps):
        if group:
            atoms, kinds, params, u = mv
            chain.step(atoms[k], None, u[k], moved_real=group_new_real(chain.real[atoms[k]], kinds[k], params[k]))
        else:
            a, v, u = mv
            chain.step(a[k], v[k][None, :], u[k])
    return steps / (time.perf_counter() - t0)


def _dropin_loop_rate(system, steps):
    """Steps/s of the plain drop-in: fullrmc's step with a
    PairDistributionConstraint (hostloop.HostPDFChain: M and F histograms
    before and after the move, the moved box coordinates through
    transform_coordinates, float32 G(r) and standard error on the host) with
    the GPU modules in place of the Cython ones, host arrays in and out."""
    import fullrmc_gb300
    from fullrmc_gb300.engine import translation_moves
    from fullrmc_gb300.hostloop import HostPDFChain
    chain = HostPDFChain(system, fullrmc_gb300.pairs_histograms, fullrmc_gb300.boundary_conditions_collection)
    chain.compute_data()
    a, v, u = translation_moves(np.random.default_rng(17), system.box_coords.shape[0], steps + 50, 0.1)
    for k in range(50):
        chain.step(a[k], v[k][None, :], u[k])
    t0 = time.perf_counter()
    for k in range(50, 50 + steps):
        chain.step(a[k], v[k][None, :], u[k])
    dt = time.perf_counter() - t0
    return {"plain_dropin_steps_per_s": steps / dt, "plain_dropin_steps": steps,
            "plain_dropin_path": "fullrmc's PDF step on the drop-in modules: 4 histogram calls and 1 coordinate "
                                 "transform per step, host arrays, float32 G(r) on the host"}


def bench_configs(torch, with_cpu):
    """Single-engine step rates of the other configurations on the GPU (and,
    on a bounded sample, of the reference CPU path): the 5,000-atom alloy,
    the 100,000-atom triclinic system (plus its FP64 S(Q) transform, Q 0.5-30
    / 0.01), and the 52,000-atom molecular system with 13-atom group moves."""
    from fullrmc_gb300 import reciprocal_space, synthetic
    out = {}
    for name, system, steps, group, cpu_steps in (
            ("alloy_5000", synthetic.alloy_5000(seed=0), 2000, False, 40),
            ("triclinic_100k", synthetic.triclinic_100k(seed=0), 1000, False, 8),
            ("ring_molecules_52000", synthetic.ring_molecules(seed=0, nmol=4000), 400, True, 4)):
        rate, counts0, acc, mv = _engine_rate(torch, system, steps, seed=5, group=group)
        d = {"atoms": int(system.box_coords.shape[0]), "atoms_per_move": 13 if group else 1,
             "gpu_steps_per_s": rate, "steps": steps, "accept_rate": round(float(acc), 4)}
        if name == "alloy_5000":
            d.update(_dropin_loop_rate(system, 2000))
        if with_cpu:
            try:
                d["cpu_reference_steps_per_s"] = _reference_config_rate(system, counts0, mv, cpu_steps, group)
                d["cpu_sample_steps"] = cpu_steps
            except Exception as exc:
                d["cpu_reference_steps_per_s"] = None
                d["cpu_error"] = str(exc)[:200]
        out[name] = d
    # the 100k system's S(Q): FP64 sine transform of its G(r), Q 0.5-30 / 0.01 (2951 points)
    s = synthetic.triclinic_100k(seed=0)
    q = (0.5 + 0.01 * np.arange(2951)).astype(np.float32)
    G = np.asarray(s.model.G_exp, np.float32)
    reciprocal_space.Gr_to_sq(s.model.r, G, q)
    t0 = time.perf_counter()
    for _ in range(5):
        reciprocal_space.Gr_to_sq(s.model.r, G, q)
    t = (time.perf_counter() - t0) / 5
    terms = float(q.size) * float(np.asarray(s.model.r).size)
    d = out["triclinic_100k"]
    d["sq_transform_ms"] = 1e3 * t
    d["sq_transform_terms"] = int(terms)
    # per term w * sin(q r) accumulated: the product q r and one FMA (3 FP64
    # flops, the sine's own arithmetic not counted); host copies included
    d["sq_transform_fp64_gflops"] = 3.0 * terms / t * 1e-9
    return out


def _call_ms(fn, reps, budget_s=None):
    """Median wall-clock milliseconds of fn() over reps calls (host buffers,
    copies and synchronisation included), after one untimed call."""
    fn()
    times = []
    t_start = time.perf_counter()
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        times.append(1e3 * (time.perf_counter() - t0))
        if budget_s is not None and time.perf_counter() - t_start > budget_s:
            break
    return statistics.median(times), len(times)


def bench_dropins(with_cpu):
    """Per-call times of the pairs_histograms, atomic_distances,
    atomic_coordination and shape-function paths through their Python API
    (host arrays in and out), beside fullrmc's Cython (ncores=1) on the same
    call: the constraints' per-move call (one atom of the 5,000-atom alloy,
    or the 13 atoms of a moved ring) and the full recomputation, on the
    52,000-atom molecular system (three species, 13-atom rings)."""
    from fullrmc_gb300 import atomic_coordination as gac
    from fullrmc_gb300 import atomic_distances as gad
    from fullrmc_gb300 import pairs_histograms as gph
    from fullrmc_gb300 import synthetic
    s = synthetic.ring_molecules(seed=0, nmol=4000)
    c, B, el, mol = s.box_coords, s.basis, s.el.astype(np.int32), s.mol.astype(np.int32)
    n, ne = c.shape[0], 3
    lo = np.full((ne, ne, 1), 1.8, np.float32)
    up = np.full((ne, ne, 1), 2.6, np.float32)
    group = np.arange(13 * 1234, 13 * 1235, dtype=np.int32)
    sub = 20000  # the full recomputation of atomic_distances on the first 20,000 atoms
    # coordination definitions: (core species, shell species, window)
    defs = [(0, 1, 1.0, 1.6), (1, 0, 1.0, 1.6), (0, 2, 0.9, 1.3), (0, 0, 1.2, 1.6)]
    cores = [np.flatnonzero(el == a).astype(np.int32) for a, _, _, _ in defs]
    shells = [np.flatnonzero(el == b).astype(np.int32) for _, b, _, _ in defs]
    lower = [np.float32(x) for _, _, x, _ in defs]
    upper = [np.float32(x) for _, _, _, x in defs]
    asCore = [[] for _ in range(n)]
    inShell = [[] for _ in range(n)]
    for d in range(len(defs)):
        for a in cores[d]:
            asCore[a].append(d)
        for a in shells[d]:
            inShell[a].append(d)
    asCore = [np.array(x, np.int32) for x in asCore]
    inShell = [np.array(x, np.int32) for x in inShell]
    L = (cores, shells, lower, upper, asCore, inShell)
    data = np.zeros(len(defs), np.float32)

    s5 = synthetic.alloy_5000(seed=0)
    m5 = s5.model
    h5 = dict(boxCoords=s5.box_coords, basis=s5.basis, isPBC=True, moleculeIndex=s5.mol.astype(np.int32),
              elementIndex=s5.el.astype(np.int32), numberOfElements=len(m5.elements_count),
              minDistance=np.float32(m5.minDistance), maxDistance=np.float32(m5.maxDistance),
              bin=np.float32(m5.bin), histSize=int(m5.hs))
    hg = dict(boxCoords=c, basis=B, isPBC=True, moleculeIndex=mol, elementIndex=el, numberOfElements=ne,
              minDistance=np.float32(-0.005), maxDistance=np.float32(15.005), bin=np.float32(0.01), histSize=1501)
    one = np.array([1234], np.int32)

    def cases(ad, ac, ph):
        return {
            # the PDF constraint's per-move histogram (fullrmc calls it for the
            # moved atoms before and after each move): one atom of the 5,000-atom
            # alloy, and a 13-atom ring of the 52,000-atom molecular system
            "pairs_histograms_move_5000": (lambda: ph.multiple_pairs_histograms_coords(one, **h5), 50),
            "pairs_histograms_group_52000": (lambda: ph.multiple_pairs_histograms_coords(group, **hg), 50),
            "intermolecular_distances_move": (lambda: ad.multiple_atomic_distances_coords(
                group, c, B, True, mol, el, ne, lo, up, intraMolecular=False, countWithinLimits=True), 50),
            "intermolecular_distances_full_20000": (lambda: ad.full_atomic_distances_coords(
                c[:sub], B, True, mol[:sub], el[:sub], ne, lo, up, intraMolecular=False), 5),
            "coordination_move": (lambda: ac.multi_atoms_coord_number_coords(group, c, B, True, *L, data), 50),
            "coordination_all_atoms": (lambda: ac.all_atoms_coord_number_coords(c, B, True, *L, data), 5),
        }

    out = {}
    # ShapeFunction of a 100,000-atom finite cluster (infinite boundary
    # conditions): every pair binned (r 0-110 A, dr 1), S(q) on q 0.001-1
    # (dq 0.005) and the shape function on r 0.005-20 (0.01)
    from fullrmc_gb300 import shape_function as gsf
    rng = np.random.default_rng(77)
    pts = rng.normal(size=(300000, 3))
    pts = pts[np.linalg.norm(pts, axis=1) < 2.0][:100000]
    cl = (pts * 25.0).astype(np.float32)
    cel = rng.integers(0, 3, size=cl.shape[0]).astype(np.int32)
    cmol = np.arange(cl.shape[0], dtype=np.int32)
    ccount = np.bincount(cel, minlength=3)
    cvol = 4.0 / 3.0 * np.pi * 50.0 ** 3
    rv = (0.005 + 0.01 * np.arange(2000)).astype(np.float32)
    sgrid = dict(qmin=0.001, qmax=1.0, dq=0.005, rmin=0.0, rmax=110.0, dr=1.0)
    eye = np.eye(3, dtype=np.float32)
    ms, _ = _call_ms(lambda: gsf.gr_shape_function(cl, eye, False, cmol, cel, ccount, [6.0, 8.0, 14.0], cvol, rv,
                                                   **sgrid), 5)
    out["shape_function_100000"] = {"gpu_ms": ms, "atoms": int(cl.shape[0]),
                                    "pairs": int(cl.shape[0]) * (int(cl.shape[0]) - 1) // 2}
    for name, (fn, reps) in cases(gad, gac, gph).items():
        ms, _ = _call_ms(fn, reps)
        atoms = 5000 if name.endswith("_5000") else (sub if name.endswith("20000") else n)
        per = 1 if name.endswith("move_5000") else (13 if ("move" in name or "group" in name) else atoms)
        out[name] = {"gpu_ms": ms, "atoms": atoms, "atoms_per_call": per}
    if with_cpu:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import build_ref
            R = build_ref.import_reference()
            for name, (fn, reps) in cases(R["atomic_distances"], R["atomic_coordination"],
                                          R["pairs_histograms"]).items():
                if name == "coordination_all_atoms":
                    # the same call on the first 2,000 atoms, scaled to all atoms
                    # (the reference loops over atoms in Python)
                    idx = np.arange(2000, dtype=np.int32)
                    ms, k = _call_ms(lambda: R["atomic_coordination"].multi_atoms_coord_number_coords(
                        idx, c, B, True, *L, data), 2)
                    out[name].update(cpu_reference_ms=ms * n / 2000.0, cpu_sample="2,000 of %d atoms, scaled" % n)
                else:
                    ms, k = _call_ms(fn, 2 if reps < 10 else 10, budget_s=20.0)
                    out[name].update(cpu_reference_ms=ms, cpu_sample="%d calls" % k)
                out[name]["gpu_over_cpu"] = out[name]["cpu_reference_ms"] / out[name]["gpu_ms"]
            # the reference's ShapeFunction cost is its all-pairs float32
            # histogram: timed on the first 10,000 atoms, scaled by pairs
            sub_n = 10000
            Q, edges, centers, mn, mx, b, hs = gsf.shape_function_grids(**sgrid)
            ms, k = _call_ms(lambda: R["pairs_histograms"].full_pairs_histograms_coords(
                cl[:sub_n], eye, False, cmol[:sub_n], cel[:sub_n], 3, mn, mx, b, hs, 1), 1)
            d = out["shape_function_100000"]
            d.update(cpu_reference_ms=ms * d["pairs"] / (sub_n * (sub_n - 1) / 2),
                     cpu_sample="all-pairs histogram of 10,000 of the atoms, scaled by pairs")
            d["gpu_over_cpu"] = d["cpu_reference_ms"] / d["gpu_ms"]
        except Exception as exc:
            out["cpu_error"] = str(exc)[:200]
    return out


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import build_ref
        build_ref.build()
        build_ref.import_reference()
        kind = "reference"
    except Exception as exc:
        print(json.dumps({"impl": "reference", "unavailable": "fullrmc Cython could not be built here: %s" % exc}))
        return 0
    cores = os.cpu_count() or 1
    engines = list(range(256))  # every engine of the workload
    value, procs = reference_rate(engines, args.steps, args.warmup, cores)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * 256 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(ws),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": kind,
                             "sample": "fullrmc Cython (ncores=1) in %d processes: all 256 engines of the workload "
                                       "(the GPU arm's engines), each moved once per step, %d timed steps; a step "
                                       "lasts as long as the slowest process" % (procs, args.steps),
                             "host": _host_cpu()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ our arm
def _flush_l2(buf):
    buf.add_(1)


def bench_allpairs(torch, native, dev, reps=5):
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300._native import F32P
    s = synthetic.triclinic_100k(seed=0)
    m = s.model
    n = s.box_coords.shape[0]
    ne = len(m.elements_count)
    total = ne * ne * m.hs
    st = torch.cuda.Stream()
    c_t = torch.from_numpy(s.box_coords).to(dev)
    el_t = torch.from_numpy(s.el).to(dev)
    mol_t = torch.from_numpy(s.mol).to(dev)
    a4 = torch.empty((n, 4), dtype=torch.float32, device=dev)
    cnt = torch.zeros(2 * total, dtype=torch.int32, device=dev)
    B = np.ascontiguousarray(s.basis)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    with torch.cuda.stream(st):
        native.call("frmc_dev_pack_atoms", c_t.data_ptr(), el_t.data_ptr(), n, a4.data_ptr(), st.cuda_stream)
        args = (a4.data_ptr(), mol_t.data_ptr(), n, B.ctypes.data_as(F32P), 1, ne, m.minDistance, m.maxDistance,
                m.bin, m.hs, cnt.data_ptr(), st.cuda_stream)
        native.call("frmc_dev_full_hist_counts", *args)
        times = []
        for _ in range(reps):
            _flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            native.call("frmc_dev_full_hist_counts", *args)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    counted = int(cnt.sum().item())
    ms = statistics.median(times)
    pairs = n * (n - 1) / 2
    return {"atoms": n, "ms": ms, "pair_distances_per_s": pairs / (ms * 1e-3), "pairs_in_range": counted,
            "launches": 1}


def run_ours(args):
    import torch
    ws, rank = _dist()
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda", torch.cuda.current_device())
    import __graft_entry__
    __graft_entry__.build()
    import fullrmc_gb300
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet, translation_moves

    info = native.device_info()
    peaks, peaks_kind = _peaks()
    seed = 1000 * rank
    amp = 0.1
    systems = synthetic.mixed_engines(seed=seed, count=args.engines)
    E = len(systems)
    K, W = args.steps, args.warmup
    plain_steps = args.plain_steps
    total_steps = W + 3 * K + plain_steps + 8 * len(EngineSet.TUNE_CANDIDATES) + 64
    cap = total_steps
    moves = [translation_moves(np.random.default_rng([seed, 1000 + e]), s.box_coords.shape[0], total_steps, amp)
             for e, s in enumerate(systems)]
    pairs_per_step = float(sum(2 * (s.box_coords.shape[0] - 1) for s in systems))
    mean_atoms = float(np.mean([s.box_coords.shape[0] for s in systems]))

    # autotune the work list (results are identical under every tuning)
    es = EngineSet(systems, move_cap=cap)
    es.init()
    for e, (a, v, u) in enumerate(moves):
        es.push_moves(e, a, v, u, 0)
    tune = es.autotune(steps=6, warmup=2)
    es.close()

    # fresh engines for the measurement
    es = EngineSet(systems, move_cap=cap, tune=tune)
    es.init()
    for e, (a, v, u) in enumerate(moves):
        es.push_moves(e, a, v, u, 0)
    st = torch.cuda.Stream()
    sp = st.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    # the warm-up steps (up to 8) measure the placement of the batched launch
    # (batched steps like the others; the library reorders its work list)
    P = min(8, W)
    if P > 0:
        es.place(P)
    with torch.cuda.stream(st):
        for _ in range(W - P):
            es.step(1, graph=False, sync=False, stream=sp)
        torch.cuda.synchronize()
        # columns the one-CTA steps sweep: all atoms of an engine without a
        # column grid, the selected cells' atoms with one
        swept0 = sum(es.swept(e) for e in range(E))
        if ws > 1:
            torch.distributed.barrier()
        clocks = ClockSampler(dev.index)
        clocks.start()
        ev = []
        torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches
        for _ in range(K):
            _flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            es.step(1, graph=False, sync=False, stream=sp)
            e1.record(st)
            ev.append((e0, e1))
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        step_ms = [a.elapsed_time(b) for a, b in ev]
        swept_per_step = (sum(es.swept(e) for e in range(E)) - swept0) / K
        # steady state: K steps back to back in one CUDA graph (state stays in L2)
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        es.step(K, graph=True, sync=False, stream=sp)  # capture + warm
        torch.cuda.synchronize()
        steps_done = W + 2 * K
        g0.record(st)
        es.step(K, graph=True, sync=False, stream=sp)
        g1.record(st)
        torch.cuda.synchronize()
        steps_done += K
        graph_ms = g0.elapsed_time(g1) / K
        clk = clocks.stop()
    total_ms = sum(step_ms)
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / K
    value = ws * E * K / (total_ms * 1e-3)

    # plain path: the same engines, one at a time (a sample of engines)
    sample = list(range(0, E, max(1, E // args.plain_engines)))[:args.plain_engines]
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        for e in sample:  # warm
            es.step(1, engine=e, graph=False, sync=False, stream=sp)
        torch.cuda.synchronize()
        p0.record(st)
        for _ in range(plain_steps - 1):
            for e in sample:
                es.step(1, engine=e, graph=False, sync=False, stream=sp)
        p1.record(st)
        torch.cuda.synchronize()
    plain_rate = len(sample) * (plain_steps - 1) / (p0.elapsed_time(p1) * 1e-3)
    grid_engines = sum(1 for e in range(E) if es.cells(e) > 0)
    # same accepts: the first W + 3K steps of every engine were batched steps;
    # replay them with the same moves one engine at a time on fresh engines
    # and compare every decision and every chi2 bit pattern
    batched_steps = W + 3 * K
    batched_res = [es.results(e, 0, batched_steps) for e in range(E)]
    es.close()
    es3 = EngineSet(systems, move_cap=batched_steps + 8, tune=tune)
    es3.init()
    for e, (a, v, u) in enumerate(moves):
        es3.push_moves(e, a[:batched_steps], v[:batched_steps], u[:batched_steps], 0)
    for e in range(E):
        es3.step(batched_steps, engine=e, graph=False, sync=False)
    es3.sync()
    mismatch = 0
    for e in range(E):
        c2, acc, _ = es3.results(e, 0, batched_steps)
        if not (np.array_equal(acc, batched_res[e][1]) and
                np.array_equal(c2.view(np.int64), batched_res[e][0].view(np.int64))):
            mismatch += 1
    es3.close()
    same = {"equal": mismatch == 0, "engines": E, "steps": batched_steps, "engines_differing": mismatch,
            "check": "every engine's batched steps (warm-up, timed, graph) replayed one engine at a time on fresh "
                     "engines with the same moves: accept decisions and chi2 bit patterns compared"}

    # e2e: public API with host buffers; every step passes all engines' moves
    # from numpy arrays and reads all engines' chi2 and decisions back into
    # numpy arrays (one result pair per slot).  Two staging slots: the host
    # submits step k + 1 before it collects step k's results.
    es2 = EngineSet(systems, move_cap=4, tune=tune)
    es2.init()
    # the placement of the batched launch, measured on three ring steps
    pm = [translation_moves(np.random.default_rng([seed, 6000 + e]), s.box_coords.shape[0], 3, amp)
          for e, s in enumerate(systems)]
    for e, (a, v, u) in enumerate(pm):
        es2.push_moves(e, a, v, u, 0)
    es2.place(3)
    hm = [translation_moves(np.random.default_rng([seed, 5000 + e]), s.box_coords.shape[0], W + K, amp)
          for e, s in enumerate(systems)]
    A = np.ascontiguousarray(np.stack([m[0] for m in hm]).T)        # (steps, engines)
    V = np.ascontiguousarray(np.stack([m[1] for m in hm]).transpose(1, 0, 2))
    U = np.ascontiguousarray(np.stack([m[2] for m in hm]).T)
    res = [(np.empty(E, np.float64), np.empty(E, np.int32)) for _ in range(2)]
    accepted_e2e = 0
    for k in range(W + K):
        if k == W:
            if k > 0:
                accepted_e2e += int(es2.step_host_collect((k - 1) % 2, res[(k - 1) % 2])[1].sum())
            t0 = time.perf_counter()
        es2.step_host_submit(A[k], V[k], U[k], k % 2)
        if k > W or (k > 0 and k < W):
            accepted_e2e += int(es2.step_host_collect((k - 1) % 2, res[(k - 1) % 2])[1].sum())
    accepted_e2e += int(es2.step_host_collect((W + K - 1) % 2, res[(W + K - 1) % 2])[1].sum())
    t_e2e = time.perf_counter() - t0
    es2.close()
    e2e_value = E * K / t_e2e
    h2d = E * 20  # packed (atom, vector, u) per engine
    d2h = E * 16  # (chi2, accepted, atom) per engine

    allp = bench_allpairs(torch, native, dev)
    configs = dropins = None
    if not args.no_configs and rank == 0:
        configs = bench_configs(torch, with_cpu=not args.no_cpu)
        dropins = bench_dropins(with_cpu=not args.no_cpu)
    serving = None
    if args.serve_seconds > 0 and rank == 0:
        from fullrmc_gb300 import serve
        serving = serve.benchmark_stream(args.serve_seconds, args.serve_limit, seed=seed)
    sms = info["sms"]
    fmax = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    issue_peak = sms * fmax * 128.0 / OPS_PER_PAIR  # pair distances / s
    step_pairs_rate = pairs_per_step / (ms_per_step * 1e-3)
    traffic_path = os.path.join(ROOT, "profiles", "traffic.json")
    traffic = None
    try:
        with open(traffic_path) as fh:
            traffic = json.load(fh).get("k_engine_step_bytes_per_launch")
    except Exception:
        pass

    # reference CPU path on a bounded sample of the same workload
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import build_ref
            build_ref.build()
            build_ref.import_reference()
            pick = stratified(systems, 16)
            rate, procs = reference_rate(pick, 200, 3, 1, seed=seed, amp=amp)
            sample_atoms = float(np.mean([systems[e].box_coords.shape[0] for e in pick]))
            cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "reference",
                   "sample": "fullrmc Cython (ncores=1) on 1 core: 16 of the 256 engines, spread evenly over the "
                             "engines sorted by atom count (mean %.0f atoms; all 256: %.0f), 200 timed steps each"
                             % (sample_atoms, mean_atoms),
                   "host": _host_cpu()}
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "reference", "sample": "failed: %s" % exc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": workload_config(ws, E, amp, seed),
            "tune": {"tile": tune[0], "threads": tune[1], "ctas_per_sm": tune[2]},
            "same_accepts": same,
            "plain": {"steps_per_s": plain_rate, "engines_sampled": len(sample),
                      "batched_over_plain": value / ws / plain_rate},
            "steady_graph": {"ms_per_step": graph_ms, "steps_per_s": E / (graph_ms * 1e-3),
                             "note": "K steps in one CUDA graph, no L2 flush"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "frmc_engines_step_host_submit/collect from numpy arrays; the moves go through "
                            "mapped pinned host memory, which the step kernel reads, and it writes the "
                            "results there (zero-copy over NVLink-C2C)"},
            "roofline": {"bound": "issue", "achieved": step_pairs_rate / 1e9, "peak": issue_peak / 1e9,
                         "unit": "Gpair/s", "frac": step_pairs_rate / issue_peak, "traffic": traffic,
                         "kernel": "k_engine_step", "pairs_per_launch": pairs_per_step,
                         "pairs_evaluated_per_launch": 2.0 * swept_per_step,
                         "evaluated_frac": 2.0 * swept_per_step / (ms_per_step * 1e-3) / issue_peak,
                         "column_grid_engines": grid_engines,
                         "peak_basis": "%d SMs x %.0f MHz (%s) x 128 lanes / %d ops per pair"
                                       % (sms, fmax / 1e6, peaks_kind, OPS_PER_PAIR),
                         "note": "achieved counts the reference's pair evaluations (2 (n - 1) per engine and "
                                 "step); engines with a column grid evaluate only the columns of the cells a "
                                 "moved atom may reach (pairs_evaluated_per_launch)",
                         "allpairs_kernel": "k_full_tiles",
                         "allpairs_workload": "100,000 atoms, triclinic 103 A gamma 120, 3 species, r 0-20 A",
                         "allpairs_ms": allp["ms"],
                         "allpairs_pairs_per_s": allp["pair_distances_per_s"],
                         "allpairs_frac": allp["pair_distances_per_s"] / issue_peak},
            "allpairs": dict(allp, roofline_frac=allp["pair_distances_per_s"] / issue_peak,
                             issue_peak_pairs_per_s=issue_peak),
            "serving": serving,
            "configs": configs,
            "dropins": dropins,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": K,
        }
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--engines", type=int, default=256)
    ap.add_argument("--plain-engines", type=int, default=64)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window of the serving stream (0: skip)")
    ap.add_argument("--no-configs", action="store_true", help="skip the single-engine rates of the other configurations")
    ap.add_argument("--serve-limit", type=float, default=60.0, help="wall-clock limit of the serving run")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
