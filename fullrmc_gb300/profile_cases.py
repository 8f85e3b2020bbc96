"""Small, self-contained runs of the hot kernels, sized for profiling.

    python -m fullrmc_gb300.profile_cases allpairs --n 30000 --reps 3 [--aggregate 1]
    python -m fullrmc_gb300.profile_cases engines --count 64 --steps 5 [--tune 1024,1024,1] [--sq]
    python -m fullrmc_gb300.profile_cases serve --seconds 3 --limit 30

``allpairs`` runs the all-pairs histogram (three species, triclinic box with
gamma = 120 degrees at 0.1057 atoms/A^3, r 0-20 A) on device buffers;
``engines`` runs batched Metropolis steps of ``count`` mixed-size engines
(with ``--sq`` each also has an S(Q) term on Q 0.5-25 A^-1, dQ 0.01);
``serve`` runs the serving loop on a Poisson stream of fits.  Each prints one
JSON line (CUDA-event times per launch for the first two).
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def allpairs(n, reps, aggregate=0):
    import torch
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300._native import F32P
    s = synthetic.triclinic_100k(seed=0, n=n)
    m = s.model
    ne = len(m.elements_count)
    total = ne * ne * m.hs
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream()
    c = torch.from_numpy(s.box_coords).to(dev)
    el = torch.from_numpy(s.el).to(dev)
    mol = torch.from_numpy(s.mol).to(dev)
    a4 = torch.empty((n, 4), dtype=torch.float32, device=dev)
    cnt = torch.zeros(2 * total, dtype=torch.int32, device=dev)
    B = np.ascontiguousarray(s.basis)
    native.call("frmc_set_full_aggregate", int(aggregate))
    with torch.cuda.stream(st):
        native.call("frmc_dev_pack_atoms", c.data_ptr(), el.data_ptr(), n, a4.data_ptr(), st.cuda_stream)
        args = (a4.data_ptr(), mol.data_ptr(), n, B.ctypes.data_as(F32P), 1, ne, m.minDistance, m.maxDistance,
                m.bin, m.hs, cnt.data_ptr(), st.cuda_stream)
        ev = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            native.call("frmc_dev_full_hist_counts", *args)
            e1.record(st)
            ev.append((e0, e1))
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    native.call("frmc_set_full_aggregate", 0)
    return {"case": "allpairs", "atoms": n, "aggregate": int(aggregate), "ms": ms, "pairs": n * (n - 1) / 2,
            "in_range": int(cnt.sum().item())}


def engines(count, steps, tune=None, sq=False):
    import torch
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet, translation_moves
    systems = synthetic.mixed_engines(seed=0, count=count)
    if sq:
        from fullrmc_gb300.engine import SQModel
        q = synthetic.q_grid()
        for k, s in enumerate(systems):
            s.sq = SQModel(pdf=s.model, q=q, S_exp=np.zeros(len(q)))
            s.sq.S_exp = synthetic.synthetic_S(np.random.default_rng([k, 3]), s.sq, s.model.G_exp)
    es = EngineSet(systems, move_cap=steps + 4, tune=tune)
    es.init()
    for e, s in enumerate(systems):
        a, v, u = translation_moves(np.random.default_rng([0, e]), s.box_coords.shape[0], steps, 0.1)
        es.push_moves(e, a, v, u, 0)
    st = torch.cuda.Stream()
    ev = []
    with torch.cuda.stream(st):
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            es.step(1, graph=False, sync=False, stream=st.cuda_stream)
            e1.record(st)
            ev.append((e0, e1))
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    pairs = sum(2 * (s.box_coords.shape[0] - 1) for s in systems)
    acc = sum(es.state(e)[2] for e in range(count))
    es.close()
    return {"case": "engines", "engines": count, "steps": steps, "sq": sq, "ms": ms, "pairs_per_step": pairs,
            "accepted": acc}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["allpairs", "engines", "serve"])
    ap.add_argument("--n", type=int, default=30000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--aggregate", type=int, default=0, help="all-pairs binning: 1 = warp-aggregated atomics")
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--tune", default=None, help="tile,threads,ctas_per_sm of the engine work list")
    ap.add_argument("--sq", action="store_true")
    ap.add_argument("--seconds", type=float, default=3.0)
    ap.add_argument("--limit", type=float, default=30.0)
    a = ap.parse_args()
    tune = tuple(int(x) for x in a.tune.split(",")) if a.tune else None
    if a.case == "allpairs":
        out = allpairs(a.n, a.reps, a.aggregate)
    elif a.case == "engines":
        out = engines(a.count, a.steps, tune, a.sq)
    else:
        from fullrmc_gb300 import serve
        out = serve.benchmark_stream(a.seconds, a.limit)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
