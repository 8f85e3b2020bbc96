"""Parity at the full sizes of the benchmark workloads.

* The all-pairs histogram of the 100,000-atom triclinic system (three
  species 0.5/0.3/0.2, a = b = c = 103 A, gamma = 120 degrees, r 0-20 A in
  2001 bins; about 5e9 pairs, so the tiled kernel runs with thousands of work
  items per persistent CTA and per-bin counts in the tens of thousands) equals
  the compiled reference's histograms bit for bit (golden files written by
  ``tests/golden/make_cfg2_golden.py``), atomic and with 4-atom molecules.
* The batching workload itself: 256 engines of 1,000-20,000 atoms, 1-4
  species, cubic or triclinic, r 0-12 A.  Stepped together and stepped one
  engine at a time with the same moves, every chain has the same accept
  sequence, bit-identical chi2 values and identical final counts and
  coordinates; the smallest engines' final counts also equal the oracle's
  all-pairs histogram of their final coordinates (up to orientation).
"""
import hashlib

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _set_tune(threads=512, rows=2, queued=-1, qcap=16, ctas=1, min_pairs=8.0e6, aggregate=0):
    from fullrmc_gb300._native import call
    call("frmc_set_full_tune", threads, rows, queued, qcap, ctas, float(min_pairs))
    call("frmc_set_full_aggregate", aggregate)


@pytest.mark.parametrize("name", ["cfg2_triclinic_100k", "cfg2_triclinic_100k_mol4"])
@pytest.mark.parametrize("tune", [dict(), dict(threads=256, rows=1, queued=0), dict(aggregate=1)])
def test_all_pairs_100k_triclinic_equals_reference(name, tune):
    import fullrmc_gb300
    from fullrmc_gb300 import synthetic
    fullrmc_gb300.load()
    g = golden(name)
    s = synthetic.triclinic_100k(seed=int(g["seed"]))
    if int(g["molsize"]) > 1:
        s.mol = (np.arange(s.box_coords.shape[0]) // int(g["molsize"])).astype(np.int32)
    assert _digest(s.box_coords, s.el, s.mol) == str(g["inputs_sha256"]), \
        "the regenerated system differs from the one the golden file was made from"
    m = s.model
    assert (m.minDistance, m.maxDistance, m.bin, m.hs) == (g["minDistance"], g["maxDistance"], g["bin"],
                                                           g["histSize"])
    _set_tune(**tune)
    try:
        hi, he = fullrmc_gb300.pairs_histograms.full_pairs_histograms_coords(
            boxCoords=s.box_coords, basis=s.basis, isPBC=True, moleculeIndex=s.mol, elementIndex=s.el,
            numberOfElements=len(m.elements_count), minDistance=m.minDistance, maxDistance=m.maxDistance,
            bin=m.bin, histSize=m.hs)
    finally:
        _set_tune()
    assert np.array_equal(hi, g["hintra"])
    assert np.array_equal(he, g["hinter"])
    assert he.sum() > 1e8 and (hi.sum() > 0) == (int(g["molsize"]) > 1)


def _sym(h):
    h = np.asarray(h, np.float64)
    return h + np.swapaxes(h, 0, 1) - np.einsum("iik->ik", h)[:, None, :] * np.eye(h.shape[0])[:, :, None]


def test_batching_workload_256_engines_batched_equals_solo(oracle_mod):
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet, translation_moves
    systems = synthetic.mixed_engines(seed=0, count=256)
    steps = 60
    moves = [translation_moves(np.random.default_rng([77, e]), s.box_coords.shape[0], steps, 0.1)
             for e, s in enumerate(systems)]
    runs = {}
    for mode in ("batched", "solo"):
        es = EngineSet(systems, move_cap=64)
        es.init()
        for e, (a, v, u) in enumerate(moves):
            es.push_moves(e, a, v, u, 0)
        if mode == "batched":
            es.step(steps, engine=-1, graph=True)
        else:
            for e in range(len(systems)):
                es.step(steps, engine=e, graph=False)
        runs[mode] = [dict(res=es.results(e, 0, steps), state=es.state(e), counts=es.counts(e),
                           coords=es.coords(e)) for e in range(len(systems))]
        es.close()
    accepted = 0
    for b, s_ in zip(runs["batched"], runs["solo"]):
        assert np.array_equal(b["res"][1], s_["res"][1])                        # accept sequence
        assert np.array_equal(b["res"][0].view(np.int64), s_["res"][0].view(np.int64))  # chi2 bits
        assert b["state"] == s_["state"]
        assert all(np.array_equal(x, y) for x, y in zip(b["counts"], s_["counts"]))
        assert all(np.array_equal(x, y) for x, y in zip(b["coords"], s_["coords"]))
        accepted += int(b["res"][1].sum())
    assert 0 < accepted < 256 * steps
    smallest = np.argsort([s.box_coords.shape[0] for s in systems])[:3]
    for e in smallest:
        s, m = systems[e], systems[e].model
        box = runs["batched"][e]["coords"][0]
        want = oracle_mod.full_pairs_histograms_coords(box, s.basis, True, s.mol, s.el, len(m.elements_count),
                                                       m.minDistance, m.maxDistance, m.bin, m.hs)
        got = runs["batched"][e]["counts"]
        for k in (0, 1):
            assert np.array_equal(_sym(got[k]), _sym(want[k]))
