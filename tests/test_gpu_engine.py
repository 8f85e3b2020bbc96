"""Device-resident engines: exactness against the oracle, and identical
chains alone or batched, under any tile configuration or graph capture."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(count=6, seed=3, nmin=600, nmax=3000):
    from fullrmc_gb300 import synthetic
    return synthetic.mixed_engines(seed=seed, count=count, nmin=nmin, nmax=nmax, rmax=10.0)


def _moves(systems, steps, seed=11, amp=0.3):
    from fullrmc_gb300.engine import translation_moves
    return [translation_moves(np.random.default_rng([seed, k]), s.box_coords.shape[0], steps, amp)
            for k, s in enumerate(systems)]


def _run(systems, moves, steps, mode, tune=None, graph=True, chunk=None):
    from fullrmc_gb300.engine import EngineSet
    es = EngineSet(systems, move_cap=max(64, steps), tune=tune)
    es.init()
    chi2_0 = [es.state(e)[0] for e in range(len(systems))]
    for e, (a, v, u) in enumerate(moves):
        es.push_moves(e, a[:steps], v[:steps], u[:steps], 0)
    chunk = chunk or steps
    if mode == "batched":
        for s0 in range(0, steps, chunk):
            es.step(min(chunk, steps - s0), engine=-1, graph=graph)
    else:
        for e in range(len(systems)):
            for s0 in range(0, steps, chunk):
                es.step(min(chunk, steps - s0), engine=e, graph=graph)
    out = []
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        out.append(dict(chi2=c2, acc=a, atoms=at, state=es.state(e), counts=es.counts(e), coords=es.coords(e),
                        chi2_0=chi2_0[e]))
    es.close()
    return out


def _same(r1, r2):
    for a, b in zip(r1, r2):
        assert np.array_equal(a["acc"], b["acc"])
        assert np.array_equal(a["chi2"].view(np.int64), b["chi2"].view(np.int64))  # bit-identical FP64
        assert a["state"] == b["state"]
        assert np.array_equal(a["counts"][0], b["counts"][0]) and np.array_equal(a["counts"][1], b["counts"][1])
        assert np.array_equal(a["coords"][0], b["coords"][0]) and np.array_equal(a["coords"][1], b["coords"][1])


def test_init_counts_match_oracle(oracle_mod):
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=3)
    es = EngineSet(systems, move_cap=8)
    es.init()
    for e, s in enumerate(systems):
        m = s.model
        want = oracle_mod.full_pairs_histograms_coords(s.box_coords, s.basis, True, s.mol, s.el,
                                                       len(m.elements_count), m.minDistance, m.maxDistance, m.bin,
                                                       m.hs)
        got = es.counts(e)
        assert np.array_equal(got[0].astype(np.float32), want[0])
        assert np.array_equal(got[1].astype(np.float32), want[1])
        c2 = es.state(e)[0]
        ref = m.chi2_fp64(want[0], want[1])
        assert abs(c2 - ref) <= 1e-10 * abs(ref)
    es.close()


def test_batched_equals_solo():
    systems = _systems()
    steps = 120
    mv = _moves(systems, steps)
    batched = _run(systems, mv, steps, "batched")
    solo = _run(systems, mv, steps, "solo")
    _same(batched, solo)
    assert sum(int(r["acc"].sum()) for r in batched) > 0


def test_tune_and_graph_do_not_change_results():
    systems = _systems(count=4, seed=5)
    steps = 80
    mv = _moves(systems, steps, seed=2)
    base = _run(systems, mv, steps, "batched", tune=(1024, 256, 4))
    _same(base, _run(systems, mv, steps, "batched", tune=(128, 128, 8), graph=False))
    _same(base, _run(systems, mv, steps, "batched", tune=(4096, 512, 1), chunk=7))
    _same(base, _run(systems, mv, steps, "solo", tune=(256, 64, 2), chunk=9))


def test_engine_replays_on_oracle(oracle_mod):
    """Replay the device chain on the host with the oracle's histograms and
    the device's decisions: every step's chi2 agrees to 1e-10 relative, the
    decisions follow the FP64 rule, and the final counts and coordinates are
    bit-identical."""
    from fullrmc_gb300.hostloop import HostPDFChain
    systems = _systems(count=2, seed=9, nmin=800, nmax=1500)
    steps = 150
    mv = _moves(systems, steps, seed=4, amp=0.4)
    res = _run(systems, mv, steps, "batched")
    for e, s in enumerate(systems):
        chain = HostPDFChain(s, oracle_mod, oracle_mod)
        chain.compute_data()
        m = s.model
        chi2 = res[e]["chi2_0"]
        assert abs(chi2 - m.chi2_fp64(*chain.data)) <= 1e-10 * abs(chi2)
        a, v, u = mv[e]
        for k in range(steps):
            acc = bool(res[e]["acc"][k])
            chain.step(a[k], v[k][None, :], u[k], force=acc)
            c_new = m.chi2_fp64(chain.last[0], chain.last[1])
            assert abs(c_new - res[e]["chi2"][k]) <= 1e-10 * abs(c_new), k
            expect = not (res[e]["chi2"][k] > chi2 and u[k] > 0.0)
            assert acc == expect, k
            if acc:
                chi2 = res[e]["chi2"][k]
        got = res[e]["counts"]
        assert np.array_equal(got[0].astype(np.float32), chain.data[0])
        assert np.array_equal(got[1].astype(np.float32), chain.data[1])
        assert np.array_equal(res[e]["coords"][0], chain.box)
        assert np.array_equal(res[e]["coords"][1], chain.real)


def test_step_host_matches_ring_steps():
    """The host-buffer batched step gives the same chains as pushed moves."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=5, seed=13)
    steps = 40
    mv = _moves(systems, steps, seed=8)
    ring = _run(systems, mv, steps, "batched")
    es = EngineSet(systems, move_cap=4)
    es.init()
    A = np.stack([m[0] for m in mv])
    V = np.stack([m[1] for m in mv])
    U = np.stack([m[2] for m in mv])
    for k in range(steps):
        c2, acc = es.step_host(A[:, k], V[:, k, :], U[:, k])
        for e in range(len(systems)):
            assert c2[e] == ring[e]["chi2"][k] and acc[e] == ring[e]["acc"][k]
    for e in range(len(systems)):
        assert es.state(e) == ring[e]["state"]
    es.close()


@pytest.mark.parametrize("fused", [1, 0])
def test_step_host_two_slots_match_ring_steps(fused):
    """Submitting step k + 1 before collecting step k (two staging slots)
    gives the same chains as pushed moves -- one kernel on the mapped staging
    buffers when every engine runs in one CTA, copies and tile-split steps
    otherwise; misuse of a slot is refused."""
    from fullrmc_gb300._native import NativeError
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=5, seed=14)
    steps = 41
    mv = _moves(systems, steps, seed=9)
    ring = _run(systems, mv, steps, "batched")
    es = EngineSet(systems, move_cap=4)
    es.set_mode(fused)
    es.init()
    A = np.ascontiguousarray(np.stack([m[0] for m in mv]).T)
    V = np.ascontiguousarray(np.stack([m[1] for m in mv]).transpose(1, 0, 2))
    U = np.ascontiguousarray(np.stack([m[2] for m in mv]).T)
    out = {}
    with pytest.raises(ValueError):
        es.step_host_submit(A[0][:-1], V[0], U[0], 0)  # one engine's move missing
    es.step_host_submit(A[0], V[0], U[0], 0)
    with pytest.raises(NativeError):
        es.step_host_submit(A[1], V[1], U[1], 0)  # slot 0 not collected yet
    # the set cannot change while a step is in flight
    with pytest.raises(NativeError):
        es.add(systems[0])
    with pytest.raises(NativeError):
        es.remove(0)
    assert len(es.live()) == len(systems) and es.E == len(systems)
    bufs = [(np.empty(len(systems), np.float64), np.empty(len(systems), np.int32)) for _ in range(2)]
    for k in range(1, steps):
        es.step_host_submit(A[k], V[k], U[k], k % 2)
        if k % 3:
            out[k - 1] = es.step_host_collect((k - 1) % 2)
        else:  # into caller-owned arrays
            c2, acc = es.step_host_collect((k - 1) % 2, bufs[(k - 1) % 2])
            out[k - 1] = (c2.copy(), acc.copy())
    out[steps - 1] = es.step_host_collect((steps - 1) % 2)
    with pytest.raises(NativeError):
        es.step_host_collect(0)  # nothing in flight
    for k in range(steps):
        c2, acc = out[k]
        for e in range(len(systems)):
            assert c2[e] == ring[e]["chi2"][k] and acc[e] == ring[e]["acc"][k]
    for e in range(len(systems)):
        assert es.state(e) == ring[e]["state"]
        c2, a, at = es.results(e, steps - 4, 4)  # the ring keeps the last move_cap results
        assert np.array_equal(c2.view(np.int64), ring[e]["chi2"][steps - 4:].view(np.int64))
        assert np.array_equal(at, ring[e]["atoms"][steps - 4:])
        assert all(np.array_equal(x, y) for x, y in zip(es.counts(e), ring[e]["counts"]))
        assert all(np.array_equal(x, y) for x, y in zip(es.coords(e), ring[e]["coords"]))
    es.close()


def test_add_remove_keeps_other_chains_exact():
    """Engines added and removed between steps (the serving pattern) do not
    change the results of the others."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=4, seed=17)
    steps = 30
    mv = _moves(systems, steps, seed=3)
    base = _run(systems[:2], mv[:2], steps, "batched")
    es = EngineSet([], move_cap=64)
    ids = [es.add(systems[0]), es.add(systems[1])]
    for e, i in enumerate(ids):
        a, v, u = mv[e]
        es.push_moves(i, a, v, u, 0)
    es.step(10, graph=False)
    extra = es.add(systems[2])
    es.push_moves(extra, *mv[2], 0)
    es.step(10, graph=True)
    es.remove(extra)
    es.step(10, graph=False)
    for e, i in enumerate(ids):
        c2, acc, _ = es.results(i, 0, steps)
        assert np.array_equal(acc, base[e]["acc"])
        assert np.array_equal(c2.view(np.int64), base[e]["chi2"].view(np.int64))
    es.close()


def test_fused_and_split_batched_paths_agree():
    """One-CTA-per-engine steps (shared-memory deltas) and tile-split steps
    (global deltas) give bit-identical chains."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=5, seed=23, nmin=700, nmax=4000)
    steps = 60
    mv = _moves(systems, steps, seed=6)
    out = []
    for fused in (1, 0):
        es = EngineSet(systems, move_cap=64)
        es.set_mode(fused)
        es.init()
        for e, (a, v, u) in enumerate(mv):
            es.push_moves(e, a, v, u, 0)
        es.step(steps, graph=bool(fused))
        out.append([dict(zip(("chi2", "acc", "atoms"), es.results(e, 0, steps)), state=es.state(e),
                         counts=es.counts(e), coords=es.coords(e)) for e in range(len(systems))])
        es.close()
    _same(out[0], out[1])


def test_real_data_chain_replays_on_oracle(oracle_mod):
    """fullrmc's own NiTi example (6,750 atoms, its experimental G(r) as the
    target): a device chain of single-atom moves replays on the oracle with
    every chi2 within 1e-10 and identical final counts and coordinates."""
    from conftest import golden
    from fullrmc_gb300.engine import EngineSystem, PDFModel, normalized_weighting
    from fullrmc_gb300.hostloop import HostPDFChain
    g = golden("niti_pdb")
    el = g["el"]
    counts = np.bincount(el, minlength=int(g["ne"]))
    L = float(g["basis"][0, 0])
    model = PDFModel(r=g["r"], G_exp=g["G_exp"].astype(np.float64), elements_count=counts,
                     weights=normalized_weighting(counts, [10.3, -3.44]), volume=L ** 3)
    s = EngineSystem(box_coords=g["coords"], real_coords=g["real"], el=el, mol=g["mol"], basis=g["basis"],
                     rbasis=g["rbasis"], isPBC=True, model=model)
    steps = 120
    mv = _moves([s], steps, seed=21, amp=0.1)
    res = _run([s], mv, steps, "batched")[0]
    chain = HostPDFChain(s, oracle_mod, oracle_mod)
    chain.compute_data()
    assert np.array_equal(chain.data[1], g["full_inter"])
    chi2 = res["chi2_0"]
    assert abs(chi2 - model.chi2_fp64(*chain.data)) <= 1e-10 * abs(chi2)
    a, v, u = mv[0]
    for k in range(steps):
        acc = bool(res["acc"][k])
        chain.step(a[k], v[k][None, :], u[k], force=acc)
        c_new = model.chi2_fp64(chain.last[0], chain.last[1])
        assert abs(c_new - res["chi2"][k]) <= 1e-10 * abs(c_new), k
        if acc:
            chi2 = res["chi2"][k]
    assert np.array_equal(res["counts"][1].astype(np.float32), chain.data[1])
    assert np.array_equal(res["coords"][0], chain.box)
    assert 0 < int(res["acc"].sum()) < steps


def test_moves_pushed_after_a_step_replace_the_staged_ones():
    """A single-atom step stages the next step's move (and its atom's data)
    while it runs; pushing new moves for those steps afterwards must win.  A
    chain whose moves for steps K.. are replaced after K steps equals a chain
    that had the replacements from the start, batched and alone; so does one
    whose grids are rebuilt between the two halves."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=4, seed=21)
    K = 30
    first = _moves(systems, 2 * K, seed=22)
    second = _moves(systems, 2 * K, seed=23)
    merged = [(np.concatenate([a1[:K], a2[K:]]), np.concatenate([v1[:K], v2[K:]]), np.concatenate([u1[:K], u2[K:]]))
              for (a1, v1, u1), (a2, v2, u2) in zip(first, second)]
    want = _run(systems, merged, 2 * K, "batched", graph=False)
    for engine, regrid in ((-1, False), (1, False), (-1, True)):
        es = EngineSet(systems, move_cap=2 * K)
        es.init()
        for e, (a, v, u) in enumerate(first):
            es.push_moves(e, a, v, u, 0)
        for e in ([-1] if engine == -1 else range(len(systems))):
            es.step(K, engine=e, graph=False)
        for e, (a, v, u) in enumerate(second):
            es.push_moves(e, a[K:], v[K:], u[K:], K)
        if regrid:
            for e in range(len(systems)):
                es.regrid(e)
        for e in ([-1] if engine == -1 else range(len(systems))):
            es.step(K, engine=e, graph=False)
        for e in range(len(systems)):
            c2, acc, _ = es.results(e, 0, 2 * K)
            assert np.array_equal(acc, want[e]["acc"]), (engine, regrid, e)
            assert np.array_equal(c2.view(np.int64), want[e]["chi2"].view(np.int64)), (engine, regrid, e)
            assert all(np.array_equal(x, y) for x, y in zip(es.counts(e), want[e]["counts"]))
        es.close()


def test_lattice_deltas_beyond_four_agree_and_replay(oracle_mod):
    """A simple cubic lattice of one element: an atom moved off its site
    leaves six neighbours at one distance, twelve at the next, so its
    element-pair deltas reach -6 and -12 in one bin, beyond the evaluation's
    -4..4 table.  One-CTA and tile-split steps give bit-identical chains, and
    the chain replays on the oracle."""
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet
    from fullrmc_gb300.hostloop import HostPDFChain
    m, a = 12, 2.2
    L = m * a
    s = synthetic.make_system(np.random.default_rng(17), m ** 3, [1.0], np.diag([L, L, L]), 10.0)
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    s.real_coords = (g * a + 0.1).astype(np.float32)
    s.box_coords = synthetic.transform_f32(s.rbasis, s.real_coords)
    systems = [s]
    steps = 60
    mv = _moves(systems, steps, seed=8, amp=0.3)
    out = []
    for fused in (1, 0):
        es = EngineSet(systems, move_cap=64)
        es.set_mode(fused)
        es.init()
        a_, v_, u_ = mv[0]
        es.push_moves(0, a_, v_, u_, 0)
        es.step(steps, graph=False)
        out.append([dict(zip(("chi2", "acc", "atoms"), es.results(0, 0, steps)), state=es.state(0),
                         counts=es.counts(0), coords=es.coords(0))])
        es.close()
    _same(out[0], out[1])
    res = out[0][0]
    chain = HostPDFChain(s, oracle_mod, oracle_mod)
    chain.compute_data()
    a_, v_, u_ = mv[0]
    for k in range(steps):
        acc = bool(res["acc"][k])
        chain.step(a_[k], v_[k][None, :], u_[k], force=acc)
        c_new = s.model.chi2_fp64(chain.last[0], chain.last[1])
        assert abs(c_new - res["chi2"][k]) <= 1e-10 * abs(c_new), k
    assert np.array_equal(res["counts"][0].astype(np.float32), chain.data[0])
    assert np.array_equal(res["counts"][1].astype(np.float32), chain.data[1])


def test_bins_past_the_histogram_land_in_the_next_row(oracle_mod):
    """maxDistance 40 bins beyond minDistance + hs * bin: a pair in one of
    those bins is counted in bins 0.. of the next oriented row, as the
    reference's unchecked index does (and dropped past the last row).  The
    element-pair deltas follow the same rows; one-CTA and tile-split steps
    agree bit for bit and the chain replays on the oracle."""
    from fullrmc_gb300.engine import EngineSet
    from fullrmc_gb300.hostloop import HostPDFChain
    systems = _systems(count=2, seed=29, nmin=900, nmax=1600)
    for s in systems:
        m = s.model
        m.maxDistance = np.float32(m.minDistance + np.float32(m.hs + 40) * m.bin)
    steps = 60
    mv = _moves(systems, steps, seed=10, amp=0.4)
    out = []
    for fused in (1, 0):
        es = EngineSet(systems, move_cap=64)
        es.set_mode(fused)
        es.init()
        for e, (a_, v_, u_) in enumerate(mv):
            es.push_moves(e, a_, v_, u_, 0)
        es.step(steps, graph=False)
        out.append([dict(zip(("chi2", "acc", "atoms"), es.results(e, 0, steps)), state=es.state(e),
                         counts=es.counts(e), coords=es.coords(e)) for e in range(len(systems))])
        es.close()
    _same(out[0], out[1])
    for e, s in enumerate(systems):
        res = out[0][e]
        chain = HostPDFChain(s, oracle_mod, oracle_mod)
        chain.compute_data()
        a_, v_, u_ = mv[e]
        for k in range(steps):
            chain.step(a_[k], v_[k][None, :], u_[k], force=bool(res["acc"][k]))
            c_new = s.model.chi2_fp64(chain.last[0], chain.last[1])
            assert abs(c_new - res["chi2"][k]) <= 1e-10 * abs(c_new), k
        assert np.array_equal(res["counts"][0].astype(np.float32), chain.data[0])
        assert np.array_equal(res["counts"][1].astype(np.float32), chain.data[1])


def test_measured_placement_keeps_chains():
    """frmc_engines_place reorders the batched work list from recorded SMs
    and times; the chains equal those of a set stepped in the cost order."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=6, seed=31, nmin=700, nmax=3000)
    steps = 40
    mv = _moves(systems, steps, seed=12)
    out = []
    for place in (False, True):
        es = EngineSet(systems, move_cap=64)
        es.init()
        for e, (a_, v_, u_) in enumerate(mv):
            es.push_moves(e, a_, v_, u_, 0)
        if place:
            es.place(3)
            es.step(steps - 3, graph=False)
        else:
            es.step(steps, graph=False)
        es.sync()
        out.append([dict(zip(("chi2", "acc", "atoms"), es.results(e, 0, steps)), state=es.state(e),
                         counts=es.counts(e), coords=es.coords(e)) for e in range(len(systems))])
        es.close()
    _same(out[0], out[1])


def test_host_steps_after_a_placement_match_ring_steps():
    """After frmc_engines_place reorders the work list, host-buffer steps
    (whose moves and results follow the live-engine order) still give every
    engine its own chain."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(count=7, seed=37, nmin=700, nmax=2500)
    steps = 30
    mv = _moves(systems, steps, seed=14)
    ring = _run(systems, mv, steps, "batched")
    es = EngineSet(systems, move_cap=8)
    es.init()
    for e, (a_, v_, u_) in enumerate(mv):
        es.push_moves(e, a_[:3], v_[:3], u_[:3], 0)
    es.place(3)
    A = np.stack([m[0] for m in mv])
    V = np.stack([m[1] for m in mv])
    U = np.stack([m[2] for m in mv])
    for k in range(3, steps):
        c2, acc = es.step_host(A[:, k], V[:, k, :], U[:, k])
        for e in range(len(systems)):
            assert c2[e] == ring[e]["chi2"][k] and acc[e] == ring[e]["acc"][k], (k, e)
    for e in range(len(systems)):
        assert es.state(e) == ring[e]["state"]
    es.close()
