"""Group moves in the device engines: whole molecules translated or rotated
about their centroid (fullrmc's TranslationGenerator / RotationGenerator on
molecule groups).  A device chain replayed on the host with the oracle's
histograms (fullrmc's M - F before/after-move data) agrees at every step to
1e-10 in chi2 and bit for bit in the final counts and coordinates, and a group
chain is bit-identical alone, batched with single-atom engines, fused or
tile-split, and with an S(Q) term.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _groups(system, steps, seed, amp=0.3, angle=25.0):
    from fullrmc_gb300.engine import group_moves
    return group_moves(np.random.default_rng(seed), system.groups, steps, amp, angle)


def _run(systems, moves, steps, mode="batched", fused=1, graph=True, initial=None):
    from fullrmc_gb300.engine import EngineSet
    es = EngineSet(systems, move_cap=max(64, steps))
    es.set_mode(fused)
    es.init()
    if initial is not None:
        initial.extend(es.counts(e) for e in range(len(systems)))
    for e, (s, mv) in enumerate(zip(systems, moves)):
        if s.group_size > 1:
            es.push_group_moves(e, *mv, 0)
        else:
            es.push_moves(e, *mv, 0)
    for eng in ([-1] if mode == "batched" else range(len(systems))):
        es.step(steps, engine=eng, graph=graph)
    out = []
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        out.append(dict(chi2=c2, acc=a, state=es.state(e), counts=es.counts(e), coords=es.coords(e)))
    es.close()
    return out


def _same(r1, r2):
    for a, b in zip(r1, r2):
        assert np.array_equal(a["acc"], b["acc"])
        assert np.array_equal(a["chi2"].view(np.int64), b["chi2"].view(np.int64))
        assert a["state"] == b["state"]
        for k in (0, 1):
            assert np.array_equal(a["counts"][k], b["counts"][k])
            assert np.array_equal(a["coords"][k], b["coords"][k])


def _replay(oracle_mod, s, res, mv, steps, data0=None):
    from fullrmc_gb300.engine import group_new_real
    from fullrmc_gb300.hostloop import HostPDFChain
    chain = HostPDFChain(s, oracle_mod, oracle_mod)
    if data0 is None:
        chain.compute_data()
    else:  # the initial all-pairs counts (checked against the oracle elsewhere)
        chain.data = (data0[0].astype(np.float32), data0[1].astype(np.float32))
        chain.error = chain.standard_error(*chain.data)
    m = s.model
    chi2 = m.chi2_fp64(*chain.data)
    atoms, kinds, params, u = mv
    for k in range(steps):
        acc = bool(res["acc"][k])
        new = group_new_real(chain.real[atoms[k]], kinds[k], params[k])
        chain.step(atoms[k], None, u[k], force=acc, moved_real=new)
        c_new = m.chi2_fp64(chain.last[0], chain.last[1])
        assert abs(c_new - res["chi2"][k]) <= 1e-10 * abs(c_new), k
        assert acc == (not (res["chi2"][k] > chi2 and u[k] > 0.0)), k
        if acc:
            chi2 = res["chi2"][k]
    assert np.array_equal(res["counts"][0].astype(np.float32), chain.data[0])
    assert np.array_equal(res["counts"][1].astype(np.float32), chain.data[1])
    assert np.array_equal(res["coords"][0], chain.box)
    assert np.array_equal(res["coords"][1], chain.real)
    assert 0 < int(res["acc"].sum()) < steps or steps < 5


def test_group_chain_replays_on_oracle(oracle_mod):
    from fullrmc_gb300 import synthetic
    s = synthetic.ring_molecules(seed=2, nmol=60, rmax=9.0)
    steps = 80
    mv = _groups(s, steps, seed=5)
    assert 0 < mv[1].sum() < steps  # both rotations and translations
    res = _run([s], [mv], steps)[0]
    _replay(oracle_mod, s, res, mv, steps)


def test_large_group_engine_split_path_replays(oracle_mod):
    """52,000 atoms (4,000 molecules): above the one-CTA limit, so the batched
    step uses the tile-split path.  The replay starts from the device's
    initial all-pairs counts (a 52,000-atom oracle histogram takes minutes)."""
    from fullrmc_gb300 import synthetic
    s = synthetic.ring_molecules(seed=3, nmol=4000, rmax=15.0)
    steps = 6
    mv = _groups(s, steps, seed=6)
    initial = []
    res = _run([s], [mv], steps, initial=initial)[0]
    _replay(oracle_mod, s, res, mv, steps, data0=initial[0])


def test_group_chains_identical_in_any_mix():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import translation_moves
    g1 = synthetic.ring_molecules(seed=7, nmol=40, rmax=8.0)
    g2 = synthetic.ring_molecules(seed=8, nmol=90, rmax=8.0)
    single = synthetic.mixed_engines(seed=9, count=2, nmin=600, nmax=1500, rmax=8.0)
    steps = 40
    systems = [g1, single[0], g2, single[1]]
    moves = [_groups(g1, steps, 1), translation_moves(np.random.default_rng(2), single[0].box_coords.shape[0],
                                                      steps, 0.3),
             _groups(g2, steps, 3), translation_moves(np.random.default_rng(4), single[1].box_coords.shape[0],
                                                      steps, 0.3)]
    base = _run(systems, moves, steps)
    _same(base, _run(systems, moves, steps, mode="solo", graph=False))
    _same(base, _run(systems, moves, steps, fused=0))
    for k in (0, 2):
        _same([base[k]], _run([systems[k]], [moves[k]], steps))


def test_group_engine_with_sq_term_identical_solo_and_batched():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import SQModel
    s = synthetic.ring_molecules(seed=11, nmol=50, rmax=8.0)
    q = synthetic.q_grid(0.5, 20.0, 0.05)
    s.sq = SQModel(pdf=s.model, q=q, S_exp=np.zeros(len(q)))
    s.sq.S_exp = synthetic.synthetic_S(np.random.default_rng(1), s.sq, s.model.G_exp)
    steps = 30
    mv = _groups(s, steps, seed=12)
    a = _run([s], [mv], steps)
    _same(a, _run([s], [mv], steps, mode="solo", graph=False))
    _same(a, _run([s], [mv], steps, fused=0))


def test_group_moves_are_validated():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet
    s = synthetic.ring_molecules(seed=1, nmol=10, rmax=6.0)
    es = EngineSet([s], move_cap=8)
    atoms = np.tile(np.arange(13, dtype=np.int32), (2, 1))
    atoms[1, 5] = atoms[1, 4]  # an atom twice in one group
    with pytest.raises(ValueError):
        es.push_group_moves(0, atoms, np.zeros(2, np.int32), np.zeros((2, 9), np.float32), np.ones(2, np.float32), 0)
    with pytest.raises(ValueError):
        es.push_moves(0, np.zeros(1, np.int32), np.zeros((1, 3), np.float32), np.ones(1, np.float32), 0)
    es.close()
