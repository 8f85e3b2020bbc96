"""Column grids of the device engines.  The one-CTA step that sweeps only the
cells a moved atom may reach gives chains bit-identical to the full sweep:
cubic, triclinic (mildly and strongly skewed) and free-boundary systems, box
coordinates outside [0, 1), moves of several Angstrom that widen the cells,
group moves and an S(Q) term.  A grid chain replays on the oracle, and the
grid is in use where it pays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shifted(system, rng, lo=-0.4, hi=1.4):
    """The system with fractional coordinates drawn from [lo, hi) instead of
    [0, 1) (fullrmc keeps box coordinates unwrapped after moves)."""
    from fullrmc_gb300 import synthetic
    n = system.box_coords.shape[0]
    frac = lo + (hi - lo) * rng.random((n, 3))
    real = (frac @ system.basis.astype(np.float64)).astype(np.float32)
    system.real_coords = real
    system.box_coords = synthetic.transform_f32(system.rbasis, real)
    return system


def _free(system):
    """The system with free boundaries (box coordinates = real coordinates)."""
    system.isPBC = False
    system.box_coords = system.real_coords.copy()
    return system


def _systems(seed=21):
    from fullrmc_gb300 import synthetic
    rng = np.random.default_rng(seed)
    mk = synthetic.make_system
    out = [
        mk(rng, 4000, [0.6, 0.4], np.diag([36.0, 36.0, 36.0]), 8.0),
        mk(rng, 5000, [0.5, 0.3, 0.2], synthetic.triclinic(40.0, 38.0, 41.0, 84, 97, 112), 9.0),
        mk(rng, 3000, [1.0], synthetic.triclinic(40.0, 36.0, 30.0, 70, 75, 128), 7.0),
        _shifted(mk(rng, 3500, [0.5, 0.5], np.diag([34.0, 33.0, 35.0]), 8.0), rng),
        _shifted(mk(rng, 3000, [0.7, 0.3], synthetic.triclinic(35.0, 35.0, 35.0, 90, 90, 120), 8.0), rng),
        _free(mk(rng, 3000, [0.5, 0.5], np.diag([32.0, 32.0, 32.0]), 7.0)),
    ]
    return out


def _run(systems, moves, steps, cells, graph=True):
    from fullrmc_gb300.engine import EngineSet
    es = EngineSet(systems, move_cap=max(64, steps), cells=cells)
    ncells = [es.cells(e) for e in range(len(systems))]
    es.init()
    for e, (s, mv) in enumerate(zip(systems, moves)):
        if s.group_size > 1:
            es.push_group_moves(e, *mv, 0)
        else:
            es.push_moves(e, *mv, 0)
    es.step(steps, engine=-1, graph=graph)
    out = []
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        out.append(dict(chi2=c2, acc=a, state=es.state(e), counts=es.counts(e), coords=es.coords(e),
                        swept=es.swept(e)))
    es.close()
    return out, ncells


def _same(r1, r2):
    for a, b in zip(r1, r2):
        assert np.array_equal(a["acc"], b["acc"])
        assert np.array_equal(a["chi2"].view(np.int64), b["chi2"].view(np.int64))
        assert a["state"] == b["state"]
        for k in (0, 1):
            assert np.array_equal(a["counts"][k], b["counts"][k])
            assert np.array_equal(a["coords"][k], b["coords"][k])


def _moves(systems, steps, seed, amp):
    from fullrmc_gb300.engine import translation_moves
    return [translation_moves(np.random.default_rng([seed, k]), s.box_coords.shape[0], steps, amp)
            for k, s in enumerate(systems)]


@pytest.mark.parametrize("amp", [0.3, 4.0])
def test_grid_chains_equal_full_sweep(amp):
    systems = _systems()
    steps = 150
    mv = _moves(systems, steps, seed=5, amp=amp)
    with_grid, nc = _run(systems, mv, steps, cells=True)
    without, nc0 = _run(systems, mv, steps, cells=False)
    assert all(c > 0 for c in nc), nc
    assert all(c == 0 for c in nc0)
    _same(with_grid, without)
    assert sum(int(r["acc"].sum()) for r in with_grid) > 0
    for s, r, r0 in zip(systems, with_grid, without):
        n = s.box_coords.shape[0]
        assert r0["swept"] == steps * n
        assert 0 < r["swept"] < 0.8 * steps * n, (r["swept"], steps * n)


def test_grid_group_and_sq_chains_equal_full_sweep():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import group_moves, translation_moves
    rings = synthetic.ring_molecules(seed=4, nmol=300, rho=0.1, rmax=8.0)
    rng = np.random.default_rng(8)
    sq = synthetic.make_system(rng, 4000, [0.5, 0.5], np.diag([36.0, 36.0, 36.0]), 8.0,
                               q=synthetic.q_grid(0.5, 12.0, 0.05))
    systems = [rings, sq]
    steps = 120
    mv = [group_moves(np.random.default_rng(3), rings.groups, steps, 0.4, 20.0),
          translation_moves(np.random.default_rng(4), 4000, steps, 0.5)]
    with_grid, nc = _run(systems, mv, steps, cells=True)
    without, _ = _run(systems, mv, steps, cells=False)
    assert all(c > 0 for c in nc), nc
    _same(with_grid, without)


def test_grid_chain_replays_on_oracle(oracle_mod):
    """A grid engine's chain replayed on the host with the oracle's
    histograms: chi2 to 1e-10 at every step and bit-identical final counts
    and coordinates."""
    from fullrmc_gb300.hostloop import HostPDFChain
    systems = _systems()[1:2]
    steps = 120
    mv = _moves(systems, steps, seed=6, amp=1.5)
    res, nc = _run(systems, mv, steps, cells=True)
    assert nc[0] > 0
    s = systems[0]
    chain = HostPDFChain(s, oracle_mod, oracle_mod)
    chain.compute_data()
    m = s.model
    a, v, u = mv[0]
    for k in range(steps):
        acc = bool(res[0]["acc"][k])
        chain.step(a[k], v[k][None, :], u[k], force=acc)
        c_new = m.chi2_fp64(chain.last[0], chain.last[1])
        assert abs(c_new - res[0]["chi2"][k]) <= 1e-10 * abs(c_new), k
    got = res[0]["counts"]
    assert np.array_equal(got[0].astype(np.float32), chain.data[0])
    assert np.array_equal(got[1].astype(np.float32), chain.data[1])
    assert np.array_equal(res[0]["coords"][0], chain.box)
    assert np.array_equal(res[0]["coords"][1], chain.real)


def test_small_engine_gets_no_grid():
    """Where a moved atom reaches most of the box (maxD near half the box)
    the engine sweeps every column."""
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import EngineSet
    s = synthetic.make_system(np.random.default_rng(1), 800, [1.0], np.diag([20.0, 20.0, 20.0]), 9.0)
    es = EngineSet([s], move_cap=8)
    assert es.cells(0) == 0
    es.close()


def test_large_grid_engine_runs_fused_and_equals_split_path():
    """An engine of 60,000 atoms is beyond one CTA's full sweep (it runs
    split over atom tiles without a grid) but sweeps a few thousand columns
    with one, so its batched and one-engine steps run in one CTA; the chains
    are bit-identical."""
    from fullrmc_gb300 import synthetic
    big = synthetic.make_system(np.random.default_rng(12), 60000, [0.5, 0.3, 0.2],
                                synthetic.triclinic(86.0, 86.0, 86.0, 90, 90, 120), 10.0)
    small = _systems()[0]
    systems = [big, small]
    steps = 60
    mv = _moves(systems, steps, seed=9, amp=0.5)
    with_grid, nc = _run(systems, mv, steps, cells=True)
    without, _ = _run(systems, mv, steps, cells=False)
    assert nc[0] > 0
    assert 0 < with_grid[0]["swept"] < 0.2 * steps * 60000   # one-CTA steps
    assert without[0]["swept"] == 0                           # tile-split steps
    _same(with_grid, without)


def test_regrid_mid_chain_keeps_results():
    """Rebuilding the grids from the current coordinates halfway through a
    chain of large moves (their cells have widened) changes nothing."""
    from fullrmc_gb300.engine import EngineSet
    systems = _systems()[:4]
    steps = 120
    mv = _moves(systems, steps, seed=13, amp=4.0)
    without, _ = _run(systems, mv, steps, cells=False)
    es = EngineSet(systems, move_cap=max(64, steps), cells=True)
    es.init()
    for e, (a, v, u) in enumerate(mv):
        es.push_moves(e, a, v, u, 0)
    es.step(steps // 2, engine=-1)
    for e in range(len(systems)):
        es.regrid(e)
    assert all(es.cells(e) > 0 for e in range(len(systems)))
    es.step(steps - steps // 2, engine=-1)
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        assert np.array_equal(a, without[e]["acc"])
        assert np.array_equal(c2.view(np.int64), without[e]["chi2"].view(np.int64))
        assert es.state(e) == without[e]["state"]
        for k in (0, 1):
            assert np.array_equal(es.counts(e)[k], without[e]["counts"][k])
    es.close()
