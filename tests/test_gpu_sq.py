"""Engines with a StructureFactorConstraint term on the device.

S(Q), the S(Q) standard error and chi2 are checked against the oracle's FP64
restatement of StructureFactorConstraints.py (total G(r) on the S(Q) shells,
the dr sin(Qr)/Q matrix, sum w (S_exp - S)^2) from the same integer counts;
every step of a device chain is replayed on the host with the oracle's
histograms; and a chain gives bit-identical results solo, batched, fused,
tile-split and next to engines without an S(Q) term.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative, FP64 S(Q) / chi2 against the oracle


def _systems(count, seed, nmin=600, nmax=2500, dq=0.02):
    from fullrmc_gb300 import synthetic
    rng = np.random.default_rng(seed)
    q = synthetic.q_grid(0.5, 25.0, dq)
    out = []
    for k in range(count):
        n = int(rng.integers(nmin, nmax))
        ns = int(rng.integers(1, 4))
        fr = rng.dirichlet(np.ones(ns) * 3.0)
        B = synthetic.random_box(rng, n, rng.uniform(0.08, 0.10))
        out.append(synthetic.make_system(np.random.default_rng([seed, k]), n, fr, B, 10.0, q=q))
    return out


def _moves(systems, steps, seed=11, amp=0.3):
    from fullrmc_gb300.engine import translation_moves
    return [translation_moves(np.random.default_rng([seed, k]), s.box_coords.shape[0], steps, amp)
            for k, s in enumerate(systems)]


def _oracle_S(oracle_mod, s, intra, inter):
    """S(Q) and its standard error by the oracle's functions."""
    sq, m = s.sq, s.model
    e = sq.edges
    centers = ((e[:-1] + e[1:]) / np.float32(2.0)).astype(np.float32)
    e64 = e.astype(np.float64)
    vols = 4.0 / 3.0 * np.pi * (e64[1:] ** 3 - e64[:-1] ** 3)
    Gr = oracle_mod.total_Gr_fp64(intra, inter, m.elements_count, m.weights, m.volume, vols, centers, m.rho0)
    S = oracle_mod.sq_from_Gr_fp64(Gr, oracle_mod.gr2sq_matrix_fp64(centers, sq.q))
    return S, oracle_mod.standard_error_fp64(sq.S_exp, S, sq.data_weights)


def _oracle_chi2(oracle_mod, s, intra, inter):
    _S, sd_sq = _oracle_S(oracle_mod, s, intra, inter)
    return s.model.chi2_fp64(intra, inter) + sd_sq / s.sq.variance_squared


def _run(systems, moves, steps, mode="batched", fused=1, graph=True, chunk=None, tune=None, gemm_limit=None,
         splits=None):
    from fullrmc_gb300.engine import EngineSet
    es = EngineSet(systems, move_cap=max(64, steps), tune=tune)
    es.set_mode(fused)
    if gemm_limit is not None:
        es.set_sq_gemm_limit(gemm_limit)
    if splits is not None:
        es.set_sq_splits(splits)
    es.init()
    for e, (a, v, u) in enumerate(moves):
        es.push_moves(e, a[:steps], v[:steps], u[:steps], 0)
    chunk = chunk or steps
    engines = [-1] if mode == "batched" else list(range(len(systems)))
    for eng in engines:
        for s0 in range(0, steps, chunk):
            es.step(min(chunk, steps - s0), engine=eng, graph=graph)
    out = []
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        out.append(dict(chi2=c2, acc=a, state=es.state(e), terms=es.terms(e), counts=es.counts(e),
                        coords=es.coords(e)))
    es.close()
    return out


def _same(r1, r2):
    for a, b in zip(r1, r2):
        assert np.array_equal(a["acc"], b["acc"])
        assert np.array_equal(a["chi2"].view(np.int64), b["chi2"].view(np.int64))
        assert a["state"] == b["state"] and a["terms"] == b["terms"]
        assert np.array_equal(a["counts"][0], b["counts"][0]) and np.array_equal(a["counts"][1], b["counts"][1])
        assert np.array_equal(a["coords"][0], b["coords"][0]) and np.array_equal(a["coords"][1], b["coords"][1])


def test_initial_sq_and_chi2_match_oracle(oracle_mod):
    from fullrmc_gb300.engine import EngineSet
    systems = _systems(3, seed=1)
    es = EngineSet(systems, move_cap=8)
    es.init()
    for e, s in enumerate(systems):
        intra, inter = es.counts(e)
        S_ref, sd_ref = _oracle_S(oracle_mod, s, intra, inter)
        S = es.sq(e)
        assert np.max(np.abs(S - S_ref)) <= TOL * np.max(np.abs(S_ref))
        sd, sd_sq = es.terms(e)
        assert abs(sd_sq - sd_ref) <= TOL * sd_ref
        chi2 = es.state(e)[0]
        ref = _oracle_chi2(oracle_mod, s, intra, inter)
        assert abs(chi2 - ref) <= TOL * ref
    assert len(es.tables) == 1  # one table for the shared grids
    es.close()


def test_sq_chain_replays_on_oracle(oracle_mod):
    """Every step's chi2 (G(r) + S(Q) terms) agrees with the oracle's FP64
    value to 1e-10 relative, decisions follow the rule, and the final counts,
    coordinates and S(Q) agree."""
    from fullrmc_gb300.hostloop import HostPDFChain
    systems = _systems(2, seed=5, nmin=700, nmax=1200)
    steps = 120
    mv = _moves(systems, steps, seed=4, amp=0.4)
    res = _run(systems, mv, steps)
    for e, s in enumerate(systems):
        chain = HostPDFChain(s, oracle_mod, oracle_mod)
        chain.compute_data()
        chi2 = _oracle_chi2(oracle_mod, s, *chain.data)
        a, v, u = mv[e]
        for k in range(steps):
            acc = bool(res[e]["acc"][k])
            chain.step(a[k], v[k][None, :], u[k], force=acc)
            c_new = _oracle_chi2(oracle_mod, s, chain.last[0], chain.last[1])
            assert abs(c_new - res[e]["chi2"][k]) <= TOL * abs(c_new), k
            assert acc == (not (res[e]["chi2"][k] > chi2 and u[k] > 0.0)), k
            if acc:
                chi2 = res[e]["chi2"][k]
        got = res[e]["counts"]
        assert np.array_equal(got[0].astype(np.float32), chain.data[0])
        assert np.array_equal(got[1].astype(np.float32), chain.data[1])
        assert np.array_equal(res[e]["coords"][0], chain.box)
        _S, sd_ref = _oracle_S(oracle_mod, s, *chain.data)
        assert abs(res[e]["terms"][1] - sd_ref) <= TOL * sd_ref
        assert int(res[e]["acc"].sum()) > 0


def test_sq_chains_identical_solo_batched_fused_split():
    systems = _systems(4, seed=9, nmin=500, nmax=3000)
    steps = 60
    mv = _moves(systems, steps, seed=2)
    base = _run(systems, mv, steps)
    _same(base, _run(systems, mv, steps, mode="solo", chunk=7))
    _same(base, _run(systems, mv, steps, fused=0, graph=False))
    _same(base, _run(systems, mv, steps, tune=(128, 128, 8), chunk=13))


def test_sq_gemm_digits_give_the_integer_sums_exactly():
    """The tensor-core product (fp16 digit planes of T times fp16 deltas,
    fp32 accumulators in tensor memory) yields the same integers as the exact
    sum over the list of deltas (limit 0) and the dense integer loop (limit
    -1): the chains agree bit for bit, fused and tile-split."""
    systems = _systems(3, seed=17, nmin=800, nmax=2600)
    steps = 40
    mv = _moves(systems, steps, seed=6, amp=0.5)
    base = _run(systems, mv, steps)
    _same(base, _run(systems, mv, steps, gemm_limit=0))
    _same(base, _run(systems, mv, steps, gemm_limit=-1, graph=False))
    _same(base, _run(systems, mv, steps, gemm_limit=1, fused=0))


def test_sq_and_plain_engines_mixed():
    """Engines with and without an S(Q) term in one set keep their solo chains."""
    from fullrmc_gb300 import synthetic
    sq_sys = _systems(2, seed=21)
    plain = synthetic.mixed_engines(seed=4, count=2, nmin=600, nmax=2000, rmax=10.0)
    steps = 50
    mixed = [sq_sys[0], plain[0], sq_sys[1], plain[1]]
    mv = _moves(mixed, steps, seed=8)
    both = _run(mixed, mv, steps)
    for k in range(4):
        _same([both[k]], _run([mixed[k]], [mv[k]], steps))


def test_table_shape_mismatch_is_refused():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300._native import NativeError
    from fullrmc_gb300.engine import EngineSet, SQModel
    a = _systems(1, seed=3)[0]
    es = EngineSet([], move_cap=8)
    other = SQModel(pdf=a.model, q=synthetic.q_grid(0.5, 10.0, 0.05), S_exp=np.zeros(191))
    tid = es.sq_table(other)
    from fullrmc_gb300.engine import make_spec
    from fullrmc_gb300._native import load, check
    import ctypes
    sp, _keep = make_spec(a, 8, sq_table=tid)
    i = ctypes.c_int32()
    with pytest.raises((ValueError, NativeError)):
        check(load().frmc_engines_add(es.handle, ctypes.byref(sp), ctypes.byref(i)))
    es.close()


def test_sq_many_engines_span_several_column_blocks():
    """More delta columns than one tile block holds (128): the product is
    tiled over several blocks of whole engines; every chain is still the
    same batched, split and alone."""
    systems = _systems(56, seed=31, nmin=300, nmax=900)
    assert sum(len(s.model.pair_i) for s in systems) > 128
    steps = 25
    mv = _moves(systems, steps, seed=32)
    base = _run(systems, mv, steps)
    _same(base, _run(systems, mv, steps, mode="solo", graph=False))
    _same(base, _run(systems, mv, steps, fused=0))
    _same(base, _run(systems, mv, steps, gemm_limit=0))


def test_sq_large_group_moves_take_the_exact_sum():
    """16-atom group moves in a dense one-species system with a long r range
    (0-36 A, 3,601 bins) change more than 2^14 unit counts in one delta
    column (the per-bin changes partly cancel, so a short range stays far
    below), beyond the tensor-core product's exact range (2^13): those
    columns take the exact integer sum, and the chain equals the all-list
    chain (limit 0) bit for bit."""
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import SQModel
    rng = np.random.default_rng(41)
    n, G = 40000, 16
    L = (n / 0.1) ** (1.0 / 3.0)
    s = synthetic.make_system(rng, n, [1.0], np.diag([L, L, L]), 36.0, molsize=G)
    q = synthetic.q_grid(0.5, 20.0, 0.05)
    s.sq = SQModel(pdf=s.model, q=q, S_exp=np.zeros(len(q)))
    s.sq.S_exp = synthetic.synthetic_S(np.random.default_rng(2), s.sq, s.model.G_exp)
    s.group_size = G
    s.groups = np.arange(n, dtype=np.int32).reshape(-1, G)
    steps = 12
    from fullrmc_gb300.engine import group_moves
    mv = group_moves(np.random.default_rng(5), s.groups, steps, 0.4, 20.0)
    # the first move's unit count changes in the one delta column, on the host
    import oracle
    m = s.model
    kw = dict(basis=s.basis, isPBC=True, numberOfElements=1, minDistance=m.minDistance,
              maxDistance=m.maxDistance, bin=m.bin, histSize=m.hs)
    from fullrmc_gb300.engine import group_new_real
    def delta(box, idx):
        iM, eM = oracle.multiple_pairs_histograms_coords(idx, box, moleculeIndex=s.mol, elementIndex=s.el,
                                                         allAtoms=True, **kw)
        iF, eF = oracle.full_pairs_histograms_coords(box[idx], moleculeIndex=s.mol[idx], elementIndex=s.el[idx],
                                                     **kw)
        return (iM - iF) + (eM - eF)
    l1 = []
    for k in range(3):
        idx = mv[0][k]
        box2 = s.box_coords.copy()
        box2[idx] = synthetic.transform_f32(s.rbasis, group_new_real(s.real_coords[idx], mv[1][k], mv[2][k]))
        l1.append(np.abs(delta(box2, idx) - delta(s.box_coords, idx)).sum())
    assert max(l1) > 2 ** 14, l1

    def run(limit):
        from fullrmc_gb300.engine import EngineSet
        es = EngineSet([s], move_cap=64)
        if limit is not None:
            es.set_sq_gemm_limit(limit)
        es.init()
        es.push_group_moves(0, *mv, 0)
        es.step(steps, graph=False)
        out = dict(res=es.results(0, 0, steps), state=es.state(0), terms=es.terms(0), counts=es.counts(0))
        es.close()
        return out
    a, b = run(None), run(0)
    assert np.array_equal(a["res"][1], b["res"][1])
    assert np.array_equal(a["res"][0].view(np.int64), b["res"][0].view(np.int64))
    assert a["state"] == b["state"] and a["terms"] == b["terms"]
    assert all(np.array_equal(x, y) for x, y in zip(a["counts"], b["counts"]))


def test_sq_k_splits_do_not_change_the_chain():
    """The tensor-core product splits each 128-row block's bins over K
    splits whose fp32 partial sums are added in L2 in any order; every
    partial sum is an exact integer, so one split, a few and as many as fill
    the SMs give bit-identical chains, batched and alone."""
    systems = _systems(12, seed=23, nmin=900, nmax=3000)
    steps = 30
    mv = _moves(systems, steps, seed=24)
    base = _run(systems, mv, steps)
    _same(base, _run(systems, mv, steps, splits=1))
    _same(base, _run(systems, mv, steps, splits=3, graph=False))
    _same(base, _run(systems, mv, steps, splits=2, mode="solo", chunk=9))


def test_sq_odd_small_and_largest_histograms_in_one_batch(oracle_mod):
    """Three S(Q) tables in one batched step: 338 bins (neither K chunks of 32
    nor row blocks of 128 divide it), 1,001 bins and 4,091 bins (32 row
    blocks of 128, next to the 4,096-bin limit); each engine's chain replays
    on the oracle to 1e-10 and equals the same engine stepped alone."""
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.hostloop import HostPDFChain
    specs = [(900, 3.37, (0.5, 25.0, 0.02)), (1200, 10.0, (0.5, 20.0, 0.02)), (2500, 40.9, (0.5, 10.0, 0.05))]
    systems = []
    for k, (n, rmax, qg) in enumerate(specs):
        rng = np.random.default_rng([61, k])
        B = synthetic.random_box(rng, n, 0.09)
        systems.append(synthetic.make_system(np.random.default_rng([62, k]), n, [0.6, 0.4], B, rmax,
                                             q=synthetic.q_grid(*qg)))
    assert [s.model.hs for s in systems] == [338, 1001, 4091]
    steps = 40
    mv = _moves(systems, steps, seed=63, amp=0.4)
    res = _run(systems, mv, steps)
    _same(res, _run(systems, mv, steps, mode="solo", graph=False))
    for e, s in enumerate(systems):
        chain = HostPDFChain(s, oracle_mod, oracle_mod)
        chain.compute_data()
        chi2 = _oracle_chi2(oracle_mod, s, *chain.data)
        a, v, u = mv[e]
        for k in range(steps):
            acc = bool(res[e]["acc"][k])
            chain.step(a[k], v[k][None, :], u[k], force=acc)
            c_new = _oracle_chi2(oracle_mod, s, chain.last[0], chain.last[1])
            assert abs(c_new - res[e]["chi2"][k]) <= TOL * abs(c_new), (e, k)
            assert acc == (not (res[e]["chi2"][k] > chi2 and u[k] > 0.0)), (e, k)
            if acc:
                chi2 = res[e]["chi2"][k]
        assert np.array_equal(res[e]["counts"][0].astype(np.float32), chain.data[0])
        assert np.array_equal(res[e]["counts"][1].astype(np.float32), chain.data[1])
        assert int(res[e]["acc"].sum()) > 0
