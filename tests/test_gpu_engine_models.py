"""The engines' constraint model beyond plain G(r): a fixed scale factor, a
scale factor refitted every N accepted moves, a window function, g(r)
(PairCorrelationConstraint) and the reduced S(Q).

Each device chain is replayed on the host: the oracle's histograms (with the
device's decisions) and the oracle's literal FP64 restatement of the
constraint (``oracle.pdc_model_fp64`` / ``pcf_model_fp64``: scale factor,
then window; the fit of Core/Constraint.py:1363-1424 on the proposal when
the accepted count is a multiple of the frequency; an accepted move keeps its
scale factor) give every step's chi2 to 1e-10 relative, and the decisions
follow fullrmc's rule.  Chains are also bit-identical alone and batched.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10
F32 = np.float32


def _system(seed, n=900, ns=2, kind="pdf", scale=1.0, fit=(0, 0.8, 1.2), window=None, weights=False, sq=False,
            reduced=False):
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import PDFModel, SQModel
    rng = np.random.default_rng(seed)
    fr = rng.dirichlet(np.ones(ns) * 3.0)
    B = synthetic.random_box(rng, n, rng.uniform(0.08, 0.10))
    s = synthetic.make_system(np.random.default_rng([seed, 1]), n, fr, B, 9.0)
    m = s.model
    exp = np.asarray(m.G_exp, np.float64)
    if kind == "gr":
        c = 4.0 * np.pi * np.asarray(m.r, np.float64) * m.rho0
        exp = np.where(c > 0, 1.0 + exp / np.where(c > 0, c, 1.0), 0.0)
    dw = None
    if weights:
        dw = np.random.default_rng(seed + 7).uniform(0.5, 1.5, len(m.r))
        dw = dw / dw.sum() * len(dw)
    s.model = PDFModel(r=m.r, G_exp=exp.astype(F32), elements_count=m.elements_count, weights=m.weights,
                       volume=m.volume, data_weights=dw, kind=kind, scale_factor=scale, adjust_scale_factor=fit,
                       window=window)
    if sq:
        q = synthetic.q_grid(0.5, 15.0, 0.05)
        s.sq = SQModel(pdf=s.model, q=q, S_exp=np.zeros(len(q)), reduced=reduced)
        S = synthetic.synthetic_S(np.random.default_rng(seed + 3), s.sq, m.G_exp)
        s.sq.S_exp = (S - (1.0 if reduced else 0.0)).astype(F32)
    return s


def _oracle_term(oracle_mod, s, intra, inter, scale):
    m = s.model
    fn = oracle_mod.pcf_model_fp64 if m.kind == "gr" else oracle_mod.pdc_model_fp64
    model = fn(intra, inter, m.elements_count, m.weights, m.volume, m.shell_volumes, m.r, m.rho0, scale,
               m.window_fp64)
    return oracle_mod.standard_error_fp64(m.G_exp, model, m.data_weights) / m.variance_squared


def _oracle_fit(oracle_mod, s, intra, inter):
    m = s.model
    if m.kind == "gr":
        g = oracle_mod.total_gr_fp64(intra, inter, m.elements_count, m.weights, m.volume, m.shell_volumes)
        return oracle_mod.pcf_fit_scale_factor_fp64(m.G_exp, g, m.r, m.rho0, m.data_weights, m.fit_min, m.fit_max)
    G = oracle_mod.total_Gr_fp64(intra, inter, m.elements_count, m.weights, m.volume, m.shell_volumes, m.r, m.rho0)
    return oracle_mod.fit_scale_factor_fp64(m.G_exp, G, m.data_weights, m.fit_min, m.fit_max)


def _oracle_sq_term(oracle_mod, s, intra, inter):
    sq, m = s.sq, s.model
    e = sq.edges
    centers = ((e[:-1] + e[1:]) / F32(2.0)).astype(F32)
    e64 = e.astype(np.float64)
    vols = 4.0 / 3.0 * np.pi * (e64[1:] ** 3 - e64[:-1] ** 3)
    Gr = oracle_mod.total_Gr_fp64(intra, inter, m.elements_count, m.weights, m.volume, vols, centers, m.rho0)
    S = oracle_mod.sq_from_Gr_fp64(Gr, oracle_mod.gr2sq_matrix_fp64(centers, sq.q), reduced=sq.reduced)
    return oracle_mod.standard_error_fp64(sq.S_exp, S, sq.data_weights) / sq.variance_squared


def _chi2(oracle_mod, s, intra, inter, scale):
    c = _oracle_term(oracle_mod, s, intra, inter, scale)
    if s.sq is not None:
        c += _oracle_sq_term(oracle_mod, s, intra, inter)
    return c


def _run(systems, steps, seed, mode="batched", first=0):
    from fullrmc_gb300.engine import EngineSet, translation_moves
    mv = [translation_moves(np.random.default_rng([seed, first + k]), s.box_coords.shape[0], steps, 0.4)
          for k, s in enumerate(systems)]
    es = EngineSet(systems, move_cap=max(64, steps))
    es.init()
    chi2_0 = [es.state(e)[0] for e in range(len(systems))]
    for e, (a, v, u) in enumerate(mv):
        es.push_moves(e, a, v, u, 0)
    for eng in ([-1] if mode == "batched" else range(len(systems))):
        es.step(steps, engine=eng, graph=False)
    out = []
    for e in range(len(systems)):
        c2, a, at = es.results(e, 0, steps)
        out.append(dict(chi2=c2, acc=a, chi2_0=chi2_0[e], state=es.state(e), counts=es.counts(e),
                        coords=es.coords(e)))
    es.close()
    return out, mv


def _replay(oracle_mod, s, res, mv, steps):
    from fullrmc_gb300.hostloop import HostPDFChain
    m = s.model
    chain = HostPDFChain(s, oracle_mod, oracle_mod)
    chain.compute_data()
    # compute_data fits the scale factor for its standard error when the
    # accepted count (0) is a multiple of a non-zero frequency, and keeps the
    # initial one
    sf = m.scale_factor
    s0 = _oracle_fit(oracle_mod, s, *chain.data) if m.fit_frequency else sf
    chi2 = _chi2(oracle_mod, s, chain.data[0], chain.data[1], s0)
    assert abs(chi2 - res["chi2_0"]) <= TOL * abs(chi2)
    a, v, u = mv
    accepted = 0
    for k in range(steps):
        acc = bool(res["acc"][k])
        chain.step(a[k], v[k][None, :], u[k], force=acc)
        intra, inter = chain.last[0], chain.last[1]
        sk = _oracle_fit(oracle_mod, s, intra, inter) if (m.fit_frequency and accepted % m.fit_frequency == 0) \
            else sf
        c_new = _chi2(oracle_mod, s, intra, inter, sk)
        assert abs(c_new - res["chi2"][k]) <= TOL * abs(c_new), k
        assert acc == (not (res["chi2"][k] > chi2 and u[k] > 0.0)), k
        if acc:
            chi2, sf, accepted = res["chi2"][k], sk, accepted + 1
    assert np.array_equal(res["counts"][0].astype(F32), chain.data[0])
    assert np.array_equal(res["counts"][1].astype(F32), chain.data[1])
    assert 0 < accepted < steps


CASES = {
    "pdf_scale_1.15": dict(scale=1.15),
    "pdf_fit_every_4": dict(fit=(4, 0.5, 2.0)),
    "pdf_window_7": dict(window=np.hanning(9)[1:-1]),
    "pdf_fit_window_weights": dict(fit=(3, 0.7, 1.6), window=np.array([1.0, 2.0, 3.0, 2.0]), weights=True, ns=3),
    "gr_plain": dict(kind="gr"),
    "gr_fit_window": dict(kind="gr", fit=(5, 0.5, 2.0), window=np.hanning(7)[1:-1]),
    "pdf_reduced_sq": dict(sq=True, reduced=True),
    "pdf_fit_with_sq": dict(fit=(4, 0.5, 2.0), sq=True),
}


@pytest.mark.parametrize("case", list(CASES))
def test_model_chain_replays_on_oracle(oracle_mod, case):
    s = _system(10 + list(CASES).index(case), **CASES[case])
    steps = 90
    res, mv = _run([s], steps, seed=3)
    _replay(oracle_mod, s, res[0], mv[0], steps)


def test_model_chains_identical_alone_and_batched():
    systems = [_system(k, **CASES[c]) for k, c in enumerate(CASES)] + [_system(99)]
    steps = 40
    batched, _ = _run(systems, steps, seed=5)
    solo, _ = _run(systems, steps, seed=5, mode="solo")
    for a, b in zip(batched, solo):
        assert np.array_equal(a["acc"], b["acc"])
        assert np.array_equal(a["chi2"].view(np.int64), b["chi2"].view(np.int64))
        assert a["state"] == b["state"]
        assert all(np.array_equal(x, y) for x, y in zip(a["counts"], b["counts"]))
    for k, c in enumerate(CASES):
        alone, _ = _run([systems[k]], steps, seed=5, first=k)
        assert np.array_equal(alone[0]["chi2"].view(np.int64), batched[k]["chi2"].view(np.int64)), c


def test_unsupported_sq_options_are_refused():
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import SQModel
    s = _system(1)
    q = synthetic.q_grid(0.5, 10.0, 0.05)
    for kw in (dict(scale_factor=1.1), dict(adjust_scale_factor=(5, 0.8, 1.2)), dict(window=np.ones(3))):
        with pytest.raises(ValueError):
            SQModel(pdf=s.model, q=q, S_exp=np.zeros(len(q)), **kw)
