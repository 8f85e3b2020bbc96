"""The serving loop on the device: each fit's accept sequence, per-step chi2,
final chi2 and histograms are bit-identical whether it runs alone or in a mix
of fits that arrive and leave at other times (fits with and without an S(Q)
term, one large enough for the tile-split path)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fits():
    from fullrmc_gb300 import synthetic
    q = synthetic.q_grid(0.5, 25.0, 0.05)
    rng = np.random.default_rng(42)
    fits = []
    for k, (n, steps, with_sq) in enumerate([(1500, 150, True), (3000, 90, False), (900, 200, True),
                                             (52000, 40, True), (2200, 130, True)]):
        B = synthetic.random_box(rng, n, 0.09)
        fr = rng.dirichlet(np.ones(1 + k % 3) * 3.0)
        s = synthetic.make_system(np.random.default_rng([7, k]), n, fr, B, 10.0, q=q if with_sq else None)
        fits.append((s, steps))
    return fits


def _server(move_cap=64):
    from fullrmc_gb300 import serve
    from fullrmc_gb300.engine import EngineSet, footprint
    es = EngineSet([], move_cap=move_cap)
    return serve.Server(es, lambda s: footprint(s, move_cap), 8 << 30, max_k=16, keep_counts=True, record=True)


def test_fit_alone_equals_fit_in_mix():
    from fullrmc_gb300 import serve
    fits = _fits()
    reqs = [serve.FitRequest(i, s, steps, seed=100 + i, amplitude=0.3) for i, (s, steps) in enumerate(fits)]
    mix = _server()
    mix.submit(reqs[0])
    mix.submit(reqs[1])
    mix.iterate()
    mix.submit(reqs[2])
    mix.iterate()
    mix.iterate()
    mix.submit(reqs[3])
    mix.submit(reqs[4])
    mix.drain()
    for r in reqs:
        got = mix.results[r.rid]
        assert got.status == "done" and got.steps == r.steps, got.error
        alone = _server()
        alone.submit(serve.FitRequest(r.rid, r.system, r.steps, r.seed, r.amplitude))
        alone.drain()
        want = alone.results[r.rid]
        assert np.array_equal(got.trace[1], want.trace[1])
        assert np.array_equal(got.trace[0].view(np.int64), want.trace[0].view(np.int64))
        assert got.chi2 == want.chi2 and got.accepted == want.accepted
        assert np.array_equal(got.counts[0], want.counts[0]) and np.array_equal(got.counts[1], want.counts[1])
        alone.es.close()
    assert mix.peak_live >= 3
    assert sum(int(mix.results[r.rid].accepted) for r in reqs) > 0
    mix.es.close()


def test_served_chi2_matches_fp64_model():
    """The chi2 a served fit ends with is its final counts' FP64 chi2."""
    from fullrmc_gb300 import serve
    s, steps = _fits()[0]
    srv = _server()
    srv.submit(serve.FitRequest(0, s, 300, seed=5, amplitude=0.3))
    srv.drain()
    res = srv.results[0]
    ref = s.chi2_fp64(*res.counts)
    assert abs(res.chi2 - ref) <= 1e-10 * ref
    srv.es.close()
