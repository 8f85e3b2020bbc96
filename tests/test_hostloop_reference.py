"""Pin the host RMC loop's drop-in use against the compiled reference: the
C oracle and fullrmc's own Cython give identical chains (CPU only; skipped
where the reference sources are not present)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref():
    import build_ref
    try:
        build_ref.build()
        return build_ref.import_reference()
    except Exception as exc:  # pragma: no cover - depends on the checkout
        pytest.skip("compiled reference unavailable: %s" % exc)


def test_chain_oracle_equals_reference(oracle_mod, ref):
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import translation_moves
    from fullrmc_gb300.hostloop import HostPDFChain
    s = synthetic.alloy_5000(seed=3, n=1500)
    a_chain = HostPDFChain(s, oracle_mod, oracle_mod)
    b_chain = HostPDFChain(s, ref["pairs_histograms"], ref["boundary_conditions_collection"])
    assert a_chain.compute_data() == b_chain.compute_data()
    steps = 400
    a, v, u = translation_moves(np.random.default_rng(5), 1500, steps, 0.2)
    for k in range(steps):
        assert a_chain.step(a[k], v[k][None, :], u[k]) == b_chain.step(a[k], v[k][None, :], u[k]), k
        assert a_chain.error == b_chain.error
    assert np.array_equal(a_chain.data[1], b_chain.data[1])
    assert 0 < a_chain.accepted < steps


def test_synthetic_box_coordinates_match_reference_transform(ref):
    from fullrmc_gb300 import synthetic
    s = synthetic.triclinic_100k(seed=0, n=3000)
    box = ref["boundary_conditions_collection"].transform_coordinates(s.rbasis, s.real_coords)
    assert np.array_equal(box, s.box_coords)
