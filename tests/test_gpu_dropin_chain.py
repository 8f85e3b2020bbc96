"""The drop-in path inside a fullrmc-style Metropolis loop: with the same
moves, the GPU histograms and the oracle give identical accept/reject
sequences over 10^4 steps (the float32 host math is identical, so any
histogram difference would show up as a different decision or error)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_accept_sequence_10k_steps(oracle_mod):
    import fullrmc_gb300
    from fullrmc_gb300 import synthetic
    from fullrmc_gb300.engine import translation_moves
    from fullrmc_gb300.hostloop import HostPDFChain
    s = synthetic.alloy_5000(seed=1)
    gpu = HostPDFChain(s, fullrmc_gb300.pairs_histograms, fullrmc_gb300.boundary_conditions_collection)
    orc = HostPDFChain(s, oracle_mod, oracle_mod)
    assert gpu.compute_data() == orc.compute_data()
    steps = 10000
    a, v, u = translation_moves(np.random.default_rng(2024), s.box_coords.shape[0], steps, 0.1)
    seq_g = np.empty(steps, bool)
    seq_o = np.empty(steps, bool)
    for k in range(steps):
        seq_g[k] = gpu.step(a[k], v[k][None, :], u[k])
        seq_o[k] = orc.step(a[k], v[k][None, :], u[k])
        assert seq_g[k] == seq_o[k], k
        assert gpu.error == orc.error, k
    assert 0 < seq_g.sum() < steps
    assert np.array_equal(gpu.data[0], orc.data[0]) and np.array_equal(gpu.data[1], orc.data[1])
    assert np.array_equal(gpu.box, orc.box)
