"""The GPU drop-in inside chains of fullrmc's own constraint classes.

The chains in ``tests/golden/refclass_*.npz`` were recorded from fullrmc's
``PairDistributionConstraint`` (plain; with a fitted scale factor and a
window function; with 13-atom group moves), ``StructureFactorConstraint``
and ``PairCorrelationConstraint``, imported unmodified and run on the
compiled reference Cython (``tests/golden/make_refclass_chains.py``).  The
reference checkout is not needed here:

* every histogram call those classes made -- ``compute_data``'s all-pairs
  call and, per move, M and F before and after the move -- is issued again
  through ``fullrmc_gb300.pairs_histograms`` (with the recorded decisions),
  and the digests of all call inputs and outputs agree at every
  100-move checkpoint, as do the final data arrays and coordinates.  The
  classes' float32 host math sees identical histograms, so their decisions
  and standard errors are those of the recording;
* for the PDF chains, fullrmc's step restated in ``hostloop.HostPDFChain``
  on the drop-in replays the recorded decisions: each move's total standard
  error agrees with the classes' to float32 summation rounding (1e-5), the chain's own
  decision is the recorded one except at near-ties (a change within 1e-5 of
  the error), and the final data arrays are the classes' bit for bit.  The
  recordings were made on x86-64, and numpy's vectorised float32 pairwise
  sums round differently on other machines (the GPU hosts are aarch64), so a
  near-tie can fall either way there; on the recording machine the classes'
  standard errors and decisions are matched bit for bit
  (tests/test_reference_classes.py), and the histograms behind them are
  compared bit for bit above.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CHAINS = ["pdc_alloy_5000", "pdc_scaled_window", "pdc_groups_13", "sfc_alloy_2000", "pcf_triclinic_3000"]


def _golden(name):
    from refclasses import harness
    return harness.load_chain(os.path.join(GOLDEN, "refclass_%s.npz" % name))


@pytest.mark.parametrize("name", CHAINS)
def test_dropin_replays_reference_class_chain(name):
    import fullrmc_gb300
    from refclasses import harness
    fullrmc_gb300.load()
    g = _golden(name)
    steps = int(g["steps"])
    system, moves = harness.chain_inputs(name, steps)
    idx, vec, u = moves
    assert hashlib.sha256(idx.tobytes() + vec.tobytes() + u.tobytes()).hexdigest() == str(g["moves_sha256"])
    out = harness.replay_calls(fullrmc_gb300.pairs_histograms, fullrmc_gb300.boundary_conditions_collection,
                               system, moves, g["accepted"], g["grid"])
    assert out["calls"] == int(g["calls"])
    bad = [k for k, (a, b) in enumerate(zip(out["checkpoints"], g["checkpoints"])) if a != b]
    assert not bad, "first differing block of 100 moves: %d" % bad[0]
    assert np.array_equal(out["intra"], g["intra"]) and np.array_equal(out["inter"], g["inter"])
    assert hashlib.sha256(np.ascontiguousarray(out["box"]).tobytes()).hexdigest() == str(g["box_sha256"])


@pytest.mark.parametrize("name", ["pdc_alloy_5000", "pdc_groups_13"])
def test_dropin_chain_decides_like_reference_class(name):
    import fullrmc_gb300
    from refclasses import harness
    from fullrmc_gb300.hostloop import HostPDFChain
    g = _golden(name)
    steps = int(g["steps"])
    system, (idx, vec, u) = harness.chain_inputs(name, steps)
    chain = HostPDFChain(system, fullrmc_gb300.pairs_histograms, fullrmc_gb300.boundary_conditions_collection,
                         weights=g["weights"])
    chain.compute_data()
    own = np.zeros(steps, bool)
    err = np.zeros(steps, np.float32)
    gap = np.zeros(steps, np.float64)
    for k in range(steps):
        before = chain.error
        chain.step(idx[k], vec[k][None, :], u[k], force=bool(g["accepted"][k]))
        err[k] = chain.last[2]
        own[k] = not (err[k] > before and u[k] > 0.0)
        gap[k] = abs(float(err[k]) - float(before)) / abs(float(before))
    rel = np.abs(err.astype(np.float64) - g["errors"]) / np.abs(g["errors"].astype(np.float64))
    assert rel.max() <= 1e-5, "standard error differs by %g at move %d" % (rel.max(), int(np.argmax(rel)))
    flips = np.flatnonzero(own != g["accepted"])
    assert np.all(gap[flips] <= 1e-5), "a decision differs away from a near-tie at move %d" % flips[0]
    assert flips.size <= max(2, steps // 100)
    assert 0 < g["accepted"].sum() < steps
    assert np.array_equal(chain.data[0], g["intra"]) and np.array_equal(chain.data[1], g["inter"])
