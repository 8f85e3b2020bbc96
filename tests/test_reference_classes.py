"""fullrmc's own constraint classes, unmodified, against the recorded chains.

CPU only; skipped where the reference checkout or the compiled reference is
absent.  The chains in ``tests/golden/refclass_*.npz`` were recorded by
``tests/golden/make_refclass_chains.py`` from fullrmc's
``PairDistributionConstraint``, ``StructureFactorConstraint`` and
``PairCorrelationConstraint`` (imported as they are, on a stub engine, with
the compiled reference Cython as the histogram backend).  These tests check:

* ``fullrmc_gb300.install()`` makes those modules bind the GPU drop-in's
  functions (the import routing a user relies on);
* the classes reproduce the recordings (decisions, standard errors, digests
  of every histogram call);
* the call replay used by the GPU tests, run on the C oracle, gives the same
  digests and final data as the classes;
* ``fullrmc_gb300.hostloop.HostPDFChain`` (the restated PDF step the GPU
  tests and the benchmark drive) gives the classes' standard error bit for
  bit.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

PREFIX = {"pdc_alloy_5000": 1000}


@pytest.fixture(scope="module")
def classes():
    import build_ref
    if not os.path.isdir(os.path.join(build_ref.REFERENCE_ROOT, "Constraints")):
        pytest.skip("reference checkout absent")
    try:
        build_ref.build()
        R = build_ref.import_reference()
    except Exception as exc:  # pragma: no cover - depends on the checkout
        pytest.skip("compiled reference unavailable: %s" % exc)
    from refclasses import harness
    cls = harness.load_classes(build_ref.REFERENCE_ROOT)
    harness.use_backend(R["pairs_histograms"], R["boundary_conditions_collection"])
    return cls


def _chains():
    from refclasses import harness
    return list(harness.chain_definitions())


def _golden(name):
    from refclasses import harness
    return harness.load_chain(os.path.join(GOLDEN, "refclass_%s.npz" % name))


_INSTALL = r"""
import sys
sys.path[:0] = [ROOT, ROOT + "/oracle", ROOT + "/tests"]
import build_ref
import fullrmc_gb300
fullrmc_gb300.install()
from refclasses import harness
from fullrmc_gb300 import synthetic
PDC, SFC, PCF = harness.load_classes(build_ref.REFERENCE_ROOT, switch=False)
gph = fullrmc_gb300.pairs_histograms
for mod in ("PairDistributionConstraints", "StructureFactorConstraints", "PairCorrelationConstraints"):
    m = sys.modules["fullrmc.Constraints." + mod]
    assert m.multiple_pairs_histograms_coords is gph.multiple_pairs_histograms_coords, mod
    assert m.full_pairs_histograms_coords is gph.full_pairs_histograms_coords, mod
assert sys.modules["fullrmc.Core.pairs_histograms"] is gph
s = synthetic.alloy_5000(seed=1, n=500)
e = harness.StubEngine(s, harness.NAMES)
c = harness.make_constraint((PDC, SFC, PCF), harness.chain_definitions()["pdc_alloy_5000"], s, e)
assert c.histogramSize == 1501
print("install ok")
"""


def test_install_routes_reference_classes_to_dropin(classes):
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + _INSTALL], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "install ok" in r.stdout


@pytest.mark.parametrize("name", _chains())
def test_reference_classes_reproduce_recording(classes, name):
    from refclasses import harness
    g = _golden(name)
    steps = PREFIX.get(name, int(g["steps"]))
    res = harness.run_chain(classes, name, steps=steps)
    assert np.array_equal(res["accepted"], g["accepted"][:steps])
    assert np.array_equal(res["errors"].view(np.int32), g["errors"][:steps].view(np.int32))
    assert np.array_equal(res["checkpoints"], g["checkpoints"][:len(res["checkpoints"])])
    assert np.array_equal(res["weights"], g["weights"])
    if steps == int(g["steps"]):
        assert np.array_equal(res["intra"], g["intra"]) and np.array_equal(res["inter"], g["inter"])


@pytest.mark.parametrize("name", _chains())
def test_call_replay_on_oracle_matches_recording(oracle_mod, name):
    """Needs no reference checkout: the recorded calls replayed on the C oracle."""
    from refclasses import harness
    g = _golden(name)
    steps = PREFIX.get(name, int(g["steps"]))
    system, moves = harness.chain_inputs(name, steps)
    out = harness.replay_calls(oracle_mod, oracle_mod, system, moves, g["accepted"][:steps], g["grid"])
    assert np.array_equal(out["checkpoints"], g["checkpoints"][:len(out["checkpoints"])])
    if steps == int(g["steps"]):
        assert out["calls"] == int(g["calls"])
        assert np.array_equal(out["intra"], g["intra"]) and np.array_equal(out["inter"], g["inter"])


@pytest.mark.parametrize("name", ["pdc_alloy_5000", "pdc_groups_13"])
def test_hostloop_matches_reference_class(oracle_mod, name):
    """Needs no reference checkout: HostPDFChain on the C oracle with the
    class's weights gives the recorded decisions and standard errors."""
    from refclasses import harness
    from fullrmc_gb300.hostloop import HostPDFChain
    g = _golden(name)
    steps = min(PREFIX.get(name, int(g["steps"])), 600)
    system, (idx, vec, u) = harness.chain_inputs(name, steps)
    chain = HostPDFChain(system, oracle_mod, oracle_mod, weights=g["weights"])
    chain.compute_data()
    for k in range(steps):
        acc = chain.step(idx[k], vec[k][None, :], u[k])
        assert acc == g["accepted"][k], k
        assert np.float32(chain.last[2]).view(np.int32) == g["errors"][k].view(np.int32), k
