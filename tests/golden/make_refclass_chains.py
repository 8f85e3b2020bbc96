"""Chains of fullrmc's own constraint classes, recorded on the compiled
reference.

Run in a checkout that has the reference sources (``python
tests/golden/make_refclass_chains.py``).  For every chain of
``tests/refclasses/harness.py:chain_definitions`` this imports fullrmc's
``PairDistributionConstraint``, ``StructureFactorConstraint`` and
``PairCorrelationConstraint`` unmodified (with the harness's stub engine and
third-party shims), runs the chain with the compiled reference Cython as the
histogram backend (``ncores=1``) and writes ``tests/golden/refclass_<name>.npz``:
the decisions, the total standard error after every move (float32), digest
checkpoints of every histogram call (inputs and outputs) each 100 moves, the
final data arrays, the class's element-pair weights and its histogram grid.
"""
from __future__ import annotations

import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def main(names=None):
    import build_ref
    from refclasses import harness
    build_ref.build()
    R = build_ref.import_reference()
    classes = harness.load_classes(build_ref.REFERENCE_ROOT)
    harness.use_backend(R["pairs_histograms"], R["boundary_conditions_collection"])
    for name in names or harness.chain_definitions():
        t0 = time.time()
        res = harness.run_chain(classes, name)
        path = os.path.join(HERE, "refclass_%s.npz" % name)
        harness.save_chain(path, name, res)
        print("wrote %s: %d steps, %d accepted, %d histogram calls, %.1f s"
              % (path, len(res["accepted"]), int(res["accepted"].sum()), res["calls"], time.time() - t0))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
