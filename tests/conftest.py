import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_names(prefix=""):
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith(prefix))


HIST_CASES = ["cubic_pbc_ne2", "triclinic120_ne3", "general_triclinic_ne4_mol", "ibc_ne2", "bin_overflow_ibc",
              "bin_edges_ibc", "half_box_pbc", "niti_pdb"]
DIST_CASES = ["dist_cubic_pbc_ne2", "dist_general_triclinic_ne4_mol", "dist_ibc_ne2"]


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
