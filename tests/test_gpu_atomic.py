"""atomic_distances drop-in on the GPU: every golden case of the compiled
reference bit for bit (counts and float32 sums, whose order the device
reproduces), and seeded random systems against the oracle at sizes with
thousands of contributing pairs."""
import numpy as np
import pytest

from test_oracle_golden import check_atomic_golden

pytestmark = pytest.mark.gpu


def test_atomic_golden():
    from fullrmc_gb300 import atomic_distances
    check_atomic_golden(atomic_distances)


def _system(seed, n, ne, L):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)).astype(np.float32)
    B = (np.eye(3) * L).astype(np.float32)
    mol = (np.arange(n) // 7).astype(np.int32)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    lo = (0.5 + rng.random((ne, ne, 1))).astype(np.float32)
    up = (2.5 + 2.0 * rng.random((ne, ne, 1))).astype(np.float32)
    return c, B, mol, el, lo, up


@pytest.mark.parametrize("kw", [dict(), dict(countWithinLimits=False), dict(reduceDistance=True, allAtoms=False),
                                dict(reduceDistanceToUpper=True, interMolecular=False, countWithinLimits=False)])
def test_atomic_random_vs_oracle(oracle_mod, kw):
    from fullrmc_gb300 import atomic_distances as ad
    ne = 3
    c, B, mol, el, lo, up = _system(5, 20000, ne, 58.0)
    idx = np.random.default_rng(1).integers(0, 20000, size=13).astype(np.int32)
    got = ad.multiple_atomic_distances_coords(idx, c, B, True, mol, el, ne, lo, up, **kw)
    want = oracle_mod.multiple_atomic_distances_coords(idx, c, B, True, mol, el, ne, lo, up, **kw)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    assert got[0].sum() + got[2].sum() > 0


def test_atomic_full_vs_oracle(oracle_mod):
    from fullrmc_gb300 import atomic_distances as ad
    ne = 4
    c, B, mol, el, lo, up = _system(9, 4000, ne, 34.0)
    got = ad.full_atomic_distances_coords(c, B, True, mol, el, ne, lo, up)
    want = oracle_mod.full_atomic_distances_coords(c, B, True, mol, el, ne, lo, up)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    assert got[2].sum() > 1000  # thousands of contributing pairs summed in order
    s_got = ad.pair_elements_stats(el, mol, ne)
    s_want = oracle_mod.pair_elements_stats(el, mol, ne)
    assert np.array_equal(s_got[0], s_want[0]) and np.array_equal(s_got[1], s_want[1])
