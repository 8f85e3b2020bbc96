"""atomic_coordination drop-in on the GPU: every golden case of the compiled
reference bit for bit, seeded systems against the oracle at sizes with
hundreds of thousands of counted pairs, the float32 stop at 2^24, and the
constraint's move bookkeeping (the data updated from before/after-move
counts equals a full recomputation) on a 30,000-atom system."""
import numpy as np
import pytest

from coordination_cases import definitions
from test_oracle_golden import check_coordination_golden

pytestmark = pytest.mark.gpu
F = np.float32


def test_coordination_golden():
    from fullrmc_gb300 import atomic_coordination
    check_coordination_golden(atomic_coordination)


def _system(seed, n, L, defs, ne=3):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)).astype(F)
    B = np.diag([L, L, L]).astype(F)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    return c, B, definitions(el, defs)


DEFS = [(0, 1, 1.2, 3.1), (1, 2, 0.8, 2.7), (2, 2, 1.5, 3.6), (0, 0, 0.0, 2.4)]


@pytest.mark.parametrize("isPBC", [True, False])
def test_multi_atoms_vs_oracle(oracle_mod, isPBC):
    from fullrmc_gb300 import atomic_coordination as ac
    c, B, L = _system(4, 20000, 58.0, DEFS)
    if not isPBC:
        c = (c * F(58.0)).astype(F)
    idx = np.random.default_rng(2).integers(0, 20000, size=40).astype(np.int32)
    data0 = (np.random.default_rng(3).random(len(DEFS)) * 100).astype(F)
    got, want = data0.copy(), data0.copy()
    ac.multi_atoms_coord_number_coords(idx, c, B, isPBC, *L, got)
    oracle_mod.multi_atoms_coord_number_coords(idx, c, B, isPBC, *L, want)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    assert (got - data0).sum() > 100


def test_all_atoms_and_dists_vs_oracle(oracle_mod):
    from fullrmc_gb300 import atomic_coordination as ac
    c, B, L = _system(6, 3000, 31.0, DEFS)
    got, want = np.zeros(len(DEFS), F), np.zeros(len(DEFS), F)
    ac.all_atoms_coord_number_coords(c, B, True, *L, got)
    oracle_mod.all_atoms_coord_number_coords(c, B, True, *L, want)
    assert np.array_equal(got, want) and got.sum() > 10000
    idx = np.arange(0, 3000, 37, dtype=np.int32)
    rows = [oracle_mod.pairs_distances_to_indexcoords(int(a), c, B, True, True) for a in idx]
    got, want = np.full(len(DEFS), F(0.25)), np.full(len(DEFS), F(0.25))
    ac.multi_atoms_coord_number_totdists(idx, rows, *L, got)
    oracle_mod.multi_atoms_coord_number_totdists(idx, rows, *L, want)
    assert np.array_equal(got, want)
    s_got = ac.single_atom_multi_shells_coords(5, L[1], c, B, True, np.array(L[2], F), np.array(L[3], F))
    s_want = oracle_mod.single_atom_multi_shells_coords(5, L[1], c, B, True, np.array(L[2], F), np.array(L[3], F))
    assert np.array_equal(s_got, s_want)


def test_count_stops_at_2_pow_24():
    """A float32 sum of ones stays at 2^24 (atomic_coordination.pyx:42-43)."""
    from fullrmc_gb300 import atomic_coordination as ac
    d = np.zeros((1 << 24) + 5, F)
    assert ac.single_atom_single_shell_subdists(d, 0.0, 1.0) == float(1 << 24)
    assert ac.single_atom_single_shell_subdists(d[:1000], 0.0, 1.0) == 1000.0


def test_move_bookkeeping_matches_full_recompute():
    """The constraint's move data (AtomicCoordinationConstraints.py:520-580):
    all_atoms counts every (core, shell) pair from both of its atoms, and the
    before/after data of a moved atom count its pairs once, so for one moved
    atom the full data changes by 2 (after - before) (all integers below
    2^24: the float32 arithmetic is exact)."""
    from fullrmc_gb300 import atomic_coordination as ac
    c, B, L = _system(8, 30000, 68.0, DEFS)
    nd = len(DEFS)
    data = np.zeros(nd, F)
    ac.all_atoms_coord_number_coords(c, B, True, *L, data)
    rng = np.random.default_rng(9)
    changed = 0
    for step in range(6):
        atom = np.array([rng.integers(0, 30000)], np.int32)
        before = np.zeros(nd, F)
        ac.multi_atoms_coord_number_coords(atom, c, B, True, *L, before)
        moved = c.copy()
        moved[atom] = ((c[atom] + (rng.random((1, 3)) - 0.5).astype(F) * F(0.06)) % F(1.0)).astype(F)
        after = np.zeros(nd, F)
        ac.multi_atoms_coord_number_coords(atom, moved, B, True, *L, after)
        data = (data + F(2) * (after - before)).astype(F)
        changed += int(np.abs(after - before).sum())
        c = moved
        full = np.zeros(nd, F)
        ac.all_atoms_coord_number_coords(c, B, True, *L, full)
        assert np.array_equal(data, full), step
    assert data.sum() > 1e5 and changed > 0
