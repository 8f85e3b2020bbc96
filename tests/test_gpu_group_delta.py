"""The group-move delta in one launch (frmc_group_move_delta_histograms):
(M - F) after minus (M - F) before, where M is multiple_pairs_histograms_coords
on the group against all atoms and F is full_pairs_histograms_coords on the
group alone (PairDistributionConstraints.py:1044-1129), equals the difference
of the oracle's four histograms bin for bin: single atoms, a whole molecule,
random groups, a group of more than one 64-row chunk, triclinic periodic and
free boundaries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32 = np.float32


def _system(seed, n=2500, ne=3, molsize=4, pbc=True):
    from fullrmc_gb300 import synthetic
    rng = np.random.default_rng(seed)
    if pbc:
        B = synthetic.triclinic(30.0, 31.0, 29.0, 88.0, 93.0, 117.0).astype(F32)
    else:
        B = np.eye(3, dtype=F32)
    box = rng.random((n, 3)).astype(F32) if pbc else (rng.random((n, 3)) * 30.0).astype(F32)
    el = rng.integers(0, ne, n).astype(np.int32)
    mol = (np.arange(n) // molsize).astype(np.int32)
    kw = dict(basis=B, isPBC=pbc, numberOfElements=ne, minDistance=F32(0.3), maxDistance=F32(9.905),
              bin=F32(0.01), histSize=960)
    return box, el, mol, kw


def _oracle_delta(oracle_mod, box, new, idx, el, mol, kw):
    def mf(b):
        iM, eM = oracle_mod.multiple_pairs_histograms_coords(idx, b, moleculeIndex=mol, elementIndex=el,
                                                             allAtoms=True, **kw)
        iF, eF = oracle_mod.full_pairs_histograms_coords(b[idx], moleculeIndex=mol[idx], elementIndex=el[idx], **kw)
        return iM - iF, eM - eF
    after = box.copy()
    after[idx] = new
    (ia, ea), (ib, eb) = mf(after), mf(box)
    return (ia - ib).astype(np.int64), (ea - eb).astype(np.int64)


@pytest.mark.parametrize("case", ["one_atom", "molecule", "random13", "random70", "free_boundaries"])
def test_group_move_delta_equals_the_oracle(oracle_mod, case):
    from fullrmc_gb300.pairs_histograms import group_move_delta_histograms
    pbc = case != "free_boundaries"
    box, el, mol, kw = _system({"one_atom": 1, "molecule": 2, "random13": 3, "random70": 4,
                                "free_boundaries": 5}[case], pbc=pbc)
    rng = np.random.default_rng(7)
    n = box.shape[0]
    if case == "one_atom":
        idx = np.array([1234], np.int32)
    elif case == "molecule":
        idx = np.arange(400, 404, dtype=np.int32)
    else:
        idx = rng.choice(n, 70 if case == "random70" else 13, replace=False).astype(np.int32)
    step = (0.02 if pbc else 0.6)
    new = (box[idx] + rng.uniform(-step, step, (len(idx), 3))).astype(F32)
    di, de = group_move_delta_histograms(idx, box, new, kw["basis"], kw["isPBC"], mol, el, kw["numberOfElements"],
                                         kw["minDistance"], kw["maxDistance"], kw["bin"], kw["histSize"])
    wi, we = _oracle_delta(oracle_mod, box, new, idx, el, mol, kw)
    assert di.dtype == np.int32 and di.shape == wi.shape
    assert np.array_equal(di.astype(np.int64), wi)
    assert np.array_equal(de.astype(np.int64), we)
    assert np.abs(de).sum() > 0
    if case == "molecule":
        assert np.abs(di).sum() > 0  # the moved molecule's own pairs change bins


def test_group_move_delta_refuses_bad_arguments():
    from fullrmc_gb300.pairs_histograms import group_move_delta_histograms
    box, el, mol, kw = _system(9, n=200)
    args = (kw["basis"], kw["isPBC"], mol, el, kw["numberOfElements"], kw["minDistance"], kw["maxDistance"],
            kw["bin"], kw["histSize"])
    with pytest.raises(ValueError):
        group_move_delta_histograms(np.array([1, 2], np.int32), box, box[:3], *args)
    with pytest.raises(IndexError):
        group_move_delta_histograms(np.array([1, 500], np.int32), box, box[:2], *args)
    with pytest.raises(ValueError):
        idx = np.arange(1025, dtype=np.int32) % 200
        group_move_delta_histograms(idx, box, np.zeros((1025, 3), F32), *args)
