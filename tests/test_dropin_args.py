"""Argument handling of the drop-in modules mirrors the reference's Cython
signatures (TypeError for None / wrong types, ValueError for a wrong dtype or
number of dimensions).  All checks fire before any device work, so no GPU is
needed."""
import inspect

import numpy as np
import pytest

from fullrmc_gb300 import atomic_coordination as ac
from fullrmc_gb300 import atomic_distances as ad
from fullrmc_gb300 import pairs_distances as pd
from fullrmc_gb300 import pairs_histograms as ph
from fullrmc_gb300 import reciprocal_space as rs

F, I = np.float32, np.int32
C = np.zeros((4, 3), F)
B = np.eye(3, dtype=F)
M = np.zeros(4, I)

_COORD_LISTS = ("coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs, "
                 "coordNumData, ncores=1")

REFERENCE_SIGNATURES = {
    ph.single_pairs_histograms: "atomIndex, distances, moleculeIndex, elementIndex, hintra, hinter, minDistance, "
                                "maxDistance, bin, allAtoms=True, ncores=1",
    ph.multiple_pairs_histograms_coords: "indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex, "
                                         "numberOfElements, minDistance, maxDistance, bin, histSize, allAtoms=True, "
                                         "ncores=1",
    ph.multiple_pairs_histograms_dists: "indexes, distances, moleculeIndex, elementIndex, numberOfElements, "
                                        "minDistance, maxDistance, bin, histSize, allAtoms=True, ncores=1",
    ph.full_pairs_histograms_coords: "boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, "
                                     "minDistance, maxDistance, bin, histSize, ncores=1",
    ph.full_pairs_histograms_dists: "distances, moleculeIndex, elementIndex, numberOfElements, minDistance, "
                                    "maxDistance, bin, histSize, ncores=1",
    pd.pairs_distances_to_indexcoords: "atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1",
    pd.pairs_distances_to_point: "point, coords, basis, isPBC, ncores=1",
    pd.pairs_distances_to_multi_points: "points, coords, basis, isPBC, ncores=1",
    pd.pairs_distances_to_multi_indexcoords: "indexes, coords, basis, isPBC, allAtoms=True, ncores=1",
    pd.point_to_point_distance: "point1, point2, basis, isPBC, ncores=1",
    pd.from_to_points_differences: "pointsFrom, pointsTo, basis, isPBC, ncores=1",
    pd.pair_difference_to_point: "point1, point2, basis, isPBC, ncores=1",
    pd.pairs_differences_to_point: "point, coords, basis, isPBC, ncores=1",
    pd.pairs_differences_to_indexcoords: "atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1",
    pd.pairs_differences_to_multi_points: "points, coords, basis, isPBC, ncores=1",
    pd.pairs_differences_to_multi_indexcoords: "indexes, coords, basis, isPBC, allAtoms=True, ncores=1",
    rs.gr_to_sq: "distances, gr, qrange, rho",
    rs.Gr_to_sq: "distances, Gr, qrange",
    rs.sq_to_Gr: "qValues, rValues, sq",
    ad.single_atomic_distances_dists: "atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, nintra, "
                                      "ninter, lowerLimit, upperLimit, interMolecular=True, intraMolecular=True, "
                                      "countWithinLimits=True, reduceDistanceToUpper=False, "
                                      "reduceDistanceToLower=False, reduceDistance=False, allAtoms=True, ncores=1",
    ad.single_atomic_distances_dists_serial: "atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, "
                                             "nintra, ninter, lowerLimit, upperLimit, interMolecular=True, "
                                             "intraMolecular=True, countWithinLimits=True, "
                                             "reduceDistanceToUpper=False, reduceDistanceToLower=False, "
                                             "reduceDistance=False, allAtoms=True",
    ad.multiple_atomic_distances_coords: "indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex, "
                                         "numberOfElements, lowerLimit, upperLimit, interMolecular=True, "
                                         "intraMolecular=True, countWithinLimits=True, reduceDistanceToUpper=False, "
                                         "reduceDistanceToLower=False, reduceDistance=False, allAtoms=True, ncores=1",
    ad.multiple_atomic_distances_dists: "indexes, distances, moleculeIndex, elementIndex, numberOfElements, "
                                        "lowerLimit, upperLimit, interMolecular=True, intraMolecular=True, "
                                        "countWithinLimits=True, reduceDistanceToUpper=False, "
                                        "reduceDistanceToLower=False, reduceDistance=False, allAtoms=True, ncores=1",
    ad.full_atomic_distances_coords: "boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, "
                                     "lowerLimit, upperLimit, interMolecular=True, intraMolecular=True, "
                                     "reduceDistanceToUpper=False, reduceDistanceToLower=False, reduceDistance=False, "
                                     "countWithinLimits=True, ncores=1",
    ad.full_atomic_distances_dists: "distances, moleculeIndex, elementIndex, numberOfElements, lowerLimit, "
                                    "upperLimit, interMolecular=True, intraMolecular=True, "
                                    "reduceDistanceToUpper=False, reduceDistanceToLower=False, reduceDistance=False, "
                                    "countWithinLimits=True",
    ad.pair_elements_stats: "elementIndex, moleculeIndex, numberOfElements",
    ac.single_atom_single_shell_subdists: "distances, lowerShell, upperShell, ncores=1",
    ac.single_atom_single_shell_totdists: "distances, shellIndexes, lowerShell, upperShell, ncores=1",
    ac.single_atom_single_shell_coords: "coreIndex, shellIndexes, boxCoords, basis, isPBC, lowerShell, upperShell, "
                                        "ncores=1",
    ac.single_atom_multi_shells_totdists: "distances, shellsIndexes, lowerShells, upperShells, ncores=1",
    ac.single_atom_multi_shells_coords: "coreIndex, shellsIndexes, boxCoords, basis, isPBC, lowerShells, "
                                        "upperShells, ncores=1",
    ac.single_atom_coord_number_totdists: "atomIndex, distances, " + _COORD_LISTS,
    ac.single_atom_coord_number_coords: "atomIndex, boxCoords, basis, isPBC, " + _COORD_LISTS,
    ac.multi_atoms_coord_number_totdists: "indexes, distances, " + _COORD_LISTS,
    ac.multi_atoms_coord_number_coords: "indexes, boxCoords, basis, isPBC, " + _COORD_LISTS,
    ac.all_atoms_coord_number_totdists: "distances, " + _COORD_LISTS,
    ac.all_atoms_coord_number_coords: "boxCoords, basis, isPBC, " + _COORD_LISTS,
}


@pytest.mark.parametrize("fn", list(REFERENCE_SIGNATURES), ids=lambda f: f.__name__)
def test_signature_matches_reference(fn):
    assert str(inspect.signature(fn))[1:-1] == REFERENCE_SIGNATURES[fn]


def test_none_raises_type_error():
    with pytest.raises(TypeError):
        ph.full_pairs_histograms_coords(None, B, True, M, M, 1, 0.0, 1.0, 0.1, 10)
    with pytest.raises(TypeError):
        ph.multiple_pairs_histograms_coords(None, C, B, True, M, M, 1, 0.0, 1.0, 0.1, 10)


def test_wrong_dtype_raises_value_error():
    with pytest.raises(ValueError, match="dtype mismatch"):
        ph.full_pairs_histograms_coords(C.astype(np.float64), B, True, M, M, 1, 0.0, 1.0, 0.1, 10)
    with pytest.raises(ValueError, match="dtype mismatch"):
        ph.full_pairs_histograms_coords(C, B, True, M.astype(np.int64), M, 1, 0.0, 1.0, 0.1, 10)


def test_wrong_ndim_raises_value_error():
    with pytest.raises(ValueError, match="dimensions"):
        ph.full_pairs_histograms_coords(C.ravel(), B, True, M, M, 1, 0.0, 1.0, 0.1, 10)


def test_float_for_integer_raises_type_error():
    with pytest.raises(TypeError):
        ph.full_pairs_histograms_coords(C, B, True, M, M, 1.5, 0.0, 1.0, 0.1, 10)


def test_int32_overflow():
    with pytest.raises(OverflowError):
        ph.full_pairs_histograms_coords(C, B, True, M, M, 2 ** 40, 0.0, 1.0, 0.1, 10)


def test_short_index_arrays_rejected():
    with pytest.raises(ValueError):
        ph.full_pairs_histograms_coords(C, B, True, M[:2], M, 1, 0.0, 1.0, 0.1, 10)


def test_empty_inputs_need_no_device():
    hi, he = ph.multiple_pairs_histograms_coords(np.zeros(0, I), C, B, True, M, M, 2, 0.0, 1.0, 0.1, 10)
    assert hi.shape == (2, 2, 10) and not hi.any() and not he.any()
    hi, he = ph.full_pairs_histograms_coords(np.zeros((1, 3), F), B, True, M[:1], M[:1], 2, 0.0, 1.0, 0.1, 10)
    assert not hi.any() and not he.any()
    assert ph.full_pairs_histograms_coords(C, B, True, M, M, 0, 0.0, 1.0, 0.1, 10)[0].shape == (0, 0, 10)


def test_atomic_limits_shape_is_checked():
    lo = np.zeros((2, 2, 1), F)
    with pytest.raises(AssertionError):
        ad.multiple_atomic_distances_coords(M[:1], C, B, True, M, M, 3, lo, lo)
    with pytest.raises(AssertionError):
        ad.multiple_atomic_distances_coords(M[:1], C, B, True, M, M, 2, np.zeros((2, 2, 2), F),
                                            np.zeros((2, 2, 2), F))
    with pytest.raises(ValueError, match="dtype mismatch"):
        ad.multiple_atomic_distances_coords(M[:1], C, B, True, M, M, 2, lo.astype(np.float64), lo)


def _coord_lists():
    cores = [np.array([0, 1], I)]
    shells = [np.array([2, 3], I)]
    asCore = [np.array([0], I), np.array([0], I), np.zeros(0, I), np.zeros(0, I)]
    inShell = [np.zeros(0, I), np.zeros(0, I), np.array([0], I), np.array([0], I)]
    return cores, shells, [F(0.5)], [F(2.0)], asCore, inShell


def test_coordination_argument_checks_need_no_device():
    L = _coord_lists()
    data = np.zeros(1, F)
    with pytest.raises(TypeError, match="expected list"):
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, tuple(L[0]), *L[1:], data)
    with pytest.raises(ValueError, match="dtype mismatch"):
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, *L, np.zeros(1))
    with pytest.raises(ValueError, match="dtype mismatch"):
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, L[0], [L[1][0].astype(np.int64)], *L[2:], data)
    with pytest.raises(ValueError, match="dtype mismatch"):
        ac.multi_atoms_coord_number_coords(M[:1].astype(np.int64), C, B, True, *L, data)
    with pytest.raises(IndexError):  # the reference reads outside its list here
        ac.multi_atoms_coord_number_coords(np.array([-1], I), C, B, True, *L, data)
    with pytest.raises(IndexError):  # definition 0 on a zero-length coordNumData
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, *L, np.zeros(0, F))
    with pytest.raises(ValueError, match="read-only"):
        ro = np.zeros(1, F)
        ro.flags.writeable = False
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, *L, ro)
    with pytest.raises(TypeError, match="expected list"):
        ac.multi_atoms_coord_number_totdists(M[:1], np.zeros((1, 4), F), *L, data)
    with pytest.raises(TypeError, match="expected list, got numpy.ndarray"):
        ac.all_atoms_coord_number_totdists(np.zeros((4, 4), F), *L, data)
    with pytest.raises(ValueError, match="dtype mismatch"):
        ac.all_atoms_coord_number_totdists(np.zeros((4, 4)), *L, data)
    with pytest.raises(ValueError, match="dtype mismatch"):
        ac.single_atom_single_shell_subdists(np.zeros(3), 0.5, 1.0)
    with pytest.raises(TypeError):
        ac.single_atom_single_shell_coords(0.5, M, C, B, True, 0.5, 1.0)
    with pytest.raises(TypeError):
        ac.single_atom_multi_shells_totdists(np.zeros(4, F), (M,), np.zeros(1, F), np.zeros(1, F))
    with pytest.raises(TypeError, match="real number"):
        ac.multi_atoms_coord_number_coords(M[:1], C, B, True, L[0], L[1], ["0.5"], *L[3:], data)
    # nothing to do: no device call, data unchanged
    ac.multi_atoms_coord_number_coords(np.zeros(0, I), C, B, True, *L, data)
    ac.multi_atoms_coord_number_coords(np.array([2], I), C, B, True, L[0], L[1], L[2], L[3],
                                       [np.zeros(0, I)] * 4, [np.zeros(0, I)] * 4, data)
    assert data[0] == 0
