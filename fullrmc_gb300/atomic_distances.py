"""Drop-in replacement of ``fullrmc.Core.atomic_distances`` on the GPU.

Same function names, positional order, keyword names, defaults and return
conventions as ``Extensions/atomic_distances.pyx`` (used by
InterMolecularDistanceConstraint, ``Constraints/DistanceConstraints.py:569-697``).
The pairs are evaluated on the device; the counts are exact and the float32
sums follow the reference's loop order, so every result equals the
reference's ``ncores=1`` result bit for bit.  ``ncores`` is accepted and
ignored.
"""
from __future__ import annotations

import numpy as np

from . import _args as A
from ._native import F32P, I32P, call, ptr

NUMPY_FLOAT32 = np.float32
NUMPY_INT32 = np.int32


def _flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
           reduceDistance):
    return ((1 if A.bint(interMolecular) else 0) | (2 if A.bint(intraMolecular) else 0) |
            (4 if A.bint(countWithinLimits) else 0) | (8 if A.bint(reduceDistanceToUpper) else 0) |
            (16 if A.bint(reduceDistanceToLower) else 0) | (32 if A.bint(reduceDistance) else 0))


def _limits(numberOfElements, lowerLimit, upperLimit):
    lo = A.array("lowerLimit", lowerLimit, np.float32, 3)
    up = A.array("upperLimit", upperLimit, np.float32, 3)
    ne = A.int32("numberOfElements", numberOfElements)
    shape = lo.shape
    # atomic_distances.pyx:376-378
    assert shape[0] == shape[1] and shape[0] == ne, \
        "lowerLimit array must have numberOfElements columns and numberOfElements rows"
    assert shape[2] == 1, "lowerLimit array third dimension must have a length of exactly 1"
    if up.shape != lo.shape:
        raise ValueError("upperLimit must have the shape of lowerLimit")
    return ne, lo, up


def _outputs(ne):
    return (np.zeros((ne, ne, 1), NUMPY_INT32), np.zeros((ne, ne, 1), NUMPY_FLOAT32),
            np.zeros((ne, ne, 1), NUMPY_INT32), np.zeros((ne, ne, 1), NUMPY_FLOAT32))


def single_atomic_distances_dists(atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, nintra, ninter,
                                  lowerLimit, upperLimit, interMolecular=True, intraMolecular=True,
                                  countWithinLimits=True, reduceDistanceToUpper=False, reduceDistanceToLower=False,
                                  reduceDistance=False, allAtoms=True, ncores=1):
    """Add one atom's counted distances to dintra/dinter/nintra/ninter in
    place (``Extensions/atomic_distances.pyx:241-324``)."""
    atomIndex = A.int32("atomIndex", atomIndex)
    d = A.array("distances", distances, np.float32, 1)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    for name, arr in (("dintra", dintra), ("dinter", dinter), ("nintra", nintra), ("ninter", ninter)):
        if arr is None:
            raise TypeError("Argument '%s' must not be None" % name)
    di = A.array("dintra", dintra, np.float32, 3)
    de = A.array("dinter", dinter, np.float32, 3)
    ni = A.array("nintra", nintra, np.int32, 3)
    nn = A.array("ninter", ninter, np.int32, 3)
    lo = A.array("lowerLimit", lowerLimit, np.float32, 3)
    up = A.array("upperLimit", upperLimit, np.float32, 3)
    flags = _flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                   reduceDistance)
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n = d.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    ne = di.shape[0]
    for a in (di, de, ni, nn, lo, up):
        if a.shape != (ne, ne, 1):
            raise ValueError("accumulators and limits must have shape (numberOfElements, numberOfElements, 1)")
    if n == 0:
        return None
    call("frmc_single_atomic_distances_dists", atomIndex, ptr(d), n, ptr(mol, I32P), ptr(el, I32P), ne, ptr(di),
         ptr(de), ptr(ni, I32P), ptr(nn, I32P), ptr(lo), ptr(up), flags, int(allAtoms))
    for src, dst in ((di, dintra), (de, dinter), (ni, nintra), (nn, ninter)):
        if src is not dst:
            dst[...] = src
    return None


def single_atomic_distances_dists_serial(atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, nintra,
                                         ninter, lowerLimit, upperLimit, interMolecular=True, intraMolecular=True,
                                         countWithinLimits=True, reduceDistanceToUpper=False,
                                         reduceDistanceToLower=False, reduceDistance=False, allAtoms=True):
    """``Extensions/atomic_distances.pyx:128-238`` (the same computation)."""
    return single_atomic_distances_dists(atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, nintra,
                                         ninter, lowerLimit, upperLimit, interMolecular, intraMolecular,
                                         countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                                         reduceDistance, allAtoms)


def multiple_atomic_distances_coords(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex,
                                     numberOfElements, lowerLimit, upperLimit, interMolecular=True,
                                     intraMolecular=True, countWithinLimits=True, reduceDistanceToUpper=False,
                                     reduceDistanceToLower=False, reduceDistance=False, allAtoms=True, ncores=1):
    """Counted distances of the atoms ``indexes`` against all atoms
    (``Extensions/atomic_distances.pyx:326-417``); returns
    ``(nintra, dintra, ninter, dinter)``, each (ne, ne, 1)."""
    idx = A.array("indexes", indexes, np.int32, 1)
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    B = A.array("basis", basis, np.float32, 2)
    isPBC = A.bint(isPBC)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, lo, up = _limits(numberOfElements, lowerLimit, upperLimit)
    flags = _flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                   reduceDistance)
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n = c.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    ni, di, nn, de = _outputs(ne)
    if idx.shape[0] == 0 or n == 0:
        return ni, di, nn, de
    call("frmc_multiple_atomic_distances_coords", ptr(idx, I32P), idx.shape[0], ptr(c), n, ptr(B), int(isPBC),
         ptr(mol, I32P), ptr(el, I32P), ne, ptr(lo), ptr(up), flags, int(allAtoms), ptr(ni, I32P), ptr(di),
         ptr(nn, I32P), ptr(de))
    return ni, di, nn, de


def multiple_atomic_distances_dists(indexes, distances, moleculeIndex, elementIndex, numberOfElements, lowerLimit,
                                    upperLimit, interMolecular=True, intraMolecular=True, countWithinLimits=True,
                                    reduceDistanceToUpper=False, reduceDistanceToLower=False, reduceDistance=False,
                                    allAtoms=True, ncores=1):
    """The same from a (n, k) distance matrix, column i for atom indexes[i]
    (``Extensions/atomic_distances.pyx:419-498``)."""
    idx = A.array("indexes", indexes, np.int32, 1)
    d = A.array("distances", distances, np.float32, 2)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, lo, up = _limits(numberOfElements, lowerLimit, upperLimit)
    flags = _flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                   reduceDistance)
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n, K = d.shape
    if idx.shape[0] > K:
        raise IndexError("indexes has %d entries, the distance matrix %d columns" % (idx.shape[0], K))
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    ni, di, nn, de = _outputs(ne)
    if idx.shape[0] == 0 or n == 0:
        return ni, di, nn, de
    d = np.ascontiguousarray(d[:, :idx.shape[0]])
    call("frmc_multiple_atomic_distances_dists", ptr(idx, I32P), idx.shape[0], ptr(d), n, ptr(mol, I32P),
         ptr(el, I32P), ne, ptr(lo), ptr(up), flags, int(allAtoms), ptr(ni, I32P), ptr(di), ptr(nn, I32P), ptr(de))
    return ni, di, nn, de


def full_atomic_distances_coords(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, lowerLimit,
                                 upperLimit, interMolecular=True, intraMolecular=True, reduceDistanceToUpper=False,
                                 reduceDistanceToLower=False, reduceDistance=False, countWithinLimits=True,
                                 ncores=1):
    """All pairs i < j (``Extensions/atomic_distances.pyx:500-567``)."""
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    indexes = np.arange(c.shape[0], dtype=NUMPY_INT32)
    return multiple_atomic_distances_coords(indexes=indexes, boxCoords=c, basis=basis, isPBC=isPBC,
                                            moleculeIndex=moleculeIndex, elementIndex=elementIndex,
                                            numberOfElements=numberOfElements, lowerLimit=lowerLimit,
                                            upperLimit=upperLimit, interMolecular=interMolecular,
                                            intraMolecular=intraMolecular, countWithinLimits=countWithinLimits,
                                            reduceDistance=reduceDistance,
                                            reduceDistanceToLower=reduceDistanceToLower,
                                            reduceDistanceToUpper=reduceDistanceToUpper, allAtoms=False,
                                            ncores=ncores)


def full_atomic_distances_dists(distances, moleculeIndex, elementIndex, numberOfElements, lowerLimit, upperLimit,
                                interMolecular=True, intraMolecular=True, reduceDistanceToUpper=False,
                                reduceDistanceToLower=False, reduceDistance=False, countWithinLimits=True):
    """All pairs i < j from a square distance matrix
    (``Extensions/atomic_distances.pyx:569-630``)."""
    d = A.array("distances", distances, np.float32, 2)
    indexes = np.arange(d.shape[1], dtype=NUMPY_INT32)
    return multiple_atomic_distances_dists(indexes=indexes, distances=d, moleculeIndex=moleculeIndex,
                                           elementIndex=elementIndex, numberOfElements=numberOfElements,
                                           lowerLimit=lowerLimit, upperLimit=upperLimit,
                                           interMolecular=interMolecular, intraMolecular=intraMolecular,
                                           countWithinLimits=countWithinLimits, reduceDistance=reduceDistance,
                                           reduceDistanceToLower=reduceDistanceToLower,
                                           reduceDistanceToUpper=reduceDistanceToUpper, allAtoms=False)


def pair_elements_stats(elementIndex, moleculeIndex, numberOfElements):
    """Numbers of atom pairs i < j per element pair, intra- and
    inter-molecular (``Extensions/atomic_distances.pyx:659-672``)."""
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    ne = A.int32("numberOfElements", numberOfElements)
    n = el.shape[0]
    A.need_len("moleculeIndex", mol, n)
    ni = np.zeros((ne, ne, 1), NUMPY_INT32)
    nn = np.zeros((ne, ne, 1), NUMPY_INT32)
    if n < 2 or ne == 0:
        return ni, nn
    call("frmc_pair_elements_stats", ptr(el, I32P), ptr(mol, I32P), n, ne, ptr(ni, I32P), ptr(nn, I32P))
    return ni, nn
