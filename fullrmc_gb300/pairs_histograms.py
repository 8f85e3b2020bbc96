"""Drop-in replacement of ``fullrmc.Core.pairs_histograms`` on the GPU.

Same function names, positional order, keyword names, defaults and return
conventions as ``Extensions/pairs_histograms.pyx``; the work runs in
``libfrmc_gpu.so`` on the current CUDA device and the float32 histograms are
bit-identical to the reference's ``ncores=1`` results.  ``ncores`` is accepted
and ignored (it only selected OpenMP threads in the reference).
"""
from __future__ import annotations

import numpy as np

from . import _args as A
from ._native import F32P, I32P, call, check, fastcall, ptr

NUMPY_FLOAT32 = np.float32
NUMPY_INT32 = np.int32


def _hist_shape(numberOfElements, histSize):
    ne = A.int32("numberOfElements", numberOfElements)
    hs = A.int32("histSize", histSize)
    if ne < 0 or hs < 0:
        raise ValueError("negative dimensions are not allowed")
    return ne, hs


def single_pairs_histograms(atomIndex, distances, moleculeIndex, elementIndex, hintra, hinter,
                            minDistance, maxDistance, bin, allAtoms=True, ncores=1):
    """Add the histogram of one atom's distance row to hintra/hinter in place
    (``Extensions/pairs_histograms.pyx:77-141``)."""
    atomIndex = A.int32("atomIndex", atomIndex)
    d = A.array("distances", distances, np.float32, 1)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    if hintra is None or hinter is None:
        raise TypeError("Argument '%s' must not be None" % ("hintra" if hintra is None else "hinter"))
    hi = A.array("hintra", hintra, np.float32, 3)
    he = A.array("hinter", hinter, np.float32, 3)
    minDistance, maxDistance, bin = (A.float32("minDistance", minDistance), A.float32("maxDistance", maxDistance),
                                     A.float32("bin", bin))
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n = d.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    if hi.shape != he.shape or hi.shape[0] != hi.shape[1]:
        raise ValueError("hintra and hinter must both have shape (ne, ne, hs)")
    ne, hs = hi.shape[0], hi.shape[2]
    if n == 0:
        return None
    call("frmc_single_pairs_histograms", atomIndex, ptr(d), n, ptr(mol, I32P), ptr(el, I32P), ne, hs, ptr(hi),
         ptr(he), minDistance, maxDistance, bin, int(allAtoms))
    if hi is not hintra:
        hintra[...] = hi
    if he is not hinter:
        hinter[...] = he
    return None


def multiple_pairs_histograms_coords(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex,
                                     numberOfElements, minDistance, maxDistance, bin, histSize,
                                     allAtoms=True, ncores=1):
    """Histograms of the atoms ``indexes`` against all atoms
    (``Extensions/pairs_histograms.pyx:150-217``).  Returns (hintra, hinter)."""
    fast = fastcall()
    if fast is not None:
        r = fast.multiple(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                          minDistance, maxDistance, bin, histSize, allAtoms, ncores)
        if r is not None:
            if type(r) is int:
                check(r)
            return r
    idx = A.array("indexes", indexes, np.int32, 1)
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    B = A.array("basis", basis, np.float32, 2)
    isPBC = A.bint(isPBC)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, hs = _hist_shape(numberOfElements, histSize)
    minDistance, maxDistance, bin = (A.float32("minDistance", minDistance), A.float32("maxDistance", maxDistance),
                                     A.float32("bin", bin))
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n = c.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    hintra = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    hinter = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    if idx.shape[0] == 0 or n == 0 or hintra.size == 0:
        return hintra, hinter
    call("frmc_multiple_pairs_histograms_coords", ptr(idx, I32P), idx.shape[0], ptr(c), n, ptr(B), int(isPBC),
         ptr(mol, I32P), ptr(el, I32P), ne, minDistance, maxDistance, bin, hs, int(allAtoms), ptr(hintra),
         ptr(hinter))
    return hintra, hinter


def group_move_delta_histograms(indexes, boxCoords, newBoxCoords, basis, isPBC, moleculeIndex, elementIndex,
                                numberOfElements, minDistance, maxDistance, bin, histSize):
    """The change of a PairDistributionConstraint's data for moving the atoms
    ``indexes`` from their rows of ``boxCoords`` to ``newBoxCoords`` (one row
    per index, same order), in one device launch: (M - F) after minus (M - F)
    before, M = multiple_pairs_histograms_coords(indexes, ..., allAtoms=True)
    and F = full_pairs_histograms_coords on the group alone, which is what
    ``compute_before_move`` and ``compute_after_move`` subtract and add
    (``Constraints/PairDistributionConstraints.py:1044-1129``).  Returns
    (dintra, dinter), int32 (ne, ne, hs), equal to the differences of the four
    reference histograms.  An extension of this module (at most 1024 moved
    atoms); fullrmc's constraints keep calling the reference functions."""
    idx = A.array("indexes", indexes, np.int32, 1)
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    nc = A.array("newBoxCoords", newBoxCoords, np.float32, 2)
    B = A.array("basis", basis, np.float32, 2)
    isPBC = A.bint(isPBC)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, hs = _hist_shape(numberOfElements, histSize)
    minDistance, maxDistance, bin = (A.float32("minDistance", minDistance), A.float32("maxDistance", maxDistance),
                                     A.float32("bin", bin))
    n = c.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    if nc.shape != (idx.shape[0], 3):
        raise ValueError("newBoxCoords must be (%d, 3), one row per index" % idx.shape[0])
    dintra = np.zeros((ne, ne, hs), dtype=np.int32)
    dinter = np.zeros((ne, ne, hs), dtype=np.int32)
    if idx.shape[0] == 0 or n == 0 or dintra.size == 0:
        return dintra, dinter
    call("frmc_group_move_delta_histograms", ptr(idx, I32P), idx.shape[0], ptr(c), n, ptr(nc), ptr(B), int(isPBC),
         ptr(mol, I32P), ptr(el, I32P), ne, minDistance, maxDistance, bin, hs, ptr(dintra, I32P), ptr(dinter, I32P))
    return dintra, dinter


def multiple_pairs_histograms_dists(indexes, distances, moleculeIndex, elementIndex, numberOfElements,
                                    minDistance, maxDistance, bin, histSize, allAtoms=True, ncores=1):
    """Histograms from a (n, k) distance matrix whose column i belongs to atom
    indexes[i] (``Extensions/pairs_histograms.pyx:225-281``)."""
    idx = A.array("indexes", indexes, np.int32, 1)
    d = A.array("distances", distances, np.float32, 2)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, hs = _hist_shape(numberOfElements, histSize)
    minDistance, maxDistance, bin = (A.float32("minDistance", minDistance), A.float32("maxDistance", maxDistance),
                                     A.float32("bin", bin))
    allAtoms = A.bint(allAtoms)
    A.int32("ncores", ncores)
    n, k = d.shape[0], idx.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    if d.shape[1] < k:
        raise ValueError("distances has %d columns for %d indexes" % (d.shape[1], k))
    hintra = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    hinter = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    if k == 0 or n == 0 or hintra.size == 0:
        return hintra, hinter
    dk = d if d.shape[1] == k else np.ascontiguousarray(d[:, :k])
    call("frmc_multiple_pairs_histograms_dists", ptr(idx, I32P), k, ptr(dk), n, ptr(mol, I32P), ptr(el, I32P), ne,
         minDistance, maxDistance, bin, hs, int(allAtoms), ptr(hintra), ptr(hinter))
    return hintra, hinter


def full_pairs_histograms_coords(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                                 minDistance, maxDistance, bin, histSize, ncores=1):
    """All-pairs (i < j) histograms (``Extensions/pairs_histograms.pyx:289-335``)."""
    fast = fastcall()
    if fast is not None:
        r = fast.full(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, minDistance,
                      maxDistance, bin, histSize, ncores)
        if r is not None:
            if type(r) is int:
                check(r)
            return r
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    B = A.array("basis", basis, np.float32, 2)
    isPBC = A.bint(isPBC)
    mol = A.array("moleculeIndex", moleculeIndex, np.int32, 1)
    el = A.array("elementIndex", elementIndex, np.int32, 1)
    ne, hs = _hist_shape(numberOfElements, histSize)
    minDistance, maxDistance, bin = (A.float32("minDistance", minDistance), A.float32("maxDistance", maxDistance),
                                     A.float32("bin", bin))
    A.int32("ncores", ncores)
    n = c.shape[0]
    A.need_len("moleculeIndex", mol, n)
    A.need_len("elementIndex", el, n)
    hintra = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    hinter = np.zeros((ne, ne, hs), dtype=NUMPY_FLOAT32)
    if n < 2 or hintra.size == 0:
        return hintra, hinter
    call("frmc_full_pairs_histograms_coords", ptr(c), n, ptr(B), int(isPBC), ptr(mol, I32P), ptr(el, I32P), ne,
         minDistance, maxDistance, bin, hs, ptr(hintra), ptr(hinter))
    return hintra, hinter


def full_pairs_histograms_dists(distances, moleculeIndex, elementIndex, numberOfElements, minDistance,
                                maxDistance, bin, histSize, ncores=1):
    """All-pairs histograms from a square distance matrix
    (``Extensions/pairs_histograms.pyx:343-383``)."""
    d = A.array("distances", distances, np.float32, 2)
    indexes = np.arange(d.shape[1], dtype=NUMPY_INT32)
    return multiple_pairs_histograms_dists(indexes=indexes, distances=d, moleculeIndex=moleculeIndex,
                                           elementIndex=elementIndex, numberOfElements=numberOfElements,
                                           minDistance=minDistance, maxDistance=maxDistance, histSize=histSize,
                                           bin=bin, allAtoms=False, ncores=ncores)
