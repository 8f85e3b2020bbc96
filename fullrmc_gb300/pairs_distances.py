"""Drop-in replacement of ``fullrmc.Core.pairs_distances`` on the GPU.

Same names, positional order, keyword names, defaults and return conventions
as ``Extensions/pairs_distances.pyx``; results are bit-identical to the
reference's float32 arithmetic.  ``ncores`` is accepted and ignored.

As in the reference, ``pairs_*_to_multi_points`` read point k as
``points[:, k]`` (so ``points`` is (3, k) in practice) and the outputs that
skip rows (``allAtoms=False``) leave those rows uninitialised.
"""
from __future__ import annotations

import numpy as np

from . import _args as A
from ._native import F32P, I32P, call, ptr

NUMPY_FLOAT32 = np.float32
NUMPY_INT32 = np.int32


def _common(coords, basis, isPBC, ncores):
    c = A.array("coords", coords, np.float32, 2)
    B = A.memview("basis", basis, np.float32, 2)
    A.int32("ncores", ncores)
    return c, B, int(A.bint(isPBC))


def _points(points):
    p = A.array("points", points, np.float32, 2)
    if p.shape[0] < 3:
        raise ValueError("points must hold 3 rows (x, y, z) of k points")
    return p


def _point(name, point):
    p = A.array(name, point, np.float32, 1)
    if p.shape[0] < 3:
        raise ValueError("%s must hold 3 components" % name)
    return p


# ------------------------------------------------------------ differences
def from_to_points_differences(pointsFrom, pointsTo, basis, isPBC, ncores=1):
    """differences[i] = bc(pointsTo[i] - pointsFrom[i]) (``pairs_distances.pyx:483-521``)."""
    a = A.array("pointsFrom", pointsFrom, np.float32, 2)
    b = A.array("pointsTo", pointsTo, np.float32, 2)
    B = A.memview("basis", basis, np.float32, 2)
    A.int32("ncores", ncores)
    n = a.shape[0]
    if b.shape[0] < n:
        raise ValueError("pointsTo has fewer points than pointsFrom")
    out = np.empty((n, 3), dtype=NUMPY_FLOAT32)
    if n:
        call("frmc_from_to_points_differences", ptr(a), ptr(b), n, ptr(B), int(A.bint(isPBC)), ptr(out))
    return out


def pair_difference_to_point(point1, point2, basis, isPBC, ncores=1):
    """difference = bc(point2 - point1) (``pairs_distances.pyx:529-561``)."""
    p1, p2 = _point("point1", point1), _point("point2", point2)
    B = A.memview("basis", basis, np.float32, 2)
    A.int32("ncores", ncores)
    out = np.empty((3,), dtype=NUMPY_FLOAT32)
    call("frmc_pair_difference_to_point", ptr(p1), ptr(p2), ptr(B), int(A.bint(isPBC)), ptr(out))
    return out


def pairs_differences_to_point(point, coords, basis, isPBC, ncores=1):
    """differences[i] = bc(point - coords[i]) (``pairs_distances.pyx:569-607``)."""
    p = _point("point", point)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0], 3), dtype=NUMPY_FLOAT32)
    if c.shape[0]:
        call("frmc_pairs_differences_to_point", ptr(p), ptr(c), c.shape[0], ptr(B), pbc, ptr(out))
    return out


def pairs_differences_to_indexcoords(atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1):
    """differences[i] = bc(coords[atomIndex] - coords[i]) (``pairs_distances.pyx:615-654``)."""
    atomIndex = A.int32("atomIndex", atomIndex)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0], 3), dtype=NUMPY_FLOAT32)
    if c.shape[0]:
        call("frmc_pairs_differences_to_indexcoords", atomIndex, ptr(c), c.shape[0], ptr(B), pbc,
             int(A.bint(allAtoms)), ptr(out))
    return out


def pairs_differences_to_multi_points(points, coords, basis, isPBC, ncores=1):
    """differences[i, :, k] = bc(points[:, k] - coords[i]) (``pairs_distances.pyx:662-711``)."""
    p = _points(points)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    k = p.shape[1]
    out = np.empty((c.shape[0], 3, k), dtype=NUMPY_FLOAT32)
    if c.shape[0] and k:
        call("frmc_pairs_differences_to_multi_points", ptr(p), p.shape[1], k, ptr(c), c.shape[0], ptr(B), pbc,
             ptr(out))
    return out


def pairs_differences_to_multi_indexcoords(indexes, coords, basis, isPBC, allAtoms=True, ncores=1):
    """differences[i, :, k] = bc(coords[indexes[k]] - coords[i]) (``pairs_distances.pyx:719-774``)."""
    idx = A.array("indexes", indexes, np.int32, 1)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0], 3, idx.shape[0]), dtype=NUMPY_FLOAT32)
    if c.shape[0] and idx.shape[0]:
        call("frmc_pairs_differences_to_multi_indexcoords", ptr(idx, I32P), idx.shape[0], ptr(c), c.shape[0],
             ptr(B), pbc, int(A.bint(allAtoms)), ptr(out))
    return out


# -------------------------------------------------------------- distances
def point_to_point_distance(point1, point2, basis, isPBC, ncores=1):
    """Distance between two points (``pairs_distances.pyx:786-819``)."""
    p1, p2 = _point("point1", point1), _point("point2", point2)
    B = A.memview("basis", basis, np.float32, 2)
    A.int32("ncores", ncores)
    out = np.empty((1,), dtype=NUMPY_FLOAT32)
    call("frmc_point_to_point_distance", ptr(p1), ptr(p2), ptr(B), int(A.bint(isPBC)), ptr(out))
    return float(out[0])


def pairs_distances_to_point(point, coords, basis, isPBC, ncores=1):
    """distances[i] = |bc(point - coords[i])| (``pairs_distances.pyx:827-866``)."""
    p = _point("point", point)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0],), dtype=NUMPY_FLOAT32)
    if c.shape[0]:
        call("frmc_pairs_distances_to_point", ptr(p), ptr(c), c.shape[0], ptr(B), pbc, ptr(out))
    return out


def pairs_distances_to_indexcoords(atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1):
    """distances[i] = |bc(coords[atomIndex] - coords[i])| (``pairs_distances.pyx:874-916``)."""
    atomIndex = A.int32("atomIndex", atomIndex)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0],), dtype=NUMPY_FLOAT32)
    if c.shape[0]:
        call("frmc_pairs_distances_to_indexcoords", atomIndex, ptr(c), c.shape[0], ptr(B), pbc,
             int(A.bint(allAtoms)), ptr(out))
    return out


def pairs_distances_to_multi_points(points, coords, basis, isPBC, ncores=1):
    """distances[i, k] = |bc(points[:, k] - coords[i])| (``pairs_distances.pyx:924-966``)."""
    p = _points(points)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    k = p.shape[1]
    out = np.empty((c.shape[0], k), dtype=NUMPY_FLOAT32)
    if c.shape[0] and k:
        call("frmc_pairs_distances_to_multi_points", ptr(p), p.shape[1], k, ptr(c), c.shape[0], ptr(B), pbc,
             ptr(out))
    return out


def pairs_distances_to_multi_indexcoords(indexes, coords, basis, isPBC, allAtoms=True, ncores=1):
    """distances[i, k] = |bc(coords[indexes[k]] - coords[i])| (``pairs_distances.pyx:975-1021``)."""
    idx = A.array("indexes", indexes, np.int32, 1)
    c, B, pbc = _common(coords, basis, isPBC, ncores)
    out = np.empty((c.shape[0], idx.shape[0]), dtype=NUMPY_FLOAT32)
    if c.shape[0] and idx.shape[0]:
        call("frmc_pairs_distances_to_multi_indexcoords", ptr(idx, I32P), idx.shape[0], ptr(c), c.shape[0], ptr(B),
             pbc, int(A.bint(allAtoms)), ptr(out))
    return out
