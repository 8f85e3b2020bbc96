"""Drop-in replacement of ``fullrmc.Core.boundary_conditions_collection``.

``transform_coordinates`` (``Extensions/boundary_conditions_collection.pyx:88-110``)
is the per-move real-to-box conversion fullrmc's Engine calls
(``Engine.py:3223``); it runs on the GPU with the reference's float32 order.
``box_coordinates_real_distances`` (``:119-163``) maps onto the GPU distance
kernel (the pair distance is symmetric bit-for-bit).  ``get_reciprocal_basis``
(``:45-80``) is a 3x3 set-up helper that fullrmc never calls; it is
reproduced on the host as written, including its ``rbasis[0,1]`` term, which
reuses ``basis[0,1]`` where the cofactor would use ``basis[0,2]``.
"""
from __future__ import annotations

import numpy as np

from . import _args as A
from ._native import call, check, fastcall, ptr

NUMPY_FLOAT32 = np.float32


def get_reciprocal_basis(basis):
    """(rbasis, vol) exactly as ``boundary_conditions_collection.pyx:45-80`` computes them."""
    b = A.array("basis", basis, np.float32, 2).astype(np.float32)
    f = np.float32
    r = np.empty((3, 3), dtype=np.float32)
    r[0, 0] = f(b[1, 1] * b[2, 2]) - f(b[2, 1] * b[1, 2])
    r[0, 1] = -(f(b[0, 1] * b[2, 2]) - f(b[2, 1] * b[0, 1]))
    r[0, 2] = f(b[0, 1] * b[1, 2]) - f(b[1, 1] * b[0, 2])
    r[1, 0] = -(f(b[1, 0] * b[2, 2]) - f(b[2, 0] * b[1, 2]))
    r[1, 1] = f(b[0, 0] * b[2, 2]) - f(b[2, 0] * b[0, 2])
    r[1, 2] = -(f(b[0, 0] * b[1, 2]) - f(b[1, 0] * b[0, 2]))
    r[2, 0] = f(b[1, 0] * b[2, 1]) - f(b[2, 0] * b[1, 1])
    r[2, 1] = -(f(b[0, 0] * b[2, 1]) - f(b[2, 0] * b[0, 1]))
    r[2, 2] = f(b[0, 0] * b[1, 1]) - f(b[1, 0] * b[0, 1])
    vol = f(f(f(b[0, 0] * r[0, 0]) + f(b[1, 0] * r[0, 1])) + f(b[2, 0] * r[0, 2]))
    # vol is a Python float in the reference; the division runs in double and
    # is rounded back to float32 (identical to a float32 division).
    r = (r.astype(np.float64) / float(vol)).astype(np.float32)
    return r, float(vol)


def transform_coordinates(transMatrix, coords):
    """transCoords[i] = coords[i] . transMatrix (``boundary_conditions_collection.pyx:88-110``)."""
    fast = fastcall()
    if fast is not None:
        r = fast.transform(transMatrix, coords)
        if r is not None:
            if type(r) is int:
                check(r)
            return r
    M = A.array("transMatrix", transMatrix, np.float32, 2)
    c = A.array("coords", coords, np.float32, 2)
    out = np.empty((c.shape[0], 3), dtype=NUMPY_FLOAT32)
    if c.shape[0]:
        call("frmc_transform_coordinates", ptr(M), ptr(c), c.shape[0], ptr(out))
    return out


def box_coordinates_real_distances(atomIndex, indexes, boxCoords, basis):
    """distances[k] = |bc(boxCoords[indexes[k]] - boxCoords[atomIndex])| (``:119-163``)."""
    atomIndex = A.int32("atomIndex", atomIndex)
    idx = A.array("indexes", indexes, np.int32, 1)
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    B = A.array("basis", basis, np.float32, 2)
    if not 0 <= atomIndex < c.shape[0] or (idx.size and (idx.min() < 0 or idx.max() >= c.shape[0])):
        raise IndexError("index out of range")
    sub = np.ascontiguousarray(c[idx])
    out = np.empty((idx.shape[0],), dtype=NUMPY_FLOAT32)
    if idx.shape[0]:
        point = np.ascontiguousarray(c[atomIndex])
        call("frmc_pairs_distances_to_point", ptr(point), ptr(sub), sub.shape[0], ptr(B), 1, ptr(out))
    return out
