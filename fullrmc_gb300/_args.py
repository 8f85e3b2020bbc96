"""Argument coercion that mirrors the reference's Cython signatures.

fullrmc's entry points are typed ``ndarray[C_FLOAT32, ndim=2] x not None``,
``C_INT32`` scalars, ``C_FLOAT32`` scalars and ``bint`` flags
(e.g. ``Extensions/pairs_histograms.pyx:150-162``).  Cython then raises
``TypeError`` for ``None`` or a non-array, ``ValueError`` for a wrong dtype or
number of dimensions, ``TypeError`` when a float is passed for an integer,
and ``OverflowError`` when an integer does not fit in int32.  These helpers
raise the same exception types.
"""
from __future__ import annotations

import operator

import numpy as np

_CNAME = {np.dtype(np.float32): "C_FLOAT32", np.dtype(np.int32): "C_INT32"}


def array(name, a, dtype, ndim, allow_none=False):
    """A C-contiguous view/copy of an ndarray argument after the reference's checks."""
    if a is None:
        if allow_none:
            return None
        raise TypeError("Argument '%s' must not be None" % name)
    if not isinstance(a, np.ndarray):
        raise TypeError("Argument '%s' has incorrect type (expected numpy.ndarray, got %s)"
                        % (name, type(a).__name__))
    if a.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d)" % (ndim, a.ndim))
    dt = np.dtype(dtype)
    if a.dtype != dt:
        raise ValueError("Buffer dtype mismatch, expected '%s' but got '%s'" % (_CNAME.get(dt, dt.name), a.dtype.name))
    return np.ascontiguousarray(a)


def memview(name, a, dtype, ndim):
    """A typed memoryview argument (``C_FLOAT32[:,:] basis not None``)."""
    if a is None:
        raise TypeError("Argument '%s' must not be None" % name)
    try:
        arr = np.asarray(a)
    except Exception as exc:  # pragma: no cover - mirrors the buffer protocol failure
        raise TypeError(str(exc))
    if arr.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d)" % (ndim, arr.ndim))
    dt = np.dtype(dtype)
    if arr.dtype != dt:
        raise ValueError("Buffer dtype mismatch, expected '%s' but got '%s'" % (_CNAME.get(dt, dt.name), arr.dtype.name))
    return np.ascontiguousarray(arr)


def int32(name, v):
    if isinstance(v, (float, np.floating)):
        raise TypeError("'%s' object cannot be interpreted as an integer" % type(v).__name__)
    v = operator.index(v)
    if v < -2 ** 31 or v >= 2 ** 31:
        raise OverflowError("value too large to convert to int")
    return int(v)


def float32(name, v):
    if v is None:
        raise TypeError("must be real number, not NoneType")
    return np.float32(float(v))


def bint(v):
    return bool(v)


def need_len(name, a, n):
    if a.shape[0] < n:
        raise ValueError("'%s' has %d entries, fewer than the %d atoms" % (name, a.shape[0], n))
