"""Drop-in replacement of ``fullrmc.Core.reciprocal_space`` with FP64 transforms.

Same names and arguments as ``Extensions/reciprocal_space.pyx``.  The sums
are evaluated in double precision on the GPU and returned as float64 arrays
(the reference returns float32 accumulated in float32).  ``sq_to_Gr``
computes the transform its docstring describes; the reference's own body
(``reciprocal_space.pyx:143``) passes an array to libc ``sin`` and raises
``TypeError`` for every input.
"""
from __future__ import annotations

import numpy as np

from . import _args as A
from ._native import F64P, call, ptr

NUMPY_FLOAT32 = np.float32


def _grid(name, a, min_len=2):
    a = A.array(name, a, np.float32, 1)
    if a.shape[0] < min_len:
        raise ValueError("%s needs at least %d points" % (name, min_len))
    return a


def gr_to_sq(distances, gr, qrange, rho):
    """S(q) = 1 + 4 pi rho / q sum_r dr r (g(r) - 1) sin(q r) (``reciprocal_space.pyx:42-73``)."""
    r = _grid("distances", distances)
    g = A.array("gr", gr, np.float32, 1)
    q = A.array("qrange", qrange, np.float32, 1)
    rho = float(A.float32("rho", rho))
    if g.shape[0] < r.shape[0]:
        raise ValueError("gr is shorter than distances")
    out = np.empty((q.shape[0],), dtype=np.float64)
    if q.shape[0]:
        call("frmc_gr_to_sq", ptr(r), ptr(g), r.shape[0], ptr(q), q.shape[0], rho, ptr(out, F64P))
    return out


def Gr_to_sq(distances, Gr, qrange):
    """S(q) = 1 + 1/q sum_r dr G(r) sin(q r) (``reciprocal_space.pyx:82-109``)."""
    r = _grid("distances", distances)
    G = A.array("Gr", Gr, np.float32, 1)
    q = A.array("qrange", qrange, np.float32, 1)
    if G.shape[0] < r.shape[0]:
        raise ValueError("Gr is shorter than distances")
    out = np.empty((q.shape[0],), dtype=np.float64)
    if q.shape[0]:
        call("frmc_Gr_to_sq", ptr(r), ptr(G), r.shape[0], ptr(q), q.shape[0], ptr(out, F64P))
    return out


def sq_to_Gr(qValues, rValues, sq):
    """G(r) = 2/pi sum_q dq q (S(q) - 1) sin(q r) (``reciprocal_space.pyx:118-145``)."""
    q = _grid("qValues", qValues)
    r = A.array("rValues", rValues, np.float32, 1)
    s = A.array("sq", sq, np.float32, 1)
    if s.shape[0] < q.shape[0]:
        raise ValueError("sq is shorter than qValues")
    out = np.empty((r.shape[0],), dtype=np.float64)
    if r.shape[0]:
        call("frmc_sq_to_Gr", ptr(q), q.shape[0], ptr(r), r.shape[0], ptr(s), ptr(out, F64P))
    return out
