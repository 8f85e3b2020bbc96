"""fullrmc's ShapeFunction on the GPU, in FP64.

``Constraints/Collection.py:15-160`` builds a StructureFactorConstraint over
(rmin, rmax, dr) with Q = arange(qmin, qmax, dq), computes its data (the
all-pairs histogram, ``StructureFactorConstraints.py:933-960``), its total
S(q) (``:836-896``: g(r) from the weighted element-pair counts, G(r) =
4 pi r rho0 (g(r) - 1), S(q) = 1 + sum_r G(r) dr sin(q r) / q) and transforms
S(q) back to r (``Collection.py:131-139``: G(r) = 2/pi sum_q q (S(q) - 1) dq
sin(q r)).  PairDistributionConstraint subtracts that curve from its model and
recomputes it every ``updateFreq`` accepted moves
(``PairDistributionConstraints.py:316-343, 363-375``).

Here the whole chain is one call of ``frmc_shape_function``: the all-pairs
counts on the GPU (the tiled all-pairs kernel), then G, S and the shape
function in FP64 on the device.  The grids follow the reference's float32
construction exactly (Q and the histogram edges are float32 arrays built the
same way); the arithmetic after the counts is FP64 with exact counts, where
the reference works in float32 and its float32 histogram stops counting at
2^24 per bin.

The element weights come from pdbparser's element tables in fullrmc
(``get_real_elements_weight``, ``Core/Collection.py:91-120``), which are not
available here: pass them as ``weights`` (element name -> weight, or one
weight per element index); they are normalised with
``engine.normalized_weighting`` (w_ij = (2 - delta_ij) c_i c_j b_i b_j /
(sum_k c_k b_k)^2).
"""
from __future__ import annotations

import numpy as np

from ._native import F32P, F64P, I32P, call, ptr
from .engine import normalized_weighting

F32 = np.float32


def shape_function_grids(qmin=0.001, qmax=1.0, dq=0.005, rmin=0.0, rmax=100.0, dr=1.0):
    """(Q, edges, shellCenters, minDistance, maxDistance, bin, histSize) as the
    reference builds them: Q = arange(qmin, qmax, dq) cast to float32
    (``Collection.py:64-75``); edges = arange(rmin, rmax + dr, dr) cast to
    float32 with float32 rmin, rmax, dr (``StructureFactorConstraints.py:
    502-575, 336-350``), centers = (e[:-1] + e[1:]) / 2 in float32."""
    qmin, qmax, dq = F32(qmin), F32(qmax), F32(dq)
    if not (qmin > 0 and qmax > qmin and dq > 0):
        raise ValueError("need 0 < qmin < qmax and dq > 0")
    Q = np.arange(qmin, qmax, dq).astype(F32)
    mn, mx, b = F32(rmin), F32(rmax), F32(dr)
    if not (mx > mn and b > 0):
        raise ValueError("need rmin < rmax and dr > 0")
    edges = np.arange(mn, F32(mx + b), b).astype(F32)
    centers = ((edges[:-1] + edges[1:]) / F32(2.0)).astype(F32)
    return Q, edges, centers, F32(edges[0]), F32(edges[-1]), b, int(len(edges) - 1)


def _pair_terms(elements_count, weights, volume):
    """Element pairs i <= j with coef = w_ij V / N_ij
    (``StructureFactorConstraints.py:853-872``)."""
    n = np.asarray(elements_count, np.float64)
    w = normalized_weighting(n, weights)
    pi, pj, pc = [], [], []
    for i in range(len(n)):
        for j in range(i, len(n)):
            Nij = n[i] * (n[i] - 1.0) / 2.0 if i == j else n[i] * n[j]
            if Nij == 0.0:
                continue
            pi.append(i)
            pj.append(j)
            pc.append(w[i, j] * float(volume) / Nij)
    return (np.array(pi, np.int32), np.array(pj, np.int32), np.array(pc, np.float64))


def gr_shape_function(boxCoords, basis, isPBC, moleculeIndex, elementIndex, elementsCount, weights, volume, rValues,
                      qmin=0.001, qmax=1.0, dq=0.005, rmin=0.0, rmax=100.0, dr=1.0, details=False):
    """The G(r) shape function on rValues (FP64).  With details=True also
    returns the StructureFactorConstraint's G (on its shell centers) and S(q)
    (on Q): (Gshape, {"Q", "shellCenters", "Gr", "Sq"})."""
    c = np.ascontiguousarray(boxCoords, F32)
    if c.ndim != 2 or c.shape[1] != 3:
        raise ValueError("boxCoords must be (n, 3) float32")
    B = np.ascontiguousarray(basis, F32).reshape(3, 3)
    n = c.shape[0]
    mol = np.ascontiguousarray(moleculeIndex, np.int32)
    el = np.ascontiguousarray(elementIndex, np.int32)
    if mol.shape[0] < n or el.shape[0] < n:
        raise ValueError("moleculeIndex and elementIndex need one entry per atom")
    counts = np.asarray(elementsCount, np.float64)
    ne = len(counts)
    Q, edges, centers, mn, mx, b, hs = shape_function_grids(qmin, qmax, dq, rmin, rmax, dr)
    e64 = edges.astype(np.float64)
    vol = 4.0 / 3.0 * np.pi * (e64[1:] ** 3 - e64[:-1] ** 3)
    pi, pj, pc = _pair_terms(counts, weights, volume)
    rho0 = float(n) / float(volume)
    r = np.ascontiguousarray(rValues, np.float64).reshape(-1)
    q64 = Q.astype(np.float64)
    c64 = centers.astype(np.float64)
    G = np.empty(hs, np.float64)
    S = np.empty(len(Q), np.float64)
    Gs = np.empty(len(r), np.float64)
    call("frmc_shape_function", ptr(c), n, ptr(B), int(bool(isPBC)), ptr(mol, I32P), ptr(el, I32P), ne, mn, mx, b,
         hs, len(pi), ptr(pi, I32P), ptr(pj, I32P), ptr(pc, F64P), ptr(c64, F64P), ptr(vol, F64P), rho0,
         ptr(q64, F64P), len(Q), ptr(r, F64P), len(r), ptr(G, F64P), ptr(S, F64P), ptr(Gs, F64P))
    if details:
        return Gs, {"Q": Q, "shellCenters": centers, "Gr": G, "Sq": S}
    return Gs


class ShapeFunction:
    """GPU counterpart of fullrmc's ShapeFunction (``Constraints/Collection.py:
    15-160``) with the same grid parameters and methods.  ``engine`` is a
    fullrmc Engine or any object with its attributes boxCoordinates,
    basisVectors, isPBC, moleculesIndex, elementsIndex, elements,
    numberOfAtomsPerElement and volume; ``weights`` gives each element's
    scattering weight (a dict by element name or a sequence by element
    index)."""

    def __init__(self, engine, weights, qmin=0.001, qmax=1, dq=0.005, rmin=0.00, rmax=100, dr=1):
        self.engine = engine
        self._grid = (qmin, qmax, dq, rmin, rmax, dr)
        Q, edges, centers, _, _, _, hs = shape_function_grids(qmin, qmax, dq, rmin, rmax, dr)
        self.qValues, self.edges, self.shellCenters, self.histogramSize = Q, edges, centers, hs
        self._weights = weights
        self.Gr = self.Sq = None

    def _system(self):
        e = self.engine
        elements = list(getattr(e, "elements", range(len(np.atleast_1d(self._weights)))))
        per = getattr(e, "numberOfAtomsPerElement")
        counts = [per[x] for x in elements] if isinstance(per, dict) else list(per)
        w = self._weights
        b = [w[x] for x in elements] if isinstance(w, dict) else list(w)
        return counts, b

    def get_Gr_shape_function(self, rValues, compute=True):
        """Shape function of G(r) on rValues (Collection.py:141-152).  The
        histogram is always recomputed (compute=False is accepted)."""
        e = self.engine
        counts, b = self._system()
        Gs, info = gr_shape_function(e.boxCoordinates, e.basisVectors, e.isPBC, e.moleculesIndex, e.elementsIndex,
                                     counts, b, e.volume, rValues, *self._grid, details=True)
        self.Gr, self.Sq = info["Gr"], info["Sq"]
        return Gs

    def get_gr_shape_function(self, rValues, compute=True):
        """Shape function of g(r): G / (4 pi rho0 r) (Collection.py:154-160)."""
        Gs = self.get_Gr_shape_function(rValues, compute)
        rho0 = float(np.asarray(self.engine.boxCoordinates).shape[0]) / float(self.engine.volume)
        return Gs / (4.0 * np.pi * rho0 * np.asarray(rValues, np.float64))
