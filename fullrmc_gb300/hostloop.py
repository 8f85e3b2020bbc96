"""A host-side RMC chain that drives the histogram path the way fullrmc does.

This is fullrmc's plain step with a PairDistributionConstraint, restated so
that it can run against any module with the ``pairs_histograms`` /
``boundary_conditions_collection`` interface -- the GPU drop-in of this
package, or fullrmc's own Cython:

* ``compute_data``: ``full_pairs_histograms_coords`` on all atoms
  (``Constraints/PairDistributionConstraints.py:1000-1042``);
* one step: ``compute_before_move`` = M - F with M =
  ``multiple_pairs_histograms_coords(allAtoms=True)`` on the group and F =
  ``full_pairs_histograms_coords`` on the group's coordinates (``:1044-1079``);
  ``compute_after_move`` repeats both with the moved coordinates written into
  the coordinate array (``:1081-1129``); new data = data - before + after;
* G(r) in float32 in the reference's operation order (``:847-895``), the
  standard error ``np.add.reduce((exp - G)**2)`` (``:810-838``) divided by
  varianceSquared, and fullrmc's acceptance rule: reject iff the new error is
  larger and ``u > tolerance`` (``Engine.py:3300-3317``).
* the moved box coordinates are ``transform_coordinates(reciprocalBasis,
  real + v)`` (``Engine.py:3222-3223``).

Because the float32 host math is identical whichever module supplies the
histograms, two chains fed the same moves accept and reject identically
exactly when the histogram modules agree bit for bit.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
PI = F32(np.pi)


class HostPDFChain:
    def __init__(self, system, hist_module, transform_module=None, weights=None):
        """`weights`: float32 element-pair weights w[i][j] to use instead of
        the system model's (e.g. those a fullrmc constraint computed)."""
        self.h = hist_module
        self.t = transform_module
        s = system
        m = s.model
        self.box = np.array(s.box_coords, F32, copy=True)
        self.real = np.array(s.real_coords, F32, copy=True)
        self.el = np.ascontiguousarray(s.el, np.int32)
        self.mol = np.ascontiguousarray(s.mol, np.int32)
        self.basis = np.ascontiguousarray(s.basis, F32)
        self.rbasis = np.ascontiguousarray(s.rbasis, F32)
        self.isPBC = bool(s.isPBC)
        self.tolerance = F32(s.tolerance)
        self.ne = len(m.elements_count)
        self.counts = [int(c) for c in m.elements_count]
        self.hs = int(m.hs)
        self.minD, self.maxD, self.bin = m.minDistance, m.maxDistance, m.bin
        self.shellCenters = np.asarray(m.r, F32)
        edges = np.asarray(m.edges, F32)
        self.shellVolumes = F32(4.0 / 3.0) * PI * (edges[1:] ** 3 - edges[0:-1] ** 3)
        self.volume = F32(m.volume)
        # fullrmc's number density: float32 atoms / float32 volume (Engine.py:2274)
        self.rho0 = F32(sum(self.counts)) / F32(m.volume)
        self.exp = np.asarray(m.G_exp, F32)
        self.varianceSquared = F32(m.variance_squared)
        w = m.weights if weights is None else weights
        self.weights = {(i, j): F32(w[i][j]) for i in range(self.ne) for j in range(i, self.ne)}
        self.data = None
        self.error = None
        self.accepted = 0
        self.tried = 0

    # ---------------------------------------------------------------- hist
    def _hist_kw(self):
        return dict(basis=self.basis, isPBC=self.isPBC, numberOfElements=self.ne, minDistance=self.minD,
                    maxDistance=self.maxD, histSize=self.hs, bin=self.bin, ncores=1)

    def _full(self, idx=None):
        if idx is None:
            return self.h.full_pairs_histograms_coords(boxCoords=self.box, moleculeIndex=self.mol,
                                                       elementIndex=self.el, **self._hist_kw())
        return self.h.full_pairs_histograms_coords(boxCoords=self.box[idx], moleculeIndex=self.mol[idx],
                                                   elementIndex=self.el[idx], **self._hist_kw())

    def _multiple(self, idx):
        return self.h.multiple_pairs_histograms_coords(indexes=idx, boxCoords=self.box, moleculeIndex=self.mol,
                                                       elementIndex=self.el, allAtoms=True, **self._hist_kw())

    # ----------------------------------------------------------------- G(r)
    def total_Gr(self, intra, inter):
        Gr = np.zeros(self.hs, dtype=F32)
        for i in range(self.ne):
            for j in range(i, self.ne):
                ni, nj = self.counts[i], self.counts[j]
                wij = self.weights[(i, j)]
                if i == j:
                    Nij = ni * (ni - 1) / 2.0
                    if Nij <= 0:
                        continue
                    Dij = F32(Nij / self.volume)
                    nij = intra[i, j, :] + inter[i, j, :]
                else:
                    Nij = ni * nj
                    if Nij <= 0:
                        continue
                    Dij = F32(Nij / self.volume)
                    nij = intra[i, j, :] + intra[j, i, :] + inter[i, j, :] + inter[j, i, :]
                Gr += wij * nij / Dij
        Gr /= self.shellVolumes
        return (F32(4.0) * PI * self.shellCenters * self.rho0) * (Gr - F32(1))

    def standard_error(self, intra, inter):
        diff = self.exp - self.total_Gr(intra, inter)
        return np.add.reduce(diff ** 2) / self.varianceSquared

    # ----------------------------------------------------------------- steps
    def compute_data(self):
        intra, inter = self._full()
        self.data = (intra, inter)
        self.error = self.standard_error(intra, inter)
        return self.error

    def _delta(self, idx):
        iM, eM = self._multiple(idx)
        iF, eF = self._full(idx)
        return iM - iF, eM - eF

    def _transform(self, coords):
        if self.t is not None:
            return self.t.transform_coordinates(self.rbasis, coords)
        M, c = self.rbasis, coords
        out = np.empty_like(c)
        for k in range(3):
            out[:, k] = (c[:, 0] * M[0, k] + c[:, 1] * M[1, k]) + c[:, 2] * M[2, k]
        return out

    def step(self, atoms, vec, u, force=None, moved_real=None):
        """One move of the atoms ``atoms`` by ``vec`` (or to ``moved_real``);
        returns True if accepted.  ``force`` (True/False) overrides the
        decision (used to replay a chain)."""
        idx = np.ascontiguousarray(np.atleast_1d(atoms), np.int32)
        if moved_real is None:
            moved_real = self.real[idx] + np.asarray(vec, F32)
        moved_real = np.asarray(moved_real, F32)
        moved_box = self._transform(moved_real) if self.isPBC else moved_real
        before = self._delta(idx)
        saved = np.array(self.box[idx], F32)
        self.box[idx] = moved_box
        after = self._delta(idx)
        self.box[idx] = saved
        intra = self.data[0] - before[0] + after[0]
        inter = self.data[1] - before[1] + after[1]
        new = self.standard_error(intra, inter)
        self.tried += 1
        reject = bool(new > self.error) and bool(F32(u) > self.tolerance)
        accept = (not reject) if force is None else bool(force)
        self.last = (intra, inter, new)
        if accept:
            self.data = (intra, inter)
            self.error = new
            self.real[idx] = moved_real
            self.box[idx] = moved_box
            self.accepted += 1
        return accept
