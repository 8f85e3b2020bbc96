"""Golden all-pairs histograms of the 100,000-atom triclinic system, written
by the compiled reference Cython.

The system: 100,000 atoms, three species at fractions 0.5/0.3/0.2, uniform
random coordinates in a triclinic periodic box a = b = c = 103 A,
alpha = beta = 90, gamma = 120 degrees, r 0-20 A in 0.01 A bins (2001 bins),
from ``fullrmc_gb300.synthetic.triclinic_100k(seed=SEED)``.

Run in a checkout that has the reference sources (``python
tests/golden/make_cfg2_golden.py [processes]``).  The compiled reference's
``full_pairs_histograms_coords`` is ``multiple_pairs_histograms_coords``
over ``indexes = arange(N)`` with ``allAtoms=False``
(``Extensions/pairs_histograms.pyx:289-335``): row i counts the atoms
j > i.  This script calls ``multiple_pairs_histograms_coords(indexes=rows,
allAtoms=False, ncores=1)`` on disjoint row ranges in separate processes
(``ncores=1``: the reference's OpenMP histogram loop increments shared bins
without a reduction) and adds the partial histograms.  Every bin stays far
below 2^24, so the float32 partial counts are exact integers and their sum
equals the single-process result.  About 5e9 pair distances: a few minutes
on one core per 1e9 pairs.

A second file holds the same system with its atoms grouped into molecules of
four consecutive indexes (``moleculeIndex = arange(N) // 4``), so that the
intramolecular histogram is exercised at this size too.

Each file keeps the seed, SHA-256 digests of the regenerated inputs (so a test
can tell a changed generator from a changed kernel) and the two float32
(3, 3, 2001) histograms.
"""
from __future__ import annotations

import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

SEED = 2
OUTS = {1: os.path.join(HERE, "cfg2_triclinic_100k.npz"), 4: os.path.join(HERE, "cfg2_triclinic_100k_mol4.npz")}


def system(molsize=1):
    from fullrmc_gb300 import synthetic
    s = synthetic.triclinic_100k(seed=SEED)
    if molsize > 1:
        s.mol = (np.arange(s.box_coords.shape[0]) // molsize).astype(np.int32)
    return s


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def row_chunks(n, parts):
    """Contiguous row ranges with about equal pair counts (row i has n-1-i)."""
    pairs = np.arange(n - 1, -1, -1, dtype=np.float64)
    cum = np.cumsum(pairs)
    cuts = np.searchsorted(cum, cum[-1] * np.arange(1, parts) / parts)
    edges = [0, *[int(c) for c in cuts], n]
    return [(a, b) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def _work(args):
    lo, hi, molsize = args
    import build_ref
    ph = build_ref.import_reference()["pairs_histograms"]
    s = system(molsize)
    m = s.model
    idx = np.arange(lo, hi, dtype=np.int32)
    return ph.multiple_pairs_histograms_coords(
        indexes=idx, boxCoords=s.box_coords, basis=s.basis, isPBC=True, moleculeIndex=s.mol,
        elementIndex=s.el, numberOfElements=len(m.elements_count), minDistance=m.minDistance,
        maxDistance=m.maxDistance, bin=m.bin, histSize=m.hs, allAtoms=False, ncores=1)


def main(procs, molsize):
    import build_ref
    build_ref.build()
    s = system(molsize)
    m = s.model
    n = s.box_coords.shape[0]
    t0 = time.time()
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        parts = pool.map(_work, [(a, b, molsize) for a, b in row_chunks(n, 8 * procs)], chunksize=1)
    intra = np.zeros_like(parts[0][0], dtype=np.float64)
    inter = np.zeros_like(parts[0][1], dtype=np.float64)
    for a, b in parts:
        intra += a
        inter += b
    assert inter.max() < 2 ** 24
    out = OUTS[molsize]
    np.savez_compressed(out, seed=np.int64(SEED), n=np.int64(n), molsize=np.int32(molsize), basis=s.basis,
                        minDistance=m.minDistance, maxDistance=m.maxDistance, bin=m.bin, histSize=np.int32(m.hs),
                        inputs_sha256=np.array(digest(s.box_coords, s.el, s.mol)),
                        hintra=intra.astype(np.float32), hinter=inter.astype(np.float32))
    print("wrote %s: %d atoms, %.0f pairs counted, %.1f s on %d processes"
          % (out, n, inter.sum() + intra.sum(), time.time() - t0, procs))


if __name__ == "__main__":
    nproc = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count() or 1
    for size in OUTS:
        main(nproc, size)
