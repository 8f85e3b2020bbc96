"""Generate the golden vectors from the compiled reference Cython.

Run in a checkout that has the reference sources (``python
tests/golden/make_golden.py``): it builds ``oracle/_ref`` if needed, imports
the reference's own ``fullrmc.Core.pairs_distances``,
``fullrmc.Core.pairs_histograms`` and ``fullrmc.Core.reciprocal_space``
(always with ``ncores=1``; the reference's OpenMP histogram loop increments
shared bins without a reduction) and writes ``tests/golden/*.npz``.  Every
input is seeded, so the files are reproducible.  The reference ships no test
vectors of its own, so these files pin both the C oracle and the CUDA
library.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

F = np.float32


def triclinic_basis(a, b, c, alpha, beta, gamma):
    """Row-vector basis: a along x, b in the xy plane (float32)."""
    al, be, ga = np.radians([alpha, beta, gamma])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(c * c - cx * cx - cy * cy)
    B = np.array([[a, 0, 0], [b * np.cos(ga), b * np.sin(ga), 0], [cx, cy, cz]], np.float64)
    B[np.abs(B) < 1e-9] = 0.0
    return B.astype(F)


def grid(rmax, dr=0.01):
    """fullrmc's limits from an experimental r grid (PairDistributionConstraints.py:726,745-755)."""
    x = np.arange(0, rmax + dr / 10, dr).astype(F)
    b = F(x[1] - x[0])
    return F(x[0] - b / 2.0), F(x[-1] + b / 2.0), b, np.int32(len(x))


def species(rng, n, fractions):
    counts = np.floor(np.asarray(fractions) * n).astype(int)
    counts[0] += n - counts.sum()
    el = np.repeat(np.arange(len(fractions)), counts).astype(np.int32)
    rng.shuffle(el)
    return el


def main():
    import build_ref
    build_ref.build()
    R = build_ref.import_reference()
    ph, pd, rs = R["pairs_histograms"], R["pairs_distances"], R["reciprocal_space"]
    bcc = R["boundary_conditions_collection"]
    out = {}

    def hist_case(name, coords, basis, isPBC, mol, el, ne, lims, groups):
        mn, mx, b, hs = lims
        d = dict(coords=coords, basis=basis, isPBC=np.int32(isPBC), mol=mol, el=el, ne=np.int32(ne),
                 minD=mn, maxD=mx, bin=b, hs=hs)
        hi, he = ph.full_pairs_histograms_coords(coords, basis, isPBC, mol, el, ne, mn, mx, b, hs, 1)
        d["full_intra"], d["full_inter"] = hi, he
        for gi, (idx, allAtoms) in enumerate(groups):
            hi, he = ph.multiple_pairs_histograms_coords(idx, coords, basis, isPBC, mol, el, ne, mn, mx, b, hs,
                                                         allAtoms, 1)
            d["g%d_indexes" % gi] = idx
            d["g%d_allAtoms" % gi] = np.int32(allAtoms)
            d["g%d_intra" % gi], d["g%d_inter" % gi] = hi, he
        out[name] = d

    # A: cubic PBC, binary alloy (config-1 shape, smaller N), atomic molecules.
    rng = np.random.default_rng(101)
    n = 2000
    L = F(38.2 * (n / 5000.0) ** (1 / 3.0))
    hist_case("cubic_pbc_ne2", rng.random((n, 3)).astype(F), np.diag([L, L, L]).astype(F), True,
              np.arange(n, dtype=np.int32), species(rng, n, [0.5, 0.5]), 2, grid(15.0),
              [(np.array([17], np.int32), True), (np.array([5, 900, 1999], np.int32), True),
               (np.array([0, 3, 1500], np.int32), False)])

    # B: triclinic gamma=120 (config-2 shape, smaller N), 3 species 0.5/0.3/0.2.
    rng = np.random.default_rng(202)
    n = 3000
    a = F((n / 0.1057 / np.sin(np.radians(120))) ** (1 / 3.0))
    hist_case("triclinic120_ne3", rng.random((n, 3)).astype(F), triclinic_basis(a, a, a, 90, 90, 120), True,
              np.arange(n, dtype=np.int32), species(rng, n, [0.5, 0.3, 0.2]), 3, grid(10.0),
              [(np.array([1234], np.int32), True)])

    # C: general triclinic, 4 species, 13-atom molecules (non-empty intra).
    rng = np.random.default_rng(303)
    nm, k = 100, 13
    n = nm * k
    B = triclinic_basis(26.0, 24.0, 25.0, 78.0, 95.0, 110.0)
    centres = rng.random((nm, 3))
    offs = rng.normal(scale=0.04, size=(n, 3))
    coords = (np.repeat(centres, k, axis=0) + offs).astype(F)
    mol = np.repeat(np.arange(nm), k).astype(np.int32)
    el = np.tile(np.array([0, 0, 0, 0, 1, 2, 2, 2, 2, 3, 3, 3, 3]), nm).astype(np.int32)
    hist_case("general_triclinic_ne4_mol", coords, B, True, mol, el, 4, grid(12.0),
              [(np.arange(13 * 7, 13 * 8, dtype=np.int32), True), (np.arange(13 * 7, 13 * 8, dtype=np.int32), False),
               (np.array([], np.int32), True)])

    # D: infinite boundary conditions (real coordinates), 2 species, molecules of 3.
    rng = np.random.default_rng(404)
    n = 1000
    hist_case("ibc_ne2", (rng.random((n, 3)) * 30.0).astype(F), np.eye(3, dtype=F), False,
              (np.arange(n) // 3).astype(np.int32), species(rng, n, [0.6, 0.4]), 2, grid(15.0),
              [(np.array([10, 11, 12], np.int32), True)])

    # E: bin overflow.  d = 15.004999f < max = 15.005f but (d - min) / bin
    # rounds to 1501 == hs, so the count lands in bin 0 of the next row.
    mn, mx, b, hs = grid(15.0)
    dov = F(15.004999)
    assert dov < mx and int((dov - mn) / b) == hs
    coords = np.array([[0, 0, 0], [dov, 0, 0], [0, dov, 0], [0, 0, 60.0], [3.25, 60.0, 0]], F)
    el = np.array([0, 0, 1, 1, 0], np.int32)
    # pairs (0,1): [0][0] -> [0][1][0]; (0,2): [0][1] -> [1][0][0]; (1,2) d=21.2 > max;
    # atom 3 and 4 are beyond max from everyone except each other (d>max) -> no
    # out-of-array write can occur.
    hist_case("bin_overflow_ibc", coords, np.eye(3, dtype=F), False, np.arange(5, dtype=np.int32), el, 2,
              (mn, mx, b, hs), [(np.array([0], np.int32), True), (np.array([2, 1], np.int32), True)])

    # F: bin edges: atoms at exact float32 bin edges and their neighbours.
    mn, mx, b, hs = grid(5.0)
    edges = np.array([F(mn + F(i) * b) for i in range(1, hs, 37)], F)
    pos = np.concatenate([edges, np.nextafter(edges, F(100)), np.nextafter(edges, F(-100))])
    coords = np.zeros((pos.size + 1, 3), F)
    coords[1:, 0] = pos
    n = coords.shape[0]
    hist_case("bin_edges_ibc", coords, np.eye(3, dtype=F), False, np.arange(n, dtype=np.int32),
              (np.arange(n) % 2).astype(np.int32), 2, (mn, mx, b, hs), [(np.array([0], np.int32), True)])

    # G: float32 saturation: 6000 coincident atoms -> 17,997,000 increments of
    # one bin; a float32 counter stops at 2**24.
    n = 6000
    coords = np.zeros((n, 3), F)
    mn, mx, b, hs = grid(1.0)
    hi, he = ph.full_pairs_histograms_coords(coords, np.eye(3, dtype=F), False, np.arange(n, dtype=np.int32),
                                             np.zeros(n, np.int32), 1, mn, mx, b, hs, 1)
    out["saturation"] = dict(n=np.int32(n), minD=mn, maxD=mx, bin=b, hs=hs, full_intra=hi, full_inter=he)

    # G2: half-box ties.  Box-coordinate differences of exactly +-0.49999997
    # (the float just below 0.5), +-0.5 and neighbours, in a cubic box whose
    # half side 5.005 is a bin edge.  The reference's round()
    # (pairs_distances.pyx:31-32) adds the float32 HALF_BOX_LENGTH in float32,
    # where 0.49999997 + 0.5 rounds to 1.0: the difference wraps to
    # -0.50000003 (d = 5.0050003, bin 501), where exact arithmetic would keep
    # it (d = 5.0049997, bin 500).
    h = np.nextafter(F(0.5), F(0))
    pts = [(0, 0, 0), (h, 0, 0), (0, h, F(0.3)), (F(0.5), F(0.5), 0), (np.nextafter(F(0.5), F(1)), F(0.2), F(0.7)),
           (np.nextafter(F(1), F(0)), h, F(0.5)), (F(0.25), F(0.25) + h, F(0.25)), (F(0.75), F(0.75), F(0.75) - h)]
    rng = np.random.default_rng(707)
    coords = np.concatenate([np.array(pts, F), rng.random((300, 3)).astype(F)]).astype(F)
    n = coords.shape[0]
    Lh = F(10.01)
    hist_case("half_box_pbc", coords, np.diag([Lh, Lh, Lh]).astype(F), True, np.arange(n, dtype=np.int32),
              (np.arange(n) % 2).astype(np.int32), 2, grid(6.0),
              [(np.array([0, 1, 5], np.int32), True), (np.array([1, 2, 3], np.int32), False)])

    # G2: real data -- the reference's own NiTi example (6,750 atoms, cubic
    # 45.75 A, Examples/atomicNiTi/system.pdb) on the r grid of its
    # experimental.gr, box coordinates through the reference's
    # transform_coordinates as fullrmc's Engine makes them.
    niti = os.path.join(build_ref.REFERENCE_ROOT, "Examples", "atomicNiTi")
    if os.path.exists(os.path.join(niti, "system.pdb")):
        real, names, L = [], [], None
        with open(os.path.join(niti, "system.pdb")) as fh:
            for line in fh:
                if line.startswith("CRYST1"):
                    L = float(line[6:15])
                elif line.startswith(("ATOM", "HETATM")):
                    real.append((float(line[30:38]), float(line[38:46]), float(line[46:54])))
                    names.append(line[76:78].strip().lower())
        real = np.array(real, F)
        kinds = sorted(set(names))
        el = np.array([kinds.index(x) for x in names], np.int32)
        B = np.diag([L, L, L]).astype(F)
        box = bcc.transform_coordinates(np.linalg.inv(B.astype(np.float64)).astype(F), real)
        x = np.loadtxt(os.path.join(niti, "experimental.gr"))[:, 0].astype(F)
        b = F(x[1] - x[0])
        lims = (F(x[0] - b / F(2)), F(x[-1] + b / F(2)), b, np.int32(len(x)))
        n = real.shape[0]
        hist_case("niti_pdb", box, B, True, np.arange(n, dtype=np.int32), el, len(kinds), lims,
                  [(np.array([0, 3374, 3375, 6749], np.int32), True),
                   (np.arange(0, n, 519, dtype=np.int32), False)])
        out["niti_pdb"]["real"] = real
        out["niti_pdb"]["rbasis"] = np.linalg.inv(B.astype(np.float64)).astype(F)
        out["niti_pdb"]["G_exp"] = np.loadtxt(os.path.join(niti, "experimental.gr"))[:, 1].astype(F)
        out["niti_pdb"]["r"] = x

    # H: edge sizes: one atom, zero atoms.
    for nn in (0, 1):
        coords = np.zeros((nn, 3), F)
        mn, mx, b, hs = grid(3.0)
        hi, he = ph.full_pairs_histograms_coords(coords, np.eye(3, dtype=F), True, np.zeros(nn, np.int32),
                                                 np.zeros(nn, np.int32), 2, mn, mx, b, hs, 1)
        out["tiny_n%d" % nn] = dict(n=np.int32(nn), minD=mn, maxD=mx, bin=b, hs=hs, full_intra=hi, full_inter=he)

    # I: the distance / difference family.
    for case, isPBC in (("general_triclinic_ne4_mol", True), ("ibc_ne2", False), ("cubic_pbc_ne2", True)):
        src = out[case]
        c = np.ascontiguousarray(src["coords"][:300])
        B = src["basis"]
        idx = np.array([0, 7, 299, 42], np.int32)
        pts = np.ascontiguousarray(c[[3, 9, 27, 81]].T)  # (3, 4): the reference reads points[:, k]
        d = dict(coords=c, basis=B, isPBC=np.int32(isPBC), indexes=idx, points=pts)
        d["dist_to_point"] = pd.pairs_distances_to_point(c[5], c, B, isPBC, 1)
        d["dist_to_index_all"] = pd.pairs_distances_to_indexcoords(7, c, B, isPBC, True, 1)
        d["dist_to_index_from"] = pd.pairs_distances_to_indexcoords(7, c, B, isPBC, False, 1)[7:]
        d["dist_to_multi_points"] = pd.pairs_distances_to_multi_points(pts, c, B, isPBC, 1)
        d["dist_to_multi_index"] = pd.pairs_distances_to_multi_indexcoords(idx, c, B, isPBC, True, 1)
        d["diff_to_point"] = pd.pairs_differences_to_point(c[5], c, B, isPBC, 1)
        d["diff_to_index_all"] = pd.pairs_differences_to_indexcoords(7, c, B, isPBC, True, 1)
        d["diff_to_multi_points"] = pd.pairs_differences_to_multi_points(pts, c, B, isPBC, 1)
        d["diff_to_multi_index"] = pd.pairs_differences_to_multi_indexcoords(idx, c, B, isPBC, True, 1)
        d["from_to"] = pd.from_to_points_differences(c, np.ascontiguousarray(c[::-1]), B, isPBC, 1)
        d["p2p"] = np.float32(pd.point_to_point_distance(c[1], c[2], B, isPBC, 1))
        d["pair_diff"] = pd.pair_difference_to_point(c[1], c[2], B, isPBC, 1)
        out["dist_" + case] = d

    # J: single_pairs_histograms in place on non-zero histograms, and the
    # *_dists variants on a distance matrix.
    src = out["general_triclinic_ne4_mol"]
    c, B = src["coords"], src["basis"]
    mol, el = src["mol"], src["el"]
    mn, mx, b, hs = src["minD"], src["maxD"], src["bin"], src["hs"]
    rng = np.random.default_rng(505)
    h0i = rng.integers(0, 50, size=(4, 4, int(hs))).astype(F)
    h0e = rng.integers(0, 50, size=(4, 4, int(hs))).astype(F)
    d = dict(h0_intra=h0i.copy(), h0_inter=h0e.copy())
    for tag, atom, allAtoms in (("a", 100, True), ("b", 650, False)):
        dist = pd.pairs_distances_to_indexcoords(atom, c, B, True, True, 1)
        hi, he = h0i.copy(), h0e.copy()
        ph.single_pairs_histograms(atom, dist, mol, el, hi, he, mn, mx, b, allAtoms, 1)
        d["dist_" + tag] = dist
        d["intra_" + tag], d["inter_" + tag] = hi, he
    idx = np.array([4, 77, 500, 1299], np.int32)
    dm = pd.pairs_distances_to_multi_indexcoords(idx, c, B, True, True, 1)
    d["dm_indexes"], d["dm"] = idx, dm
    d["mdist_intra"], d["mdist_inter"] = ph.multiple_pairs_histograms_dists(idx, dm, mol, el, 4, mn, mx, b, hs, True, 1)
    dsq = pd.pairs_distances_to_multi_indexcoords(np.arange(40, dtype=np.int32), c[:40], B, True, True, 1)
    d["dsq"] = dsq
    d["fdist_intra"], d["fdist_inter"] = ph.full_pairs_histograms_dists(dsq, mol[:40], el[:40], 4, mn, mx, b, hs, 1)
    out["single_and_dists"] = d

    # K: reciprocal space (reference float32 outputs; FP64 results are
    # compared at about 1e-5 relative).
    r = (np.arange(1, 301) * 0.05).astype(F)
    gr = (1.0 + 0.3 * np.sin(r) * np.exp(-0.2 * r)).astype(F)
    Gr = (4 * np.pi * 0.08 * r * (gr - 1)).astype(F)
    q = (0.5 + np.arange(120) * 0.1).astype(F)
    sq = rs.Gr_to_sq(r, Gr, q)
    # The reference's sq_to_Gr (reciprocal_space.pyx:143) passes an array to
    # libc sin and raises TypeError for every input; record that fact.
    try:
        rs.sq_to_Gr(q, r, sq.astype(F))
        sq_to_Gr_raises = 0
    except TypeError:
        sq_to_Gr_raises = 1
    out["reciprocal"] = dict(r=r, gr=gr, Gr=Gr, q=q, rho=F(0.08),
                             gr_to_sq=rs.gr_to_sq(r, gr, q, F(0.08)), Gr_to_sq=sq,
                             sq_to_Gr_raises=np.int32(sq_to_Gr_raises))

    # M: atomic_distances (InterMolecularDistanceConstraint): every flag
    # combination on a PBC system with 5-atom molecules, the dists variants,
    # the in-place single-atom call and pair_elements_stats.
    if "atomic_distances" in R:
        ad = R["atomic_distances"]
        rng = np.random.default_rng(808)
        n, ne = 600, 3
        c = rng.random((n, 3)).astype(F)
        B = triclinic_basis(19.0, 18.0, 20.0, 85.0, 95.0, 105.0)
        mol = (np.arange(n) // 5).astype(np.int32)
        el = rng.integers(0, ne, size=n).astype(np.int32)
        lo = (0.8 + 0.4 * rng.random((ne, ne, 1))).astype(F)
        up = (2.2 + 1.2 * rng.random((ne, ne, 1))).astype(F)
        idx = np.array([3, 17, 250, 17, 599, 0], np.int32)
        d = dict(coords=c, basis=B, mol=mol, el=el, ne=np.int32(ne), lower=lo, upper=up, indexes=idx)
        variants = [dict(), dict(countWithinLimits=False), dict(reduceDistance=True),
                    dict(reduceDistanceToUpper=True, intraMolecular=False),
                    dict(reduceDistanceToLower=True, interMolecular=False), dict(allAtoms=False),
                    dict(countWithinLimits=False, reduceDistance=True, allAtoms=False)]
        for v, kw in enumerate(variants):
            for tag, isPBC in (("pbc", True), ("ibc", False)):
                coords = c if isPBC else (c * F(19.0)).astype(F)
                res = ad.multiple_atomic_distances_coords(idx, coords, B, isPBC, mol, el, ne, lo, up, **kw)
                for k, name in enumerate(("nintra", "dintra", "ninter", "dinter")):
                    d["m%d_%s_%s" % (v, tag, name)] = res[k]
        for v, kw in enumerate(variants[:3]):
            kw = {k: x for k, x in kw.items() if k != "allAtoms"}
            res = ad.full_atomic_distances_coords(c, B, True, mol, el, ne, lo, up, **kw)
            for k, name in enumerate(("nintra", "dintra", "ninter", "dinter")):
                d["f%d_%s" % (v, name)] = res[k]
        dm = pd.pairs_distances_to_multi_indexcoords(idx, c, B, True, True, 1)
        d["dm"] = dm
        res = ad.multiple_atomic_distances_dists(idx, dm, mol, el, ne, lo, up, countWithinLimits=False)
        for k, name in enumerate(("nintra", "dintra", "ninter", "dinter")):
            d["md_%s" % name] = res[k]
        sq = pd.pairs_distances_to_multi_indexcoords(np.arange(60, dtype=np.int32), c[:60], B, True, True, 1)
        d["dsq"] = sq
        res = ad.full_atomic_distances_dists(sq, mol[:60], el[:60], ne, lo, up, countWithinLimits=False)
        for k, name in enumerate(("nintra", "dintra", "ninter", "dinter")):
            d["fd_%s" % name] = res[k]
        di = rng.random((ne, ne, 1)).astype(F)
        de = rng.random((ne, ne, 1)).astype(F)
        ni = rng.integers(0, 5, size=(ne, ne, 1)).astype(np.int32)
        nn = rng.integers(0, 5, size=(ne, ne, 1)).astype(np.int32)
        d["s0_dintra"], d["s0_dinter"], d["s0_nintra"], d["s0_ninter"] = di.copy(), de.copy(), ni.copy(), nn.copy()
        row = pd.pairs_distances_to_indexcoords(42, c, B, True, True, 1)
        d["srow"] = row
        ad.single_atomic_distances_dists(42, row, mol, el, di, de, ni, nn, lo, up, reduceDistance=True)
        d["s_dintra"], d["s_dinter"], d["s_nintra"], d["s_ninter"] = di, de, ni, nn
        d["stats_intra"], d["stats_inter"] = ad.pair_elements_stats(el, mol, ne)
        out["atomic_distances"] = d

    # N: atomic_coordination (AtomicCoordinationNumberConstraint): every
    # function of the module on the inputs of tests/coordination_cases.py.
    if "atomic_coordination" in R:
        sys.path.insert(0, os.path.dirname(HERE))
        import coordination_cases as cc
        g = cc.make_inputs()
        rows = cc.distance_rows(pd, g, g["indexes"])
        g["rows"] = np.stack(rows)
        for key, name, args, data in cc.calls(g, rows):
            g["out_" + key] = cc.run(R["atomic_coordination"], name, args, data)
        try:
            R["atomic_coordination"].all_atoms_coord_number_totdists(g["rows"].T.copy(), *cc.unpack(g),
                                                                     np.zeros(5, F))
            g["all_tot_raises"] = np.int32(0)
        except TypeError:
            g["all_tot_raises"] = np.int32(1)
        out["atomic_coordination"] = g

    # L: transform_coordinates (box -> real through the basis, real -> box
    # through its inverse).
    B = triclinic_basis(26.0, 24.0, 25.0, 78.0, 95.0, 110.0)
    rb = np.linalg.inv(B.astype(np.float64)).astype(F)
    real = (np.random.default_rng(606).random((500, 3)) * 25.0).astype(F)
    out["transform"] = dict(basis=B, rbasis=rb, real=real, box=bcc.transform_coordinates(rb, real),
                            back=bcc.transform_coordinates(B, bcc.transform_coordinates(rb, real)))

    only = set(sys.argv[1:])  # names of the cases to (re)write; none = all
    written = 0
    for name, d in out.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        written += 1
    print("wrote %d golden files" % written)


if __name__ == "__main__":
    main()
