"""Pin the C oracle to the reference: every golden vector, bit for bit.

The golden files were produced by the compiled reference Cython
(tests/golden/make_golden.py).  These tests need no GPU.
"""
import numpy as np
import pytest

from conftest import DIST_CASES, HIST_CASES, golden


def _hist_args(g):
    return (g["coords"], g["basis"], bool(g["isPBC"]), g["mol"], g["el"], int(g["ne"]), g["minD"], g["maxD"],
            g["bin"], int(g["hs"]))


@pytest.mark.parametrize("case", HIST_CASES)
def test_full_histograms(oracle_mod, case):
    g = golden(case)
    hi, he = oracle_mod.full_pairs_histograms_coords(*_hist_args(g))
    assert np.array_equal(hi, g["full_intra"])
    assert np.array_equal(he, g["full_inter"])


@pytest.mark.parametrize("case", HIST_CASES)
def test_group_histograms(oracle_mod, case):
    g = golden(case)
    c, B, pbc, mol, el, ne, mn, mx, b, hs = _hist_args(g)
    k = 0
    while "g%d_indexes" % k in g:
        hi, he = oracle_mod.multiple_pairs_histograms_coords(g["g%d_indexes" % k], c, B, pbc, mol, el, ne, mn, mx, b,
                                                             hs, bool(g["g%d_allAtoms" % k]))
        assert np.array_equal(hi, g["g%d_intra" % k])
        assert np.array_equal(he, g["g%d_inter" % k])
        k += 1
    assert k >= 1


def test_bin_overflow_lands_in_next_row():
    """d just below max rounds to bin hs: the count lands in bin 0 of the next row."""
    g = golden("bin_overflow_ibc")
    assert g["full_inter"][0, 1, 0] == 1.0 and g["full_inter"][1, 0, 0] == 1.0
    assert g["full_inter"].sum() == 2.0


def test_float32_saturation(oracle_mod):
    g = golden("saturation")
    n = int(g["n"])
    coords = np.zeros((n, 3), np.float32)
    hi, he = oracle_mod.full_pairs_histograms_coords(coords, np.eye(3, dtype=np.float32), False,
                                                     np.arange(n, dtype=np.int32), np.zeros(n, np.int32), 1,
                                                     g["minD"], g["maxD"], g["bin"], int(g["hs"]))
    assert np.array_equal(he, g["full_inter"]) and np.array_equal(hi, g["full_intra"])
    assert he.max() == 2.0 ** 24


@pytest.mark.parametrize("nn", [0, 1])
def test_tiny(oracle_mod, nn):
    g = golden("tiny_n%d" % nn)
    z = np.zeros((nn, 3), np.float32)
    hi, he = oracle_mod.full_pairs_histograms_coords(z, np.eye(3, dtype=np.float32), True, np.zeros(nn, np.int32),
                                                     np.zeros(nn, np.int32), 2, g["minD"], g["maxD"], g["bin"],
                                                     int(g["hs"]))
    assert np.array_equal(hi, g["full_intra"]) and np.array_equal(he, g["full_inter"])


@pytest.mark.parametrize("case", DIST_CASES)
def test_distances_and_differences(oracle_mod, case):
    g = golden(case)
    c, B, pbc, idx, pts = g["coords"], g["basis"], bool(g["isPBC"]), g["indexes"], g["points"]
    o = oracle_mod
    assert np.array_equal(o.pairs_distances_to_point(c[5], c, B, pbc), g["dist_to_point"])
    assert np.array_equal(o.pairs_distances_to_indexcoords(7, c, B, pbc, True), g["dist_to_index_all"])
    assert np.array_equal(o.pairs_distances_to_indexcoords(7, c, B, pbc, False)[7:], g["dist_to_index_from"])
    assert np.array_equal(o.pairs_distances_to_multi_points(pts, c, B, pbc), g["dist_to_multi_points"])
    assert np.array_equal(o.pairs_distances_to_multi_indexcoords(idx, c, B, pbc, True), g["dist_to_multi_index"])
    assert np.array_equal(o.pairs_differences_to_point(c[5], c, B, pbc), g["diff_to_point"])
    assert np.array_equal(o.pairs_differences_to_indexcoords(7, c, B, pbc, True), g["diff_to_index_all"])
    assert np.array_equal(o.pairs_differences_to_multi_points(pts, c, B, pbc), g["diff_to_multi_points"])
    assert np.array_equal(o.pairs_differences_to_multi_indexcoords(idx, c, B, pbc, True), g["diff_to_multi_index"])
    assert np.array_equal(o.from_to_points_differences(c, np.ascontiguousarray(c[::-1]), B, pbc), g["from_to"])
    assert np.float32(o.point_to_point_distance(c[1], c[2], B, pbc)) == g["p2p"]
    assert np.array_equal(o.pair_difference_to_point(c[1], c[2], B, pbc), g["pair_diff"])


def test_single_and_dists(oracle_mod):
    g = golden("single_and_dists")
    src = golden("general_triclinic_ne4_mol")
    mol, el = src["mol"], src["el"]
    mn, mx, b, hs = src["minD"], src["maxD"], src["bin"], int(src["hs"])
    for tag, atom, allAtoms in (("a", 100, True), ("b", 650, False)):
        hi, he = g["h0_intra"].copy(), g["h0_inter"].copy()
        oracle_mod.single_pairs_histograms(atom, g["dist_" + tag], mol, el, hi, he, mn, mx, b, allAtoms)
        assert np.array_equal(hi, g["intra_" + tag]) and np.array_equal(he, g["inter_" + tag])
    hi, he = oracle_mod.multiple_pairs_histograms_dists(g["dm_indexes"], g["dm"], mol, el, 4, mn, mx, b, hs, True)
    assert np.array_equal(hi, g["mdist_intra"]) and np.array_equal(he, g["mdist_inter"])
    hi, he = oracle_mod.full_pairs_histograms_dists(g["dsq"], mol[:40], el[:40], 4, mn, mx, b, hs)
    assert np.array_equal(hi, g["fdist_intra"]) and np.array_equal(he, g["fdist_inter"])


def test_transform(oracle_mod):
    g = golden("transform")
    assert np.array_equal(oracle_mod.transform_coordinates(g["rbasis"], g["real"]), g["box"])
    assert np.array_equal(oracle_mod.transform_coordinates(g["basis"], g["box"]), g["back"])


def test_fp64_transforms_match_reference_float32(oracle_mod):
    """The FP64 restatements agree with the reference's float32 sums to ~1e-5."""
    g = golden("reciprocal")
    r, q = g["r"], g["q"]
    s64 = oracle_mod.gr_to_sq_fp64(r, g["gr"], q, g["rho"])
    assert np.allclose(s64, g["gr_to_sq"], rtol=1e-4, atol=1e-4 * np.abs(g["gr_to_sq"]).max())
    S64 = oracle_mod.Gr_to_sq_fp64(r, g["Gr"], q)
    assert np.allclose(S64, g["Gr_to_sq"], rtol=1e-4, atol=1e-4 * np.abs(g["Gr_to_sq"]).max())
    assert int(g["sq_to_Gr_raises"]) == 1
    # sq_to_Gr is the inverse sine transform: applying it to Gr_to_sq's output
    # recovers G(r) up to truncation of the q range (smoke check of the formula).
    G = oracle_mod.sq_to_Gr_fp64(q, r, S64)
    assert np.isfinite(G).all()
