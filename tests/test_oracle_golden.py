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


def _atomic_cases(g):
    """(function name, args, kwargs, golden key prefix) of the atomic_distances golden file."""
    c, B, mol, el, ne = g["coords"], g["basis"], g["mol"], g["el"], int(g["ne"])
    lo, up, idx = g["lower"], g["upper"], g["indexes"]
    variants = [dict(), dict(countWithinLimits=False), dict(reduceDistance=True),
                dict(reduceDistanceToUpper=True, intraMolecular=False),
                dict(reduceDistanceToLower=True, interMolecular=False), dict(allAtoms=False),
                dict(countWithinLimits=False, reduceDistance=True, allAtoms=False)]
    out = []
    for v, kw in enumerate(variants):
        for tag, isPBC in (("pbc", True), ("ibc", False)):
            coords = c if isPBC else (c * np.float32(19.0)).astype(np.float32)
            out.append(("multiple_atomic_distances_coords", (idx, coords, B, isPBC, mol, el, ne, lo, up), kw,
                        "m%d_%s_" % (v, tag)))
    for v, kw in enumerate(variants[:3]):
        kw = {k: x for k, x in kw.items() if k != "allAtoms"}
        out.append(("full_atomic_distances_coords", (c, B, True, mol, el, ne, lo, up), kw, "f%d_" % v))
    out.append(("multiple_atomic_distances_dists", (idx, g["dm"], mol, el, ne, lo, up),
                dict(countWithinLimits=False), "md_"))
    out.append(("full_atomic_distances_dists", (g["dsq"], mol[:60], el[:60], ne, lo, up),
                dict(countWithinLimits=False), "fd_"))
    return out


def check_atomic_golden(module):
    """Every atomic_distances golden case through `module`, bit for bit."""
    g = golden("atomic_distances")
    for name, args, kw, pre in _atomic_cases(g):
        res = getattr(module, name)(*args, **kw)
        for k, key in enumerate(("nintra", "dintra", "ninter", "dinter")):
            want = g[pre + key]
            assert res[k].dtype == want.dtype and np.array_equal(res[k], want), (name, kw, pre, key)
    di, de = g["s0_dintra"].copy(), g["s0_dinter"].copy()
    ni, nn = g["s0_nintra"].copy(), g["s0_ninter"].copy()
    module.single_atomic_distances_dists(42, g["srow"], g["mol"], g["el"], di, de, ni, nn, g["lower"], g["upper"],
                                         reduceDistance=True)
    for got, key in ((di, "s_dintra"), (de, "s_dinter"), (ni, "s_nintra"), (nn, "s_ninter")):
        assert np.array_equal(got, g[key]), key
    si, se = module.pair_elements_stats(g["el"], g["mol"], int(g["ne"]))
    assert np.array_equal(si, g["stats_intra"]) and np.array_equal(se, g["stats_inter"])


def test_oracle_atomic_distances_golden(oracle_mod):
    check_atomic_golden(oracle_mod)


def check_coordination_golden(module):
    """Every atomic_coordination golden case through `module`, bit for bit
    (returned floats as float32, coordNumData after in-place calls)."""
    import coordination_cases as cc
    g = golden("atomic_coordination")
    rows = [np.ascontiguousarray(r) for r in g["rows"]]
    for key, name, args, data in cc.calls(g, rows):
        got = cc.run(module, name, args, data)
        want = g["out_" + key]
        assert got.dtype == want.dtype and np.array_equal(got.view(np.int32), want.view(np.int32)), (key, got, want)
    assert int(g["all_tot_raises"]) == 1
    with pytest.raises(TypeError):
        module.all_atoms_coord_number_totdists(np.ascontiguousarray(g["rows"].T), *cc.unpack(g),
                                               np.zeros(len(g["lower"]), np.float32))
    for name in ("single_atom_single_shell_subdists", "single_atom_single_shell_totdists"):
        args = (rows[1], g["lower"][1], g["upper"][1]) if name.endswith("subdists") else \
            (rows[1], cc.unpack(g)[1][1], g["lower"][1], g["upper"][1])
        assert type(getattr(module, name)(*args)) is float


def test_oracle_atomic_coordination_golden(oracle_mod):
    check_coordination_golden(oracle_mod)
