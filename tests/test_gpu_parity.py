"""GPU parity: the CUDA library against the golden vectors (produced by the
compiled reference) and against the C oracle on seeded systems.  Histogram
counts, distances and differences must be bit-identical."""
import numpy as np
import pytest

from conftest import DIST_CASES, HIST_CASES, golden

pytestmark = pytest.mark.gpu

F = np.float32


@pytest.fixture(scope="module")
def gpu():
    import fullrmc_gb300
    from fullrmc_gb300 import _native
    fullrmc_gb300.load()
    info = _native.device_info()
    assert info["sms"] > 0
    yield fullrmc_gb300
    set_tune()


def set_tune(threads=512, rows=2, queued=-1, qcap=16, ctas=1, min_pairs=8.0e6):
    from fullrmc_gb300._native import call
    call("frmc_set_full_tune", threads, rows, queued, qcap, ctas, float(min_pairs))


def _hist_args(g):
    return dict(boxCoords=g["coords"], basis=g["basis"], isPBC=bool(g["isPBC"]), moleculeIndex=g["mol"],
                elementIndex=g["el"], numberOfElements=int(g["ne"]), minDistance=g["minD"], maxDistance=g["maxD"],
                bin=g["bin"], histSize=int(g["hs"]))


# ------------------------------------------------------------------ golden
@pytest.mark.parametrize("tiled", [False, True])
@pytest.mark.parametrize("case", HIST_CASES)
def test_golden_full(gpu, case, tiled):
    set_tune(min_pairs=0 if tiled else 1e30)
    g = golden(case)
    hi, he = gpu.pairs_histograms.full_pairs_histograms_coords(**_hist_args(g))
    set_tune()
    assert np.array_equal(hi, g["full_intra"])
    assert np.array_equal(he, g["full_inter"])


@pytest.mark.parametrize("case", HIST_CASES)
def test_golden_groups(gpu, case):
    g = golden(case)
    a = _hist_args(g)
    k = 0
    while "g%d_indexes" % k in g:
        hi, he = gpu.pairs_histograms.multiple_pairs_histograms_coords(
            indexes=g["g%d_indexes" % k], allAtoms=bool(g["g%d_allAtoms" % k]), **a)
        assert np.array_equal(hi, g["g%d_intra" % k]), k
        assert np.array_equal(he, g["g%d_inter" % k]), k
        k += 1


@pytest.mark.parametrize("tiled", [False, True])
def test_golden_saturation(gpu, tiled):
    set_tune(min_pairs=0 if tiled else 1e30)
    g = golden("saturation")
    n = int(g["n"])
    hi, he = gpu.pairs_histograms.full_pairs_histograms_coords(
        np.zeros((n, 3), F), np.eye(3, dtype=F), False, np.arange(n, dtype=np.int32), np.zeros(n, np.int32), 1,
        g["minD"], g["maxD"], g["bin"], int(g["hs"]))
    set_tune()
    assert np.array_equal(hi, g["full_intra"]) and np.array_equal(he, g["full_inter"])
    assert he.max() == 2.0 ** 24


@pytest.mark.parametrize("nn", [0, 1])
def test_golden_tiny(gpu, nn):
    g = golden("tiny_n%d" % nn)
    z = np.zeros((nn, 3), F)
    hi, he = gpu.pairs_histograms.full_pairs_histograms_coords(z, np.eye(3, dtype=F), True, np.zeros(nn, np.int32),
                                                               np.zeros(nn, np.int32), 2, g["minD"], g["maxD"],
                                                               g["bin"], int(g["hs"]))
    assert np.array_equal(hi, g["full_intra"]) and np.array_equal(he, g["full_inter"])


@pytest.mark.parametrize("case", DIST_CASES)
def test_golden_distances(gpu, case):
    g = golden(case)
    c, B, pbc, idx, pts = g["coords"], g["basis"], bool(g["isPBC"]), g["indexes"], g["points"]
    pd = gpu.pairs_distances
    assert np.array_equal(pd.pairs_distances_to_point(c[5], c, B, pbc), g["dist_to_point"])
    assert np.array_equal(pd.pairs_distances_to_indexcoords(7, c, B, pbc, True), g["dist_to_index_all"])
    assert np.array_equal(pd.pairs_distances_to_indexcoords(7, c, B, pbc, False)[7:], g["dist_to_index_from"])
    assert np.array_equal(pd.pairs_distances_to_multi_points(pts, c, B, pbc), g["dist_to_multi_points"])
    assert np.array_equal(pd.pairs_distances_to_multi_indexcoords(idx, c, B, pbc, True), g["dist_to_multi_index"])
    assert np.array_equal(pd.pairs_differences_to_point(c[5], c, B, pbc), g["diff_to_point"])
    assert np.array_equal(pd.pairs_differences_to_indexcoords(7, c, B, pbc, True), g["diff_to_index_all"])
    assert np.array_equal(pd.pairs_differences_to_multi_points(pts, c, B, pbc), g["diff_to_multi_points"])
    assert np.array_equal(pd.pairs_differences_to_multi_indexcoords(idx, c, B, pbc, True), g["diff_to_multi_index"])
    assert np.array_equal(pd.from_to_points_differences(c, np.ascontiguousarray(c[::-1]), B, pbc), g["from_to"])
    assert F(pd.point_to_point_distance(c[1], c[2], B, pbc)) == g["p2p"]
    assert np.array_equal(pd.pair_difference_to_point(c[1], c[2], B, pbc), g["pair_diff"])


def test_golden_single_and_dists(gpu):
    g = golden("single_and_dists")
    src = golden("general_triclinic_ne4_mol")
    mol, el = src["mol"], src["el"]
    mn, mx, b, hs = src["minD"], src["maxD"], src["bin"], int(src["hs"])
    ph = gpu.pairs_histograms
    for tag, atom, allAtoms in (("a", 100, True), ("b", 650, False)):
        hi, he = g["h0_intra"].copy(), g["h0_inter"].copy()
        assert ph.single_pairs_histograms(atom, g["dist_" + tag], mol, el, hi, he, mn, mx, b, allAtoms) is None
        assert np.array_equal(hi, g["intra_" + tag]) and np.array_equal(he, g["inter_" + tag])
    hi, he = ph.multiple_pairs_histograms_dists(g["dm_indexes"], g["dm"], mol, el, 4, mn, mx, b, hs, True)
    assert np.array_equal(hi, g["mdist_intra"]) and np.array_equal(he, g["mdist_inter"])
    hi, he = ph.full_pairs_histograms_dists(g["dsq"], mol[:40], el[:40], 4, mn, mx, b, hs)
    assert np.array_equal(hi, g["fdist_intra"]) and np.array_equal(he, g["fdist_inter"])


def test_golden_transform(gpu):
    g = golden("transform")
    bcc = gpu.boundary_conditions_collection
    assert np.array_equal(bcc.transform_coordinates(g["rbasis"], g["real"]), g["box"])
    assert np.array_equal(bcc.transform_coordinates(g["basis"], g["box"]), g["back"])


# --------------------------------------------------------- seeded systems
def _basis(kind, L):
    if kind == "cubic":
        return np.diag([L, L, L]).astype(F), True
    if kind == "xytri":
        return np.array([[L, 0, 0], [-L / 2, L * np.sin(np.radians(120)), 0], [0, 0, L]], F), True
    if kind == "lower":
        return np.array([[L, 0, 0], [0.2 * L, 0.95 * L, 0], [0.1 * L, -0.15 * L, 0.9 * L]], F), True
    if kind == "general":
        return np.array([[L, 0.05 * L, 0.02 * L], [0.2 * L, 0.95 * L, 0.01 * L], [0.1 * L, -0.15 * L, 0.9 * L]],
                        F), True
    return np.eye(3, dtype=F), False


def _system(seed, n, ne, kind, molsize=1, L=None, rmax=10.0):
    rng = np.random.default_rng(seed)
    L = L or (n / 0.1) ** (1 / 3)
    B, pbc = _basis(kind, L)
    coords = rng.random((n, 3)).astype(F) if pbc else (rng.random((n, 3)) * L).astype(F)
    mol = (np.arange(n) // molsize).astype(np.int32)
    el = rng.integers(0, ne, n).astype(np.int32)
    x = np.arange(0, rmax + 1e-4, 0.01).astype(F)
    b = F(x[1] - x[0])
    return dict(boxCoords=coords, basis=B, isPBC=pbc, moleculeIndex=mol, elementIndex=el, numberOfElements=ne,
                minDistance=F(x[0] - b / 2), maxDistance=F(x[-1] + b / 2), bin=b, histSize=len(x))


TUNES = [dict(threads=512, rows=2, queued=1), dict(threads=512, rows=2, queued=0), dict(threads=256, rows=1, queued=1),
         dict(threads=1024, rows=1, queued=0, qcap=8)]


@pytest.mark.parametrize("kind", ["cubic", "xytri", "lower", "general", "ibc"])
@pytest.mark.parametrize("tune", range(len(TUNES)))
def test_full_tiled_vs_oracle(gpu, oracle_mod, kind, tune):
    a = _system(11 + tune, 4099, 3, kind, molsize=4)
    set_tune(min_pairs=0, **TUNES[tune])
    got = gpu.pairs_histograms.full_pairs_histograms_coords(**a)
    set_tune()
    want = oracle_mod.full_pairs_histograms_coords(**a)
    assert got[1].sum() > 0
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("ne", [1, 2, 4])
def test_full_rows_kernel_vs_oracle(gpu, oracle_mod, ne):
    a = _system(5 + ne, 1500, ne, "general", molsize=13)
    got = gpu.pairs_histograms.full_pairs_histograms_coords(**a)
    want = oracle_mod.full_pairs_histograms_coords(**a)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("k", [1, 13, 200])
@pytest.mark.parametrize("allAtoms", [True, False])
def test_multiple_vs_oracle(gpu, oracle_mod, k, allAtoms):
    a = _system(99 + k, 5000, 2, "xytri", molsize=13, rmax=15.0)
    idx = np.random.default_rng(k).choice(5000, size=k, replace=False).astype(np.int32)
    got = gpu.pairs_histograms.multiple_pairs_histograms_coords(indexes=idx, allAtoms=allAtoms, **a)
    want = oracle_mod.multiple_pairs_histograms_coords(indexes=idx, allAtoms=allAtoms, **a)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_move_delta_matches_reference_formula(gpu, oracle_mod):
    """compute_before_move's M - F (PairDistributionConstraints.py:1053-1078)
    for a 13-atom molecule, GPU vs oracle."""
    a = _system(3, 4000, 3, "cubic", molsize=13)
    rel = np.arange(13 * 9, 13 * 10, dtype=np.int32)
    out = []
    for mod in (gpu.pairs_histograms, oracle_mod):
        iM, eM = mod.multiple_pairs_histograms_coords(indexes=rel, allAtoms=True, **a)
        sub = dict(a, boxCoords=a["boxCoords"][rel], moleculeIndex=a["moleculeIndex"][rel],
                   elementIndex=a["elementIndex"][rel])
        iF, eF = mod.full_pairs_histograms_coords(**sub)
        out.append((iM - iF, eM - eF))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_distances_random_vs_oracle(gpu, oracle_mod):
    a = _system(21, 3000, 1, "general")
    c, B = a["boxCoords"], a["basis"]
    idx = np.array([0, 5, 2999], np.int32)
    assert np.array_equal(gpu.pairs_distances.pairs_distances_to_multi_indexcoords(idx, c, B, True, True),
                          oracle_mod.pairs_distances_to_multi_indexcoords(idx, c, B, True, True))
    assert np.array_equal(gpu.pairs_distances.pairs_differences_to_multi_indexcoords(idx, c, B, True, True),
                          oracle_mod.pairs_differences_to_multi_indexcoords(idx, c, B, True, True))


# ------------------------------------------------------------ FP64 transforms
def test_fp64_sine_transforms(gpu, oracle_mod):
    g = golden("reciprocal")
    r, q = g["r"], g["q"]
    rs = gpu.reciprocal_space
    for got, want in ((rs.gr_to_sq(r, g["gr"], q, g["rho"]), oracle_mod.gr_to_sq_fp64(r, g["gr"], q, g["rho"])),
                      (rs.Gr_to_sq(r, g["Gr"], q), oracle_mod.Gr_to_sq_fp64(r, g["Gr"], q)),
                      (rs.sq_to_Gr(q, r, g["Gr_to_sq"]), oracle_mod.sq_to_Gr_fp64(q, r, g["Gr_to_sq"]))):
        # 1e-10 relative to the curve's scale (the sums are oscillatory)
        assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))


# ----------------------------------------------------------- error behaviour
def test_index_errors(gpu):
    a = _system(1, 100, 1, "cubic")
    with pytest.raises(IndexError):
        gpu.pairs_histograms.multiple_pairs_histograms_coords(indexes=np.array([100], np.int32), **a)
    with pytest.raises(IndexError):
        gpu.pairs_distances.pairs_distances_to_indexcoords(-1, a["boxCoords"], a["basis"], True)


_COPY_BRANCH = r"""
import sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/oracle", ROOT + "/tests"]
import fullrmc_gb300
import oracle
from fullrmc_gb300 import pairs_histograms as ph
from test_gpu_parity import _system
a = _system(31, 5000, 2, "xytri", molsize=13, rmax=15.0)
for k in (1, 13, 64, 65):
    idx = np.random.default_rng(k).choice(5000, size=k, replace=False).astype(np.int32)
    for allAtoms in (True, False):
        got = ph.multiple_pairs_histograms_coords(indexes=idx, allAtoms=allAtoms, **a)
        want = oracle.multiple_pairs_histograms_coords(indexes=idx, allAtoms=allAtoms, **a)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (k, allAtoms)
print("copy branch ok")
"""


def test_multiple_copy_branch_vs_oracle(gpu):
    """With FRMC_HOST_DIRECT=0 the per-move call copies its inputs to the
    device instead of letting the kernels read the caller's arrays (the path
    of devices without coherent pageable-memory access); run in a fresh
    process, since the switch is read when the library's context is made."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FRMC_HOST_DIRECT="0")
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % root + _COPY_BRANCH], env=env, cwd=root,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "copy branch ok" in r.stdout


def test_fast_path_equals_ctypes_path(gpu):
    """The compiled fast path of the per-move calls gives the ctypes
    wrappers' results bit for bit (same C entry points)."""
    from fullrmc_gb300 import _native
    f = _native.fastcall()
    if f is None:
        pytest.skip("fast path not built")
    a = _system(71, 5000, 3, "xytri", molsize=13, rmax=15.0)
    try:
        for idx in (np.array([17], np.int32), np.arange(13 * 40, 13 * 41, dtype=np.int32)):
            _native._fast = f
            got_m = gpu.pairs_histograms.multiple_pairs_histograms_coords(indexes=idx, allAtoms=True, **a)
            sub = dict(a, boxCoords=a["boxCoords"][idx], moleculeIndex=a["moleculeIndex"][idx],
                       elementIndex=a["elementIndex"][idx])
            got_f = gpu.pairs_histograms.full_pairs_histograms_coords(**sub)
            got_t = gpu.boundary_conditions_collection.transform_coordinates(a["basis"], a["boxCoords"][idx])
            _native._fast = None
            want_m = gpu.pairs_histograms.multiple_pairs_histograms_coords(indexes=idx, allAtoms=True, **a)
            want_f = gpu.pairs_histograms.full_pairs_histograms_coords(**sub)
            want_t = gpu.boundary_conditions_collection.transform_coordinates(a["basis"], a["boxCoords"][idx])
            for g_, w_ in zip(got_m + got_f, want_m + want_f):
                assert g_.dtype == w_.dtype and np.array_equal(g_, w_)
            assert np.array_equal(got_t, want_t)
        _native._fast = f
        with pytest.raises(IndexError):
            gpu.pairs_histograms.multiple_pairs_histograms_coords(indexes=np.array([5000], np.int32), **a)
    finally:
        _native._fast = f
