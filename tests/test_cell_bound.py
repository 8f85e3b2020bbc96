"""The column grids' distance bound, on the CPU: for boxes of every shape, the
lower bound the engine step uses to skip a cell (from frmc_cell_metric and
the per-axis gaps of two bounding boxes) never exceeds the reference's
float32 minimum-image distance (the oracle) between any points of the two
boxes by more than float32 rounding -- far below the step's margin
(1e-2 A + 1e-4 maxD)."""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401


@pytest.fixture(scope="module")
def lib():
    from fullrmc_gb300 import build
    build.build()
    from fullrmc_gb300 import engine
    return engine


def _metric(lib, B, pbc):
    return lib.cell_metric(B, pbc)


def _gap(a, b, pbc):
    """Distance from [a, b] to the nearest integer (periodic) or to zero."""
    if not pbc:
        return a if a > 0 else (-b if b < 0 else 0.0)
    n = np.floor(b)
    return 0.0 if n >= a else min(a - n, n + 1.0 - b)


def _bound(alo, ahi, blo, bhi, w, lam, mode, pbc):
    f = np.array([_gap(float(alo[k]) - float(bhi[k]), float(ahi[k]) - float(blo[k]), pbc) for k in range(3)])
    m = f * w
    lb2 = float((m * m).sum()) if mode == 0 else max(float((m * m).max()), lam * float((f * f).sum()))
    return np.sqrt(lb2)


def _basis(kind):
    from fullrmc_gb300 import synthetic
    if kind == "cubic":
        return np.diag([31.0, 31.0, 31.0]), True
    if kind == "orthorhombic":
        return np.diag([22.0, 37.0, 29.0]), True
    if kind == "hexagonal":
        return synthetic.triclinic(30.0, 30.0, 34.0, 90, 90, 120), True
    if kind == "triclinic":
        return synthetic.triclinic(33.0, 29.0, 31.0, 84, 97, 112), True
    if kind == "skewed":
        return synthetic.triclinic(40.0, 36.0, 30.0, 70, 75, 128), True
    if kind == "general":
        return np.array([[25.0, 3.0, -2.0], [4.0, 27.0, 1.5], [-3.0, 2.5, 30.0]]), True
    return np.eye(3), False  # free boundaries: box coordinates are real coordinates


@pytest.mark.parametrize("kind", ["cubic", "orthorhombic", "hexagonal", "triclinic", "skewed", "general", "free"])
def test_cell_bound_below_reference_distance(lib, oracle_mod, kind):
    B, pbc = _basis(kind)
    B32 = np.asarray(B, np.float32)
    w, lam, mode = _metric(lib, B32, pbc)
    rng = np.random.default_rng([7, sum(map(ord, kind))])
    span = 1.0 if pbc else 30.0
    worst, close = -np.inf, 0
    for _ in range(300):
        a0 = rng.uniform(-1.5, 2.5, 3) * span
        ea = rng.uniform(0.0, 0.25, 3) * span
        # the second box near the first, often an integer number of boxes away
        shift = rng.uniform(-0.6, 0.6, 3) * span + (rng.integers(-2, 3, 3) if pbc else 0)
        b0 = a0 + shift
        eb = rng.uniform(0.0, 0.25, 3) * span
        pa = (a0 + ea * rng.random((24, 3))).astype(np.float32)
        pb = (b0 + eb * rng.random((48, 3))).astype(np.float32)
        alo, ahi, blo, bhi = pa.min(0), pa.max(0), pb.min(0), pb.max(0)
        lb = _bound(alo, ahi, blo, bhi, w, lam, mode, pbc)
        d = min(float(oracle_mod.pairs_distances_to_point(p, pb, B32, pbc).min()) for p in pa)
        worst = max(worst, lb - d)
        close += lb > 0.5 * d > 0
    assert worst <= 1e-3, worst
    assert close > 20  # the bound is not trivially zero


def test_cell_metric_values(lib):
    """Orthorhombic: w = the edges; hexagonal cell: w = perpendicular widths,
    lam = 0.999 of the smallest eigenvalue of B B^T; free boundaries: w = 1."""
    from fullrmc_gb300 import synthetic
    w, lam, mode = _metric(lib, np.diag([22.0, 37.0, 29.0]), True)
    assert mode == 0 and np.allclose(w, [22.0, 37.0, 29.0])
    B = np.asarray(synthetic.triclinic(30.0, 30.0, 34.0, 90, 90, 120), np.float32).astype(np.float64)
    w, lam, mode = _metric(lib, B, True)
    inv = np.linalg.inv(B)
    assert mode == 1
    assert np.allclose(w, 1.0 / np.linalg.norm(inv, axis=0), rtol=1e-6)
    assert np.isclose(lam, 0.999 * np.linalg.eigvalsh(B @ B.T).min(), rtol=1e-6)
    w, lam, mode = _metric(lib, np.eye(3), False)
    assert mode == 0 and np.allclose(w, 1.0)
