"""ShapeFunction (fullrmc Constraints/Collection.py:15-160) in FP64.

CPU: the oracle's float64 chain agrees with a port of the reference's own
float32 arithmetic (to float32 accuracy), and the grids follow the
reference's construction.  GPU: frmc_shape_function agrees with the oracle's
float64 chain to 1e-10 of the curve's largest value, for a finite cluster
(infinite boundary conditions, the case the shape function exists for) and
a periodic box, through the function and through the engine-style class.
"""
import types

import numpy as np
import pytest

F = np.float32


def _cluster(seed=3, n=600, ne=3, R=14.0):
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(4 * n, 3))
    pts = pts[np.linalg.norm(pts, axis=1) < 2.0][:n]
    real = (pts * (R / 2.0)).astype(F)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    mol = np.arange(n, dtype=np.int32)
    counts = np.bincount(el, minlength=ne)
    volume = 4.0 / 3.0 * np.pi * R ** 3
    return real, np.eye(3, dtype=F), False, mol, el, counts, np.array([6.0, 8.0, 14.0])[:ne], volume


def _box(seed=4, n=800, ne=2, L=22.0):
    rng = np.random.default_rng(seed)
    box = rng.random((n, 3)).astype(F)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    mol = (np.arange(n) // 4).astype(np.int32)
    return box, np.diag([L, L, L]).astype(F), True, mol, el, np.bincount(el, minlength=ne), np.array([5.0, 9.0]), L ** 3


GRID = dict(qmin=0.02, qmax=1.5, dq=0.01, rmin=0.0, rmax=40.0, dr=0.5)
RV = np.arange(0.05, 40.0, 0.1).astype(F)


def test_grids_follow_reference(oracle_mod):
    Q, edges, centers, b = oracle_mod.shape_function_grids(**GRID)
    assert Q.dtype == F and edges.dtype == F and centers.dtype == F
    assert np.array_equal(Q, np.arange(F(0.02), F(1.5), F(0.01)).astype(F))
    assert edges[0] == F(0.0) and edges[-1] == F(40.0) and len(edges) == 81
    from fullrmc_gb300 import shape_function as sf
    Q2, e2, c2, mn, mx, b2, hs = sf.shape_function_grids(**GRID)
    assert np.array_equal(Q, Q2) and np.array_equal(edges, e2) and np.array_equal(centers, c2)
    assert hs == 80 and b2 == b


@pytest.mark.parametrize("system", [_cluster, _box])
def test_oracle_fp64_matches_reference_float32_arithmetic(oracle_mod, system):
    args = system()
    g64, G, S = oracle_mod.shape_function_fp64(*args, RV, **GRID)
    g32 = oracle_mod.shape_function_f32_port(*args, RV, **GRID)
    scale = np.abs(g64).max()
    assert scale > 0
    assert np.abs(g64 - g32).max() <= 2e-3 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("system", [_cluster, _box])
def test_device_matches_oracle_fp64(oracle_mod, system):
    from fullrmc_gb300 import shape_function as sf
    args = system()
    want, G0, S0 = oracle_mod.shape_function_fp64(*args, RV, **GRID)
    got, info = sf.gr_shape_function(*args, RV, **GRID, details=True)
    for a, b in ((got, want), (info["Gr"], G0), (info["Sq"], S0)):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()


@pytest.mark.gpu
def test_shape_function_class_on_an_engine_like_object(oracle_mod):
    from fullrmc_gb300.shape_function import ShapeFunction
    real, B, isPBC, mol, el, counts, b, volume = _cluster(seed=8, n=900)
    eng = types.SimpleNamespace(boxCoordinates=real, basisVectors=B, isPBC=isPBC, moleculesIndex=mol,
                                elementsIndex=el, elements=["C", "O", "Si"],
                                numberOfAtomsPerElement={"C": int(counts[0]), "O": int(counts[1]),
                                                         "Si": int(counts[2])}, volume=volume)
    shp = ShapeFunction(eng, weights={"C": b[0], "O": b[1], "Si": b[2]}, **GRID)
    got = shp.get_Gr_shape_function(RV)
    want, _, _ = oracle_mod.shape_function_fp64(real, B, isPBC, mol, el, counts, b, volume, RV, **GRID)
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()
    g = shp.get_gr_shape_function(RV)
    rho0 = real.shape[0] / volume
    assert np.allclose(g, got / (4.0 * np.pi * rho0 * RV.astype(np.float64)), rtol=1e-14, atol=0)
