"""CPU oracle for the pair-distance / histogram path (test infrastructure).

Two parts:

* ``frmc_oracle.c`` -- a plain-C restatement of the reference's float32
  per-pair arithmetic and histogram binning (``Extensions/pairs_distances.pyx``
  and ``Extensions/pairs_histograms.pyx``), loaded here through ctypes and
  exposed with the reference's Python signatures.  Compiled on first use into
  ``oracle/_build/`` with ``gcc -ffp-contract=off``.
* FP64 restatements (numpy float64) of the host-side reductions that turn the
  histograms into G(r), g(r), S(Q) and chi-square:
  ``Constraints/PairDistributionConstraints.py:847-895``,
  ``Constraints/PairCorrelationConstraints.py:126-167``,
  ``Constraints/StructureFactorConstraints.py:302-312,772-822``,
  ``Core/Constraint.py:1363-1395`` and ``Extensions/reciprocal_space.pyx``.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the CUDA library never calls it.

Parity pin: the C restatement is checked bit-for-bit against golden vectors
produced by the compiled reference Cython (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_SO = os.path.join(_BUILD, "libfrmc_oracle.so")
_SRC = os.path.join(HERE, "frmc_oracle.c")
_lock = threading.Lock()
_lib = None

F32P = ctypes.POINTER(ctypes.c_float)
I32P = ctypes.POINTER(ctypes.c_int32)
i64 = ctypes.c_int64
i32 = ctypes.c_int32
f32 = ctypes.c_float
cint = ctypes.c_int


def build() -> str:
    """Compile the C oracle (idempotent)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        tmp = _SO + ".tmp%d" % os.getpid()
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                        "-fno-fast-math", "-o", tmp, _SRC, "-lm"], check=True)
        os.replace(tmp, _SO)
    return _SO


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_SO)
            sig = {
                "oracle_distances_to_indexcoords": [i32, F32P, i64, F32P, cint, cint, F32P],
                "oracle_distances_to_point": [F32P, F32P, i64, F32P, cint, F32P],
                "oracle_distances_to_multi_points": [F32P, i64, i64, F32P, i64, F32P, cint, F32P],
                "oracle_distances_to_multi_indexcoords": [I32P, i64, F32P, i64, F32P, cint, cint, F32P],
                "oracle_point_to_point_distance": [F32P, F32P, F32P, cint],
                "oracle_from_to_points_differences": [F32P, F32P, i64, F32P, cint, F32P],
                "oracle_pair_difference_to_point": [F32P, F32P, F32P, cint, F32P],
                "oracle_differences_to_point": [F32P, F32P, i64, F32P, cint, F32P],
                "oracle_differences_to_indexcoords": [i32, F32P, i64, F32P, cint, cint, F32P],
                "oracle_differences_to_multi_points": [F32P, i64, i64, F32P, i64, F32P, cint, F32P],
                "oracle_differences_to_multi_indexcoords": [I32P, i64, F32P, i64, F32P, cint, cint, F32P],
                "oracle_single_pairs_histograms": [i32, F32P, i64, I32P, I32P, i32, i32, F32P, F32P, f32, f32, f32, cint],
                "oracle_multiple_pairs_histograms_coords": [I32P, i64, F32P, i64, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32, cint, F32P, F32P],
                "oracle_full_pairs_histograms_coords": [F32P, i64, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32, F32P, F32P],
                "oracle_multiple_pairs_histograms_dists": [I32P, i64, F32P, i64, I32P, I32P, i32, f32, f32, f32, i32, cint, F32P, F32P],
                "oracle_transform_coordinates": [F32P, F32P, i64, F32P],
                "oracle_atomic_distances": [I32P, i64, F32P, F32P, i64, F32P, cint, I32P, I32P, i32, F32P, F32P, cint,
                                            cint, F32P, F32P, I32P, I32P],
                "oracle_pair_elements_stats": [I32P, I32P, i64, i32, I32P, I32P],
            }
            for name, args in sig.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = f32 if name == "oracle_point_to_point_distance" else None
            _lib = lib
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a, t=F32P):
    return a.ctypes.data_as(t)


# ------------------------------------------------------------------ distances
def pairs_distances_to_indexcoords(atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1):
    c, b = _f(coords), _f(basis)
    out = np.zeros((c.shape[0],), np.float32)
    _load().oracle_distances_to_indexcoords(int(atomIndex), _p(c), c.shape[0], _p(b), int(bool(isPBC)), int(bool(allAtoms)), _p(out))
    return out


def pairs_distances_to_point(point, coords, basis, isPBC, ncores=1):
    p, c, b = _f(point), _f(coords), _f(basis)
    out = np.empty((c.shape[0],), np.float32)
    _load().oracle_distances_to_point(_p(p), _p(c), c.shape[0], _p(b), int(bool(isPBC)), _p(out))
    return out


def pairs_distances_to_multi_points(points, coords, basis, isPBC, ncores=1):
    p, c, b = _f(points), _f(coords), _f(basis)
    K = p.shape[1]
    out = np.empty((c.shape[0], K), np.float32)
    _load().oracle_distances_to_multi_points(_p(p), K, K, _p(c), c.shape[0], _p(b), int(bool(isPBC)), _p(out))
    return out


def pairs_distances_to_multi_indexcoords(indexes, coords, basis, isPBC, allAtoms=True, ncores=1):
    ix, c, b = _i(indexes), _f(coords), _f(basis)
    out = np.zeros((c.shape[0], ix.shape[0]), np.float32)
    _load().oracle_distances_to_multi_indexcoords(_p(ix, I32P), ix.shape[0], _p(c), c.shape[0], _p(b), int(bool(isPBC)), int(bool(allAtoms)), _p(out))
    return out


def point_to_point_distance(point1, point2, basis, isPBC, ncores=1):
    p1, p2, b = _f(point1), _f(point2), _f(basis)
    return _load().oracle_point_to_point_distance(_p(p1), _p(p2), _p(b), int(bool(isPBC)))


# ---------------------------------------------------------------- differences
def from_to_points_differences(pointsFrom, pointsTo, basis, isPBC, ncores=1):
    a, t, b = _f(pointsFrom), _f(pointsTo), _f(basis)
    out = np.empty((a.shape[0], 3), np.float32)
    _load().oracle_from_to_points_differences(_p(a), _p(t), a.shape[0], _p(b), int(bool(isPBC)), _p(out))
    return out


def pair_difference_to_point(point1, point2, basis, isPBC, ncores=1):
    p1, p2, b = _f(point1), _f(point2), _f(basis)
    out = np.empty((3,), np.float32)
    _load().oracle_pair_difference_to_point(_p(p1), _p(p2), _p(b), int(bool(isPBC)), _p(out))
    return out


def pairs_differences_to_point(point, coords, basis, isPBC, ncores=1):
    p, c, b = _f(point), _f(coords), _f(basis)
    out = np.empty((c.shape[0], 3), np.float32)
    _load().oracle_differences_to_point(_p(p), _p(c), c.shape[0], _p(b), int(bool(isPBC)), _p(out))
    return out


def pairs_differences_to_indexcoords(atomIndex, coords, basis, isPBC, allAtoms=True, ncores=1):
    c, b = _f(coords), _f(basis)
    out = np.zeros((c.shape[0], 3), np.float32)
    _load().oracle_differences_to_indexcoords(int(atomIndex), _p(c), c.shape[0], _p(b), int(bool(isPBC)), int(bool(allAtoms)), _p(out))
    return out


def pairs_differences_to_multi_points(points, coords, basis, isPBC, ncores=1):
    p, c, b = _f(points), _f(coords), _f(basis)
    K = p.shape[1]
    out = np.empty((c.shape[0], 3, K), np.float32)
    _load().oracle_differences_to_multi_points(_p(p), K, K, _p(c), c.shape[0], _p(b), int(bool(isPBC)), _p(out))
    return out


def pairs_differences_to_multi_indexcoords(indexes, coords, basis, isPBC, allAtoms=True, ncores=1):
    ix, c, b = _i(indexes), _f(coords), _f(basis)
    out = np.zeros((c.shape[0], 3, ix.shape[0]), np.float32)
    _load().oracle_differences_to_multi_indexcoords(_p(ix, I32P), ix.shape[0], _p(c), c.shape[0], _p(b), int(bool(isPBC)), int(bool(allAtoms)), _p(out))
    return out


# ----------------------------------------------------------------- histograms
def single_pairs_histograms(atomIndex, distances, moleculeIndex, elementIndex, hintra, hinter,
                            minDistance, maxDistance, bin, allAtoms=True, ncores=1):
    d, m, e = _f(distances), _i(moleculeIndex), _i(elementIndex)
    assert hintra.flags.c_contiguous and hintra.dtype == np.float32
    assert hinter.flags.c_contiguous and hinter.dtype == np.float32
    ne, hs = hintra.shape[0], hintra.shape[2]
    _load().oracle_single_pairs_histograms(int(atomIndex), _p(d), d.shape[0], _p(m, I32P), _p(e, I32P), ne, hs,
                                           _p(hintra), _p(hinter), np.float32(minDistance), np.float32(maxDistance),
                                           np.float32(bin), int(bool(allAtoms)))


def multiple_pairs_histograms_coords(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex,
                                     numberOfElements, minDistance, maxDistance, bin, histSize,
                                     allAtoms=True, ncores=1):
    ix, c, b, m, e = _i(indexes), _f(boxCoords), _f(basis), _i(moleculeIndex), _i(elementIndex)
    ne, hs = int(numberOfElements), int(histSize)
    hi = np.zeros((ne, ne, hs), np.float32)
    he = np.zeros((ne, ne, hs), np.float32)
    _load().oracle_multiple_pairs_histograms_coords(_p(ix, I32P), ix.shape[0], _p(c), c.shape[0], _p(b), int(bool(isPBC)),
                                                    _p(m, I32P), _p(e, I32P), ne, np.float32(minDistance),
                                                    np.float32(maxDistance), np.float32(bin), hs, int(bool(allAtoms)),
                                                    _p(hi), _p(he))
    return hi, he


def full_pairs_histograms_coords(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                                 minDistance, maxDistance, bin, histSize, ncores=1):
    c, b, m, e = _f(boxCoords), _f(basis), _i(moleculeIndex), _i(elementIndex)
    ne, hs = int(numberOfElements), int(histSize)
    hi = np.zeros((ne, ne, hs), np.float32)
    he = np.zeros((ne, ne, hs), np.float32)
    _load().oracle_full_pairs_histograms_coords(_p(c), c.shape[0], _p(b), int(bool(isPBC)), _p(m, I32P), _p(e, I32P), ne,
                                                np.float32(minDistance), np.float32(maxDistance), np.float32(bin), hs,
                                                _p(hi), _p(he))
    return hi, he


def multiple_pairs_histograms_dists(indexes, distances, moleculeIndex, elementIndex, numberOfElements,
                                    minDistance, maxDistance, bin, histSize, allAtoms=True, ncores=1):
    ix, d, m, e = _i(indexes), _f(distances), _i(moleculeIndex), _i(elementIndex)
    ne, hs = int(numberOfElements), int(histSize)
    hi = np.zeros((ne, ne, hs), np.float32)
    he = np.zeros((ne, ne, hs), np.float32)
    assert d.shape[1] >= ix.shape[0]
    # the reference reads column i of `distances` for indexes[i]
    dk = np.ascontiguousarray(d[:, :ix.shape[0]])
    _load().oracle_multiple_pairs_histograms_dists(_p(ix, I32P), ix.shape[0], _p(dk), dk.shape[0], _p(m, I32P),
                                                   _p(e, I32P), ne, np.float32(minDistance), np.float32(maxDistance),
                                                   np.float32(bin), hs, int(bool(allAtoms)), _p(hi), _p(he))
    return hi, he


def full_pairs_histograms_dists(distances, moleculeIndex, elementIndex, numberOfElements, minDistance,
                                maxDistance, bin, histSize, ncores=1):
    d = _f(distances)
    ix = np.arange(d.shape[1], dtype=np.int32)
    return multiple_pairs_histograms_dists(ix, d, moleculeIndex, elementIndex, numberOfElements, minDistance,
                                           maxDistance, bin, histSize, allAtoms=False)


def transform_coordinates(transMatrix, coords):
    M, c = _f(transMatrix), _f(coords)
    out = np.empty((c.shape[0], 3), np.float32)
    _load().oracle_transform_coordinates(_p(M), _p(c), c.shape[0], _p(out))
    return out


# ----------------------------------------------------------- FP64 reductions
def pair_density_terms(elementsCount, weights):
    """Per unordered species pair (i <= j): (i, j, w_ij, N_ij).

    ``N_ij = n_i (n_i - 1) / 2`` for i == j and ``n_i n_j`` otherwise,
    ``Constraints/PairDistributionConstraints.py:864-878``.  ``weights`` is a
    symmetric (ne, ne) array of w_ij."""
    ne = len(elementsCount)
    out = []
    for i in range(ne):
        for j in range(i, ne):
            ni, nj = float(elementsCount[i]), float(elementsCount[j])
            Nij = ni * (ni - 1.0) / 2.0 if i == j else ni * nj
            out.append((i, j, float(weights[i][j]), Nij))
    return out


def pair_counts_fp64(intra, inter, i, j):
    """n_ij(r): PairDistributionConstraints.py:869,875."""
    intra = np.asarray(intra, np.float64)
    inter = np.asarray(inter, np.float64)
    if i == j:
        return intra[i, i] + inter[i, i]
    return intra[i, j] + intra[j, i] + inter[i, j] + inter[j, i]


def total_gr_fp64(intra, inter, elementsCount, weights, volume, shellVolumes):
    """g(r) = sum_ij w_ij n_ij / (N_ij / V) / v(r): PairDistributionConstraints.py:859-881
    (the same weighted sum is PairCorrelationConstraints.py:130-152)."""
    hs = np.asarray(intra).shape[2]
    g = np.zeros(hs, np.float64)
    for i, j, w, Nij in pair_density_terms(elementsCount, weights):
        g += w * pair_counts_fp64(intra, inter, i, j) / (Nij / float(volume))
    return g / np.asarray(shellVolumes, np.float64)


def total_Gr_fp64(intra, inter, elementsCount, weights, volume, shellVolumes, shellCenters, rho0):
    """G(r) = 4 pi r rho0 (g(r) - 1): PairDistributionConstraints.py:881-884."""
    g = total_gr_fp64(intra, inter, elementsCount, weights, volume, shellVolumes)
    r = np.asarray(shellCenters, np.float64)
    return (4.0 * np.pi * r * float(rho0)) * (g - 1.0)


def gr2sq_matrix_fp64(shellCenters, qValues):
    """M[r, q] = dr sin(q r) / q: StructureFactorConstraints.py:302-312."""
    r = np.asarray(shellCenters, np.float64)
    q = np.asarray(qValues, np.float64)
    dr = r[1] - r[0]
    return dr * np.sin(np.outer(r, q)) / q


def sq_from_Gr_fp64(Gr, matrix, reduced=False):
    """S(q) = sum_r G(r) M[r, q] + 1: StructureFactorConstraints.py:772-773
    (ReducedStructureFactorConstraint drops the +1, :1255-1256)."""
    s = np.asarray(Gr, np.float64) @ np.asarray(matrix, np.float64)
    return s if reduced else s + 1.0


def standard_error_fp64(experimental, model, dataWeights=None):
    """sum w (exp - model)^2: PairDistributionConstraints.py:810-838."""
    diff = np.asarray(experimental, np.float64) - np.asarray(model, np.float64)
    if dataWeights is None:
        return float(np.sum(diff * diff))
    return float(np.sum(np.asarray(dataWeights, np.float64) * diff * diff))


def fit_scale_factor_fp64(experimental, model, dataWeights=None, lo=0.0, hi=np.inf):
    """sum(w m e) / sum(m^2), clamped: Core/Constraint.py:1363-1395."""
    e = np.asarray(experimental, np.float64)
    m = np.asarray(model, np.float64)
    num = np.sum(m * e) if dataWeights is None else np.sum(np.asarray(dataWeights, np.float64) * m * e)
    sf = num / np.sum(m * m)
    return float(min(max(sf, lo), hi))


def window_same_fp64(x, window):
    """numpy.convolve(x, window, 'same') in float64:
    PairDistributionConstraints.py:891-893, PairCorrelationConstraints.py:167-168."""
    return np.convolve(np.asarray(x, np.float64), np.asarray(window, np.float64), "same")


def pdc_model_fp64(intra, inter, elementsCount, weights, volume, shellVolumes, shellCenters, rho0, scale,
                   window=None):
    """The PairDistributionConstraint's model: total G(r), times the scale
    factor, convolved with the window (PairDistributionConstraints.py:847-895;
    no shape function, no multiframe prior)."""
    G = scale * total_Gr_fp64(intra, inter, elementsCount, weights, volume, shellVolumes, shellCenters, rho0)
    return G if window is None else window_same_fp64(G, window)


def pcf_model_fp64(intra, inter, elementsCount, weights, volume, shellVolumes, shellCenters, rho0, scale,
                   window=None):
    """The PairCorrelationConstraint's model: total g(r); with a scale factor
    g -> 1 + s G / (4 pi r rho0) with G = 4 pi r rho0 (g - 1); then the window
    (PairCorrelationConstraints.py:126-169).  Where 4 pi r rho0 is 0 (r = 0)
    the reference divides 0 by 0; there the restatement keeps 1 + s (g - 1)."""
    g = total_gr_fp64(intra, inter, elementsCount, weights, volume, shellVolumes)
    if scale != 1:
        c = 4.0 * np.pi * np.asarray(shellCenters, np.float64) * float(rho0)
        G = c * (g - 1.0) * scale
        safe = np.where(c != 0.0, c, 1.0)
        g = np.where(c != 0.0, 1.0 + G / safe, 1.0 + scale * (g - 1.0))
    return g if window is None else window_same_fp64(g, window)


def pcf_fit_scale_factor_fp64(experimental, g, shellCenters, rho0, dataWeights=None, lo=0.0, hi=np.inf):
    """PairCorrelationConstraint's fit: on G(r) = 4 pi r rho0 (g - 1) of both
    curves (PairCorrelationConstraints.py:171-184)."""
    c = 4.0 * np.pi * np.asarray(shellCenters, np.float64) * float(rho0)
    return fit_scale_factor_fp64(c * (np.asarray(experimental, np.float64) - 1.0), c * (np.asarray(g, np.float64) - 1.0),
                                 dataWeights, lo, hi)


def gr_to_sq_fp64(distances, gr, qrange, rho):
    """reciprocal_space.pyx:42-73 in float64."""
    r = np.asarray(distances, np.float64)
    q = np.asarray(qrange, np.float64)
    dr = r[1] - r[0]
    fact = 4.0 * np.pi * float(rho)
    return 1.0 + fact * ((dr * r * (np.asarray(gr, np.float64) - 1.0)) @ (np.sin(np.outer(r, q)) / q))


def Gr_to_sq_fp64(distances, Gr, qrange):
    """reciprocal_space.pyx:82-109 in float64."""
    r = np.asarray(distances, np.float64)
    q = np.asarray(qrange, np.float64)
    dr = r[1] - r[0]
    return 1.0 + (dr * np.asarray(Gr, np.float64)) @ (np.sin(np.outer(r, q)) / q)


def sq_to_Gr_fp64(qValues, rValues, sq):
    """reciprocal_space.pyx:118-145 in float64."""
    q = np.asarray(qValues, np.float64)
    r = np.asarray(rValues, np.float64)
    dq = q[1] - q[0]
    qs = q * (np.asarray(sq, np.float64) - 1.0)
    return (2.0 / np.pi) * (np.sin(np.outer(r, q)) * dq) @ qs


# ----------------------------------------------------------- atomic distances
def _atomic_flags(inter, intra, within, red_up, red_lo, red):
    return ((1 if inter else 0) | (2 if intra else 0) | (4 if within else 0) | (8 if red_up else 0) |
            (16 if red_lo else 0) | (32 if red else 0))


def _atomic(indexes, coords, dists, n, basis, isPBC, mol, el, ne, lower, upper, flags, allAtoms, acc=None):
    ix, m, e = _i(indexes), _i(mol), _i(el)
    lo, up = _f(lower), _f(upper)
    if acc is None:
        acc = (np.zeros((ne, ne, 1), np.int32), np.zeros((ne, ne, 1), np.float32),
               np.zeros((ne, ne, 1), np.int32), np.zeros((ne, ne, 1), np.float32))
    ni, di, nn, de = acc
    c = _f(coords) if coords is not None else None
    d = _f(dists) if dists is not None else None
    b = _f(basis) if basis is not None else np.eye(3, dtype=np.float32)
    _load().oracle_atomic_distances(_p(ix, I32P), ix.shape[0], _p(c) if c is not None else None,
                                    _p(d) if d is not None else None, n, _p(b), int(bool(isPBC)), _p(m, I32P),
                                    _p(e, I32P), ne, _p(lo), _p(up), flags, int(bool(allAtoms)), _p(di), _p(de),
                                    _p(ni, I32P), _p(nn, I32P))
    return ni, di, nn, de


def multiple_atomic_distances_coords(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                                     lowerLimit, upperLimit, interMolecular=True, intraMolecular=True,
                                     countWithinLimits=True, reduceDistanceToUpper=False, reduceDistanceToLower=False,
                                     reduceDistance=False, allAtoms=True, ncores=1):
    """atomic_distances.pyx:326-417; returns (nintra, dintra, ninter, dinter)."""
    c = _f(boxCoords)
    fl = _atomic_flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                       reduceDistance)
    return _atomic(indexes, c, None, c.shape[0], basis, isPBC, moleculeIndex, elementIndex, int(numberOfElements),
                   lowerLimit, upperLimit, fl, allAtoms)


def full_atomic_distances_coords(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, lowerLimit,
                                 upperLimit, interMolecular=True, intraMolecular=True, reduceDistanceToUpper=False,
                                 reduceDistanceToLower=False, reduceDistance=False, countWithinLimits=True, ncores=1):
    """atomic_distances.pyx:500-567."""
    c = _f(boxCoords)
    return multiple_atomic_distances_coords(np.arange(c.shape[0], dtype=np.int32), c, basis, isPBC, moleculeIndex,
                                            elementIndex, numberOfElements, lowerLimit, upperLimit, interMolecular,
                                            intraMolecular, countWithinLimits, reduceDistanceToUpper,
                                            reduceDistanceToLower, reduceDistance, allAtoms=False)


def multiple_atomic_distances_dists(indexes, distances, moleculeIndex, elementIndex, numberOfElements, lowerLimit,
                                    upperLimit, interMolecular=True, intraMolecular=True, countWithinLimits=True,
                                    reduceDistanceToUpper=False, reduceDistanceToLower=False, reduceDistance=False,
                                    allAtoms=True, ncores=1):
    """atomic_distances.pyx:419-498 (column i of distances for indexes[i])."""
    ix = _i(indexes)
    d = np.ascontiguousarray(_f(distances)[:, :ix.shape[0]])
    fl = _atomic_flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                       reduceDistance)
    return _atomic(ix, None, d, d.shape[0], None, False, moleculeIndex, elementIndex, int(numberOfElements),
                   lowerLimit, upperLimit, fl, allAtoms)


def full_atomic_distances_dists(distances, moleculeIndex, elementIndex, numberOfElements, lowerLimit, upperLimit,
                                interMolecular=True, intraMolecular=True, reduceDistanceToUpper=False,
                                reduceDistanceToLower=False, reduceDistance=False, countWithinLimits=True):
    """atomic_distances.pyx:569-630."""
    d = _f(distances)
    return multiple_atomic_distances_dists(np.arange(d.shape[1], dtype=np.int32), d, moleculeIndex, elementIndex,
                                           numberOfElements, lowerLimit, upperLimit, interMolecular, intraMolecular,
                                           countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                                           reduceDistance, allAtoms=False)


def single_atomic_distances_dists(atomIndex, distances, moleculeIndex, elementIndex, dintra, dinter, nintra, ninter,
                                  lowerLimit, upperLimit, interMolecular=True, intraMolecular=True,
                                  countWithinLimits=True, reduceDistanceToUpper=False, reduceDistanceToLower=False,
                                  reduceDistance=False, allAtoms=True, ncores=1):
    """atomic_distances.pyx:241-324 (in place)."""
    d = np.ascontiguousarray(_f(distances).reshape(-1, 1))
    fl = _atomic_flags(interMolecular, intraMolecular, countWithinLimits, reduceDistanceToUpper, reduceDistanceToLower,
                       reduceDistance)
    _atomic(np.array([atomIndex], np.int32), None, d, d.shape[0], None, False, moleculeIndex, elementIndex,
            dintra.shape[0], lowerLimit, upperLimit, fl, allAtoms, acc=(nintra, dintra, ninter, dinter))


def pair_elements_stats(elementIndex, moleculeIndex, numberOfElements):
    """atomic_distances.pyx:659-672."""
    e, m = _i(elementIndex), _i(moleculeIndex)
    ne = int(numberOfElements)
    ni = np.zeros((ne, ne, 1), np.int32)
    nn = np.zeros((ne, ne, 1), np.int32)
    _load().oracle_pair_elements_stats(_p(e, I32P), _p(m, I32P), e.shape[0], ne, _p(ni, I32P), _p(nn, I32P))
    return ni, nn


# -------------------------------------------------------- atomic coordination
# Restatement of Extensions/atomic_coordination.pyx, loop for loop, on top of
# the C distance restatement above (numpy for the window counts).
def _shell_count(distances, lowerShell, upperShell):
    """_single_atom_single_shell_dists (atomic_coordination.pyx:31-44): 1.0f
    added once per distance inside [lowerShell, upperShell]; a float32 sum of
    ones is exact up to 2^24 and stays at 2^24 beyond."""
    d = np.asarray(distances, np.float32)
    lo, up = np.float32(float(lowerShell)), np.float32(float(upperShell))
    k = int(np.count_nonzero((lo <= d) & (d <= up)))
    return np.float32(min(k, 1 << 24))


def single_atom_single_shell_subdists(distances, lowerShell, upperShell, ncores=1):
    """atomic_coordination.pyx:55-65."""
    return float(_shell_count(distances, lowerShell, upperShell))


def single_atom_single_shell_totdists(distances, shellIndexes, lowerShell, upperShell, ncores=1):
    """atomic_coordination.pyx:71-80."""
    return float(_shell_count(np.asarray(distances)[np.asarray(shellIndexes)], lowerShell, upperShell))


def _core_distances(coreIndex, shellIndexes, boxCoords, basis, isPBC):
    """pairs_distances_to_point(boxCoords[coreIndex], boxCoords[shellIndexes])
    (atomic_coordination.pyx:98-102)."""
    c = _f(boxCoords)
    pts = np.ascontiguousarray(c[np.asarray(shellIndexes)])
    return pairs_distances_to_point(c[int(coreIndex)], pts, basis, isPBC)


def single_atom_single_shell_coords(coreIndex, shellIndexes, boxCoords, basis, isPBC, lowerShell, upperShell,
                                    ncores=1):
    """atomic_coordination.pyx:89-108."""
    return float(_shell_count(_core_distances(coreIndex, shellIndexes, boxCoords, basis, isPBC), lowerShell,
                              upperShell))


def single_atom_multi_shells_totdists(distances, shellsIndexes, lowerShells, upperShells, ncores=1):
    """atomic_coordination.pyx:116-133."""
    out = np.zeros(len(shellsIndexes), np.float32)
    for i in range(len(shellsIndexes)):
        out[i] = _shell_count(np.asarray(distances)[np.asarray(shellsIndexes[i])], lowerShells[i], upperShells[i])
    return out


def single_atom_multi_shells_coords(coreIndex, shellsIndexes, boxCoords, basis, isPBC, lowerShells, upperShells,
                                    ncores=1):
    """atomic_coordination.pyx:139-166."""
    out = np.zeros(len(shellsIndexes), np.float32)
    for i in range(len(shellsIndexes)):
        out[i] = _shell_count(_core_distances(coreIndex, shellsIndexes[i], boxCoords, basis, isPBC), lowerShells[i],
                              upperShells[i])
    return out


def _add(coordNumData, defIdx, count):
    """coordNumData[defIdx] += coordNumber in float32."""
    coordNumData[defIdx] = np.float32(coordNumData[defIdx]) + count


def single_atom_coord_number_totdists(atomIndex, distances, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                      asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:171-198: both loops walk asCoreDefIdxs."""
    d = np.asarray(distances)
    for defIdx in asCoreDefIdxs[atomIndex]:
        _add(coordNumData, defIdx, _shell_count(d[np.asarray(shellsIndexes[defIdx])], lowerShells[defIdx],
                                                upperShells[defIdx]))
    for defIdx in asCoreDefIdxs[atomIndex]:
        _add(coordNumData, defIdx, _shell_count(d[np.asarray(coresIndexes[defIdx])], lowerShells[defIdx],
                                                upperShells[defIdx]))


def single_atom_coord_number_coords(atomIndex, boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells,
                                    upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:207-240."""
    for defIdx in asCoreDefIdxs[atomIndex]:
        d = _core_distances(atomIndex, shellsIndexes[defIdx], boxCoords, basis, isPBC)
        _add(coordNumData, defIdx, _shell_count(d, lowerShells[defIdx], upperShells[defIdx]))
    for defIdx in inShellDefIdxs[atomIndex]:
        d = _core_distances(atomIndex, coresIndexes[defIdx], boxCoords, basis, isPBC)
        _add(coordNumData, defIdx, _shell_count(d, lowerShells[defIdx], upperShells[defIdx]))


def multi_atoms_coord_number_totdists(indexes, distances, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                      asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:249-278."""
    for i in range(len(indexes)):
        single_atom_coord_number_totdists(int(indexes[i]), distances[i], coresIndexes, shellsIndexes, lowerShells,
                                          upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData)


def multi_atoms_coord_number_coords(indexes, boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells,
                                    upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:280-309."""
    for i in range(len(indexes)):
        single_atom_coord_number_coords(int(indexes[i]), boxCoords, basis, isPBC, coresIndexes, shellsIndexes,
                                        lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData)


def all_atoms_coord_number_totdists(distances, coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs,
                                    inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:317-347: the 2-D array reaches a ``list``
    argument, so the call raises TypeError."""
    raise TypeError("Argument 'distances' has incorrect type (expected list, got numpy.ndarray)")


def all_atoms_coord_number_coords(boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                  asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """atomic_coordination.pyx:349-377."""
    multi_atoms_coord_number_coords(np.arange(np.asarray(boxCoords).shape[0], dtype=np.int32), boxCoords, basis,
                                    isPBC, coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs,
                                    inShellDefIdxs, coordNumData)


# -------------------------------------------------------------- shape function
def _normalized_weights(counts, b):
    """w_ij = (2 - delta_ij) c_i c_j b_i b_j / (sum_k c_k b_k)^2, the element-pair
    weights of PairDistributionConstraints.py:66-86 (pdbparser's
    get_normalized_weighting, not installed, implements this definition)."""
    n = np.asarray(counts, np.float64)
    bb = np.asarray(b, np.float64)
    c = n / n.sum()
    s = (c * bb).sum()
    return np.outer(c * bb, c * bb) / (s * s) * (2.0 - np.eye(len(n)))


def shape_function_grids(qmin, qmax, dq, rmin, rmax, dr):
    """Collection.py:64-75 (Q) and StructureFactorConstraints.py:336-350, 502-575 (edges)."""
    F = np.float32
    Q = np.arange(F(qmin), F(qmax), F(dq)).astype(F)
    mn, mx, b = F(rmin), F(rmax), F(dr)
    edges = np.arange(mn, F(mx + b), b).astype(F)
    centers = ((edges[:-1] + edges[1:]) / F(2.0)).astype(F)
    return Q, edges, centers, b


def shape_function_fp64(boxCoords, basis, isPBC, mol, el, counts, b, volume, rValues, qmin, qmax, dq, rmin, rmax,
                        dr):
    """The ShapeFunction chain in float64 on the oracle's histogram:
    (Gshape on rValues, G on the shells, S on Q)."""
    Q, edges, centers, bin_ = shape_function_grids(qmin, qmax, dq, rmin, rmax, dr)
    hs = len(edges) - 1
    intra, inter = full_pairs_histograms_coords(boxCoords, basis, isPBC, mol, el, len(counts), edges[0], edges[-1],
                                                bin_, hs)
    e = edges.astype(np.float64)
    vol = 4.0 / 3.0 * np.pi * (e[1:] ** 3 - e[:-1] ** 3)
    w = _normalized_weights(counts, b)
    rho0 = float(np.asarray(boxCoords).shape[0]) / float(volume)
    G = total_Gr_fp64(intra, inter, counts, w, volume, vol, centers, rho0)
    S = sq_from_Gr_fp64(G, gr2sq_matrix_fp64(centers, Q))
    return sq_to_Gr_fp64(Q, rValues, S), G, S


def shape_function_f32_port(boxCoords, basis, isPBC, mol, el, counts, b, volume, rValues, qmin, qmax, dq, rmin,
                            rmax, dr):
    """The reference's own float32 arithmetic (StructureFactorConstraints.py:
    302-312, 346-350, 836-896 and Collection.py:131-139), for a loose check of
    the formulas: Gshape on rValues (float32)."""
    F = np.float32
    PI = F(np.pi)
    Q, edges, centers, bin_ = shape_function_grids(qmin, qmax, dq, rmin, rmax, dr)
    hs = len(edges) - 1
    intra, inter = full_pairs_histograms_coords(boxCoords, basis, isPBC, mol, el, len(counts), edges[0], edges[-1],
                                                bin_, hs)
    vol = F(4.0 / 3.) * PI * ((edges[1:]) ** 3 - edges[0:-1] ** 3)
    w = _normalized_weights(counts, b).astype(F)
    gr = np.zeros(hs, F)
    V = float(volume)
    for i in range(len(counts)):
        for j in range(i, len(counts)):
            ni, nj = int(counts[i]), int(counts[j])
            Nij = ni * (ni - 1) / 2.0 if i == j else ni * nj
            nij = intra[i, j] + inter[i, j] if i == j else intra[i, j] + intra[j, i] + inter[i, j] + inter[j, i]
            gr += w[i, j] * (nij / vol) / (Nij / V)
    rho0 = F(np.asarray(boxCoords).shape[0] / V)
    Gr = (F(4.) * PI * centers * rho0) * (gr - 1)
    drr = centers[1] - centers[0]
    qr = centers.reshape((-1, 1)) * (np.ones((len(centers), 1), dtype=F) * Q)
    M = drr * (np.sin(qr) / Q)
    Sq = np.sum(Gr.reshape((-1, 1)) * M, axis=0) + 1
    out = np.zeros(len(rValues), F)
    qsq_1 = Q * (Sq - 1)
    dqq = Q[1] - Q[0]
    for k, r in enumerate(np.asarray(rValues, F)):
        out[k] = (2. / PI) * np.sum(qsq_1 * (dqq * np.sin(Q * r)))
    return out
