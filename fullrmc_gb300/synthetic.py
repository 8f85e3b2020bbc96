"""Seeded synthetic systems with the shapes of the benchmark configurations.

No dataset is involved: coordinates are uniform random from a seed, and
each engine's target G(r) is a seeded synthetic curve.  All sizes follow the
workload definitions:

* ``alloy_5000``: 5,000 atoms, two species 50/50, cubic box of side 38.2 A,
  r 0-15 A, dr 0.01 A.
* ``triclinic_100k``: 100,000 atoms, three species 0.5/0.3/0.2, triclinic box
  a = b = c = 103 A, alpha = beta = 90, gamma = 120 degrees, r 0-20 A.
* ``mixed_engines``: 256 engines, atom counts log-uniform in [1,000, 20,000],
  1-4 species, cubic or triclinic boxes at 0.08-0.10 atoms/A^3, r 0-12 A.
* ``ring_molecules``: rigid five-membered rings (4 C + 1 O, bond 1.5 A; 8 H
  at C-H 1.1 A), 13 atoms each, randomly placed and oriented in a cubic box
  at 0.1 atoms/A^3 (4,000 of them = 52,000 atoms), moved as whole groups;
  r 0-15 A, dr 0.01 (the G(r) grid is not fixed by the configuration).
* ``serving_fit``: one fit of the serving stream: atoms log-uniform in
  [2,000, 200,000], 1-3 species, G(r) on r 0-12 A and S(Q) on Q 0.5-25 A^-1
  (dQ 0.01, 2451 points), 2,000-50,000 steps.
"""
from __future__ import annotations

import numpy as np

from .engine import EngineSystem, PDFModel, SQModel, normalized_weighting

F32 = np.float32


def r_grid(rmax, dr=0.01):
    return np.arange(0.0, rmax + dr / 10.0, dr).astype(F32)


def triclinic(a, b, c, alpha, beta, gamma):
    """Row-vector basis with a along x and b in the xy plane (exact zeros kept)."""
    al, be, ga = np.radians([alpha, beta, gamma])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    B = np.array([[a, 0, 0], [b * np.cos(ga), b * np.sin(ga), 0], [cx, cy, cz]], np.float64)
    B[np.abs(B) < 1e-9 * max(a, b, c)] = 0.0
    return B.astype(F32)


def transform_f32(M, coords):
    """coords . M in float32 with the reference's operation order."""
    M = np.asarray(M, F32)
    c = np.asarray(coords, F32)
    out = np.empty_like(c)
    for k in range(3):
        out[:, k] = (c[:, 0] * M[0, k] + c[:, 1] * M[1, k]) + c[:, 2] * M[2, k]
    return out


def species(rng, n, fractions):
    counts = np.floor(np.asarray(fractions, np.float64) * n).astype(int)
    counts[0] += n - counts.sum()
    el = np.repeat(np.arange(len(fractions)), counts).astype(np.int32)
    rng.shuffle(el)
    return el


def synthetic_G(rng, r, rho):
    """A damped liquid-like G(r) with seeded shape: 4 pi r rho (g - 1),
    g(r) = 1 + A exp(-r / lam) sin(2 pi (r - r0) / d) / r beyond a core."""
    r64 = r.astype(np.float64)
    A = rng.uniform(0.8, 1.6)
    lam = rng.uniform(2.0, 4.0)
    d = rng.uniform(2.5, 3.5)
    r0 = rng.uniform(2.0, 2.6)
    g = np.where(r64 < r0 * 0.85, 0.0, 1.0 + A * np.exp(-(r64 - r0) / lam) * np.cos(2 * np.pi * (r64 - r0) / d))
    G = 4 * np.pi * r64 * rho * (g - 1.0)
    return (G + rng.normal(0.0, 0.01, size=r.shape)).astype(F32)


def q_grid(qmin=0.5, qmax=25.0, dq=0.01):
    return (qmin + dq * np.arange(int(round((qmax - qmin) / dq)) + 1)).astype(F32)


def synthetic_S(rng, sq, G_target):
    """Experimental S(Q) of a target G(r): its transform on the S(Q) shells
    plus N(0, 0.01) noise, float32 like read data."""
    S = np.asarray(G_target, np.float64) @ sq.M + 1.0
    return (S + rng.normal(0.0, 0.01, size=S.shape)).astype(F32)


def make_system(rng, n, fractions, basis, rmax, molsize=1, isPBC=True, target=None, q=None):
    """One engine system: seeded coordinates, elements, molecules and an FP64
    PDF model; with `q` (Q values) also an S(Q) term on the same histograms."""
    basis = np.asarray(basis, F32)
    rbasis = np.linalg.inv(basis.astype(np.float64)).astype(F32)
    frac = rng.random((n, 3))
    real = (frac @ basis.astype(np.float64)).astype(F32)
    # box coordinates as fullrmc derives them from the real ones
    # (Engine.py:2265 -> boundary_conditions_collection.pyx:104-106, float32)
    box = transform_f32(rbasis, real)
    el = species(rng, n, fractions)
    mol = (np.arange(n) // molsize).astype(np.int32)
    volume = abs(float(np.linalg.det(basis.astype(np.float64))))
    r = r_grid(rmax)
    counts = np.bincount(el, minlength=len(fractions))
    weights = normalized_weighting(counts, np.ones(len(fractions)) + 0.25 * np.arange(len(fractions)))
    G = synthetic_G(rng, r, n / volume) if target is None else target
    model = PDFModel(r=r, G_exp=G, elements_count=counts, weights=weights, volume=volume)
    sq = None
    if q is not None:
        sq = SQModel(pdf=model, q=q, S_exp=np.zeros(len(q)))
        sq.S_exp = synthetic_S(rng, sq, G)
    return EngineSystem(box_coords=box, real_coords=real, el=el, mol=mol, basis=basis, rbasis=rbasis,
                        isPBC=isPBC, model=model, sq=sq)


def alloy_5000(seed=0, n=5000):
    rng = np.random.default_rng(seed)
    L = 38.2 * (n / 5000.0) ** (1.0 / 3.0)
    return make_system(rng, n, [0.5, 0.5], np.diag([L, L, L]), 15.0)


def triclinic_100k(seed=0, n=100000):
    rng = np.random.default_rng(seed)
    a = 103.0 * (n / 100000.0) ** (1.0 / 3.0)
    return make_system(rng, n, [0.5, 0.3, 0.2], triclinic(a, a, a, 90, 90, 120), 20.0)


def mixed_engines(seed=0, count=256, nmin=1000, nmax=20000, rmax=12.0):
    """``count`` engines with log-uniform sizes, 1-4 species, cubic or
    triclinic boxes at 0.08-0.10 atoms/A^3."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        ns = int(rng.integers(1, 5))
        fr = rng.dirichlet(np.ones(ns) * 3.0)
        rho = rng.uniform(0.08, 0.10)
        if rng.random() < 0.5:
            L = (n / rho) ** (1.0 / 3.0)
            B = np.diag([L, L, L])
        else:
            al, be, ga = rng.uniform(80, 100), rng.uniform(80, 100), rng.uniform(95, 120)
            unit = triclinic(1.0, 1.0, 1.0, al, be, ga).astype(np.float64)
            vol1 = abs(np.linalg.det(unit))
            a = (n / rho / vol1) ** (1.0 / 3.0)
            B = triclinic(a, a, a, al, be, ga)
        out.append(make_system(np.random.default_rng([seed, k]), n, fr, B, rmax))
    return out


def random_box(rng, n, rho):
    """Cubic (half the time) or triclinic box holding n atoms at density rho."""
    if rng.random() < 0.5:
        L = (n / rho) ** (1.0 / 3.0)
        return np.diag([L, L, L])
    al, be, ga = rng.uniform(80, 100), rng.uniform(80, 100), rng.uniform(95, 120)
    unit = triclinic(1.0, 1.0, 1.0, al, be, ga).astype(np.float64)
    a = (n / rho / abs(np.linalg.det(unit))) ** (1.0 / 3.0)
    return triclinic(a, a, a, al, be, ga)


def serving_fit(seed, nmin=2000, nmax=200000, smin=2000, smax=50000, rmax=12.0, sq=True):
    """One request of the serving stream: (system, steps)."""
    rng = np.random.default_rng([seed, 7])
    n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
    ns = int(rng.integers(1, 4))
    fr = rng.dirichlet(np.ones(ns) * 3.0)
    B = random_box(rng, n, rng.uniform(0.08, 0.10))
    steps = int(rng.integers(smin, smax + 1))
    return make_system(rng, n, fr, B, rmax, q=q_grid() if sq else None), steps


def _ring_template():
    """One 13-atom ring molecule: 4 C, 1 O on a regular pentagon with 1.5 A
    bonds, and 2 H on each C at 1.1 A, above and below the ring plane."""
    R = 1.5 / (2.0 * np.sin(np.radians(36.0)))
    ang = np.radians(72.0 * np.arange(5))
    ring = np.stack([R * np.cos(ang), R * np.sin(ang), np.zeros(5)], axis=1)
    th = np.radians(54.75)
    hs = []
    for k in range(4):
        radial = ring[k] / np.linalg.norm(ring[k])
        for sgn in (1.0, -1.0):
            hs.append(ring[k] + 1.1 * (np.cos(th) * radial + sgn * np.sin(th) * np.array([0.0, 0.0, 1.0])))
    xyz = np.concatenate([ring, np.array(hs)])
    el = np.array([0, 0, 0, 0, 1] + [2] * 8, np.int32)
    return xyz - xyz.mean(axis=0), el


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def ring_molecules(seed=0, nmol=4000, rho=0.1, rmax=15.0):
    """Molecular system of rigid 13-atom rings moved as groups (see above)."""
    rng = np.random.default_rng([seed, 13])
    xyz0, el0 = _ring_template()
    n = 13 * nmol
    L = (n / rho) ** (1.0 / 3.0)
    basis = np.diag([L, L, L]).astype(F32)
    real = np.empty((n, 3))
    for m in range(nmol):
        real[13 * m:13 * m + 13] = xyz0 @ _random_rotation(rng).T + rng.random(3) * L
    real = real.astype(F32)
    rbasis = np.linalg.inv(basis.astype(np.float64)).astype(F32)
    box = transform_f32(rbasis, real)
    el = np.tile(el0, nmol)
    mol = np.repeat(np.arange(nmol), 13).astype(np.int32)
    counts = np.bincount(el, minlength=3)
    volume = float(L) ** 3
    weights = normalized_weighting(counts, np.array([6.0, 8.0, 1.0]))
    r = r_grid(rmax)
    G = synthetic_G(rng, r, n / volume)
    model = PDFModel(r=r, G_exp=G, elements_count=counts, weights=weights, volume=volume)
    return EngineSystem(box_coords=box, real_coords=real, el=el, mol=mol, basis=basis, rbasis=rbasis, isPBC=True,
                        model=model, group_size=13, groups=np.arange(n, dtype=np.int32).reshape(nmol, 13))
