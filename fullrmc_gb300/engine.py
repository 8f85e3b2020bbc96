"""Device-resident RMC engines (the batched path) over ``frmc_engines_*``.

An engine is one fullrmc Metropolis chain with a PairDistributionConstraint
and optionally a StructureFactorConstraint on the same histograms, whose
whole state -- coordinates, oriented histogram counts, experimental curves,
chi2 -- lives in HBM.  A batched step
advances every engine of a set by one move in one kernel launch (captured in
a CUDA graph for runs of steps); ``step(engine=e)`` advances one engine alone
(the plain one-engine-at-a-time GPU path).  Moves are generated on the host
by seeded per-engine streams and pushed into device rings ahead of the steps,
so each chain is strictly sequential and gives the same accept sequence,
chi2 values and counts alone or in any batch.

Host-side set-up follows fullrmc's constraint definitions:
``PairDistributionConstraints.py:726-774`` (limits, edges, shell volumes),
``:847-895`` (G(r) from the histograms), ``StructureFactorConstraints.py``
``:302-312`` and ``:780-822`` (S(Q) from G(r)) and ``Engine.py:3000-3029`` /
``Core/Constraint.py`` (chi2 = sum of standard error / varianceSquared); these
constants are FP64.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from ._native import F32P, F64P, I32P, check, load, register

F32 = np.float32


class _Spec(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("ne", ctypes.c_int32), ("hs", ctypes.c_int32), ("isPBC", ctypes.c_int32),
                ("box_coords", F32P), ("real_coords", F32P), ("el", I32P), ("mol", I32P), ("basis", F32P),
                ("rbasis", F32P), ("minDistance", ctypes.c_float), ("maxDistance", ctypes.c_float),
                ("bin", ctypes.c_float), ("npairs", ctypes.c_int32), ("pair_i", I32P), ("pair_j", I32P),
                ("pair_coef", F64P), ("rfac", F64P), ("inv_shell_volume", F64P), ("experimental", F64P),
                ("data_weights", F64P), ("variance_squared", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("move_cap", ctypes.c_int32), ("sq_table", ctypes.c_int32), ("nq", ctypes.c_int32),
                ("sq_rfac", F64P), ("sq_inv_shell_volume", F64P), ("sq_experimental", F64P),
                ("sq_variance_squared", ctypes.c_double), ("sq_rho0", ctypes.c_double),
                ("group_size", ctypes.c_int32), ("scale_factor", ctypes.c_double), ("fit_frequency", ctypes.c_int32),
                ("fit_min", ctypes.c_double), ("fit_max", ctypes.c_double), ("fit_num", F64P), ("fit_den", F64P),
                ("window_len", ctypes.c_int32), ("window", F64P)]


_vp = ctypes.c_void_p
_i32, _i64 = ctypes.c_int32, ctypes.c_int64
register("frmc_engine_footprint", [ctypes.POINTER(_Spec), ctypes.POINTER(_i64)])
register("frmc_engines_new", [ctypes.POINTER(_vp)])
register("frmc_engines_create", [ctypes.POINTER(_Spec), _i32, ctypes.POINTER(_vp)])
register("frmc_engines_add", [_vp, ctypes.POINTER(_Spec), ctypes.POINTER(_i32)])
register("frmc_engines_remove", [_vp, _i32])
register("frmc_engines_live", [_vp, I32P, _i32, ctypes.POINTER(_i32)])
register("frmc_engines_step_host", [_vp, I32P, F32P, F32P, F64P, I32P])
# host-step array arguments as raw addresses (ndarray.ctypes.data): these
# calls run once per step, where building ctypes pointer objects shows up
register("frmc_engines_step_host_submit", [_vp, _vp, _vp, _vp, ctypes.c_int32])
register("frmc_engines_step_host_collect", [_vp, ctypes.c_int32, _vp, _vp])
register("frmc_engines_destroy", [_vp])
register("frmc_engines_set_tune", [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int])
register("frmc_engines_get_tune", [_vp] + [ctypes.POINTER(ctypes.c_int)] * 4)
register("frmc_engines_set_mode", [_vp, ctypes.c_int])
register("frmc_engines_set_cells", [_vp, ctypes.c_int32])
register("frmc_engines_cells", [_vp, _i32, ctypes.POINTER(_i32), ctypes.POINTER(_i64)])
register("frmc_engines_regrid", [_vp, _i32])
register("frmc_cell_metric", [F32P, _i32, F64P, F64P, ctypes.POINTER(_i32)])
register("frmc_engines_set_sq_gemm_limit", [_vp, ctypes.c_int32])
register("frmc_engines_set_sq_splits", [_vp, ctypes.c_int32])
register("frmc_engines_init", [_vp])
register("frmc_engines_push_moves", [_vp, _i32, I32P, F32P, F32P, _i32, _i64, ctypes.c_int])
register("frmc_engines_step", [_vp, _i32, _i32, ctypes.c_int, _vp])
register("frmc_engines_place", [_vp, _i32])
register("frmc_engines_place_positions", [_i32, I32P, F64P, I32P])
register("frmc_engines_push_group_moves", [_vp, _i32, I32P, I32P, F32P, F32P, _i32, _i64])
register("frmc_engines_sync", [_vp])
register("frmc_engines_state", [_vp, _i32, F64P, ctypes.POINTER(_i64), ctypes.POINTER(_i64)])
register("frmc_engines_results", [_vp, _i32, _i64, _i32, F64P, I32P, I32P])
register("frmc_engines_counts", [_vp, _i32, I32P])
register("frmc_engines_coords", [_vp, _i32, F32P, F32P])
register("frmc_engines_info", [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i64), ctypes.POINTER(_i64)])
register("frmc_engines_sq_table", [_vp, _i32, _i32, F64P, F64P, F64P, ctypes.POINTER(_i32)])
register("frmc_engines_sq", [_vp, _i32, F64P])
register("frmc_engines_terms", [_vp, _i32, F64P, F64P])


def normalized_weighting(counts, scattering):
    """w_ij = (2 - delta_ij) c_i c_j b_i b_j / (sum_k c_k b_k)^2, c_i = n_i / N.

    The definition of the element-pair weights in fullrmc's documentation
    (PairDistributionConstraints.py:66-86); sum_{i<=j} w_ij = 1."""
    n = np.asarray(counts, np.float64)
    b = np.asarray(scattering, np.float64)
    c = n / n.sum()
    s = (c * b).sum()
    w = np.outer(c * b, c * b) / (s * s)
    w = w * (2.0 - np.eye(len(n)))
    return w


def window_same(x, window):
    """numpy.convolve(x, window, 'same') in FP64."""
    return np.convolve(np.asarray(x, np.float64), np.asarray(window, np.float64), "same")


@dataclass
class PDFModel:
    """FP64 constants of one PairDistributionConstraint (kind "pdf": G(r),
    PairDistributionConstraints.py:847-895) or PairCorrelationConstraint
    (kind "gr": g(r), PairCorrelationConstraints.py:126-184) on an r grid.

    scale_factor, adjust_scale_factor = (frequency, minimum, maximum) and
    window follow the constraints' arguments (Core/Constraint.py:981-1235):
    the model is window * (s G) for G(r), and window * (1 + s (g - 1)) for
    g(r); s is refitted (clamped) on the proposal whenever the engine's
    accepted count is a multiple of a non-zero frequency, and an accepted
    move keeps its s.  The window is normalized in float32 as fullrmc does.

    On the device both kinds run as G(b) = R(b) S(b) - rfac(b) compared with
    a shifted experimental curve: for g(r), rfac = 1 (so G is g - 1) and the
    curve is g_exp - window * 1 (g_exp - 1 without a window), which leaves
    every deviation unchanged."""
    r: np.ndarray                # experimental r grid (float32, uniform)
    G_exp: np.ndarray            # experimental G(r) (kind "gr": g(r))
    elements_count: np.ndarray   # atoms per element index
    weights: np.ndarray          # (ne, ne) symmetric w_ij
    volume: float
    data_weights: np.ndarray | None = None
    variance_squared: float = 1.0
    kind: str = "pdf"
    scale_factor: float = 1.0
    adjust_scale_factor: tuple = (0, 0.8, 1.2)
    window: np.ndarray | None = None

    def __post_init__(self):
        if self.kind not in ("pdf", "gr"):
            raise ValueError("PDFModel.kind must be 'pdf' or 'gr', got %r" % (self.kind,))
        freq, lo, hi = self.adjust_scale_factor
        if int(freq) < 0 or not float(lo) <= float(hi):
            raise ValueError("adjust_scale_factor must be (frequency >= 0, minimum, maximum >= minimum)")
        self.fit_frequency, self.fit_min, self.fit_max = int(freq), float(lo), float(hi)
        if not np.isfinite(self.scale_factor) or self.scale_factor == 0:
            raise ValueError("scale_factor must be a finite non-zero number")
        x = np.asarray(self.r, F32)
        self.r = x
        b = F32(x[1] - x[0])
        self.bin = b
        self.minDistance = F32(x[0] - b / F32(2.0))
        self.maxDistance = F32(x[-1] + b / F32(2.0))
        edges = np.concatenate([x - b / F32(2.0), [x[-1] + b / F32(2.0)]]).astype(F32)
        self.edges = edges
        self.hs = len(x)
        e64 = edges.astype(np.float64)
        self.shell_volumes = 4.0 / 3.0 * np.pi * (e64[1:] ** 3 - e64[:-1] ** 3)
        n = np.asarray(self.elements_count, np.float64)
        self.n_atoms = int(n.sum())
        self.rho0 = self.n_atoms / float(self.volume)
        cfac = 4.0 * np.pi * x.astype(np.float64) * self.rho0
        self.rfac = cfac if self.kind == "pdf" else np.ones(len(x))
        win = None
        if self.window is not None:
            w32 = np.asarray(self.window, F32).ravel()
            if w32.ndim != 1 or not 0 < len(w32) <= min(255, len(x)):
                raise ValueError("window must be a 1-D array of at most min(255, bins) values")
            w32 = w32 / np.sum(w32)   # Constraints/PairDistributionConstraints.py:700 (float32)
            win = w32.astype(np.float64)
        self.window_fp64 = win
        dw = 1.0 if self.data_weights is None else np.asarray(self.data_weights, np.float64)
        exp = np.asarray(self.G_exp, np.float64)
        if self.kind == "pdf":
            self.exp_dev = exp
            self.fit_num = dw * exp
            self.fit_den = None
        else:
            self.exp_dev = exp - (window_same(np.ones(len(x)), win) if win is not None else 1.0)
            self.fit_num = dw * cfac * cfac * (exp - 1.0)
            self.fit_den = cfac * cfac
        self.dense = self.scale_factor != 1.0 or self.fit_frequency > 0 or win is not None
        ne = len(n)
        pi, pj, pc = [], [], []
        for i in range(ne):
            for j in range(i, ne):
                Nij = n[i] * (n[i] - 1.0) / 2.0 if i == j else n[i] * n[j]
                if Nij <= 0:
                    continue
                pi.append(i)
                pj.append(j)
                pc.append(float(self.weights[i][j]) * float(self.volume) / Nij)
        self.pair_i = np.asarray(pi, np.int32)
        self.pair_j = np.asarray(pj, np.int32)
        self.pair_coef = np.asarray(pc, np.float64)

    def G_fp64(self, intra, inter):
        """G(r) of oriented (ne, ne, hs) counts (the engine's formula, FP64)."""
        intra = np.asarray(intra, np.float64)
        inter = np.asarray(inter, np.float64)
        g = np.zeros(self.hs)
        for i, j, c in zip(self.pair_i, self.pair_j, self.pair_coef):
            if i == j:
                nij = intra[i, i] + inter[i, i]
            else:
                nij = intra[i, j] + intra[j, i] + inter[i, j] + inter[j, i]
            g += c * nij
        g /= self.shell_volumes
        return self.rfac * (g - 1.0)

    def fit_fp64(self, intra, inter):
        """The fitted scale factor of these counts (the device's formula)."""
        G = self.G_fp64(intra, inter)
        den = np.sum((1.0 if self.fit_den is None else self.fit_den) * G * G)
        if not den > 0:
            return None
        return float(min(max(np.sum(self.fit_num * G) / den, self.fit_min), self.fit_max))

    def chi2_fp64(self, intra, inter, scale=None):
        """The G(r) term of chi2 of these counts at scale factor `scale`
        (default: the model's scale_factor), FP64, the device's formula."""
        s = self.scale_factor if scale is None else scale
        u = s * self.G_fp64(intra, inter)
        if self.window_fp64 is not None:
            u = window_same(u, self.window_fp64)
        d = self.exp_dev - u
        w = 1.0 if self.data_weights is None else np.asarray(self.data_weights, np.float64)
        return float(np.sum(w * d * d) / self.variance_squared)


_M_CACHE = {}


def sq_matrix(centers, q):
    """M[r, Q] = dr sin(Q r) / Q in FP64 of the float32 shell centers and Q
    values, dr = r[1] - r[0] (StructureFactorConstraints.py:302-312).  Cached
    per grid, since every fit on the same grids shares it."""
    centers = np.asarray(centers, F32)
    q = np.asarray(q, F32)
    key = (centers.tobytes(), q.tobytes())
    M = _M_CACHE.get(key)
    if M is None:
        r = centers.astype(np.float64)
        q64 = q.astype(np.float64)
        M = (r[1] - r[0]) * np.sin(np.outer(r, q64)) / q64
        M.setflags(write=False)
        if len(_M_CACHE) >= 4:
            _M_CACHE.pop(next(iter(_M_CACHE)))
        _M_CACHE[key] = M
    return M


@dataclass
class SQModel:
    """FP64 constants of one StructureFactorConstraint that shares the
    engine's histograms: its rmin, dr and rmax are the G(r) constraint's
    minDistance, bin and maxDistance, so the pair counts are the same.  Its own
    shells follow StructureFactorConstraints.py:330-360 (edges = arange(rmin,
    rmax + dr, dr) in float32, centers = midpoints, volumes 4/3 pi (e1^3 -
    e0^3)); S(Q) = sum_r G_S(r) M[r, Q] + 1 (:772-822, scale factor 1, no
    window) with G_S = 4 pi r rho0 (g(r) - 1) on those shells and the same
    element-pair weights."""
    pdf: PDFModel
    q: np.ndarray                # experimental Q values (float32)
    S_exp: np.ndarray            # experimental S(Q) (reduced: S(Q) - 1)
    data_weights: np.ndarray | None = None
    variance_squared: float = 1.0
    reduced: bool = False        # ReducedStructureFactorConstraint (StructureFactorConstraints.py:1255-1262)
    scale_factor: float = 1.0
    adjust_scale_factor: tuple = (0, 0.8, 1.2)
    window: np.ndarray | None = None

    def __post_init__(self):
        if self.scale_factor != 1.0 or int(self.adjust_scale_factor[0]) != 0 or self.window is not None:
            raise ValueError("the device engines' S(Q) term has no scale factor, fitted scale factor or window "
                             "(StructureFactorConstraints.py:814-821); use scale_factor=1, "
                             "adjust_scale_factor=(0, ...) and window=None")
        m = self.pdf
        self.q = np.asarray(self.q, F32)
        self.nq = len(self.q)
        self.hs = m.hs
        e = (float(m.minDistance) + float(m.bin) * np.arange(m.hs + 1)).astype(F32)
        self.edges = e
        self.centers = ((e[:-1] + e[1:]) / F32(2.0)).astype(F32)
        e64 = e.astype(np.float64)
        self.shell_volumes = 4.0 / 3.0 * np.pi * (e64[1:] ** 3 - e64[:-1] ** 3)
        self.r0fac = 4.0 * np.pi * self.centers.astype(np.float64) / self.shell_volumes
        self.rfac = 4.0 * np.pi * self.centers.astype(np.float64) * m.rho0
        self.M = sq_matrix(self.centers, self.q)

    def key(self):
        w = None if self.data_weights is None else np.asarray(self.data_weights, np.float64).tobytes()
        return (self.centers.tobytes(), self.q.tobytes(), w)

    def table_bytes(self):
        return 8 * (self.hs * self.nq + self.hs * self.hs + self.hs + 1 +
                    (self.nq if self.data_weights is not None else 0))

    def G_fp64(self, intra, inter):
        m = self.pdf
        intra = np.asarray(intra, np.float64)
        inter = np.asarray(inter, np.float64)
        g = np.zeros(self.hs)
        for i, j, c in zip(m.pair_i, m.pair_j, m.pair_coef):
            if i == j:
                nij = intra[i, i] + inter[i, i]
            else:
                nij = intra[i, j] + intra[j, i] + inter[i, j] + inter[j, i]
            g += c * nij
        g /= self.shell_volumes
        return self.rfac * (g - 1.0)

    def S_fp64(self, intra, inter):
        return self.G_fp64(intra, inter) @ self.M + (0.0 if self.reduced else 1.0)

    def sd_fp64(self, intra, inter):
        d = np.asarray(self.S_exp, np.float64) - self.S_fp64(intra, inter)
        w = 1.0 if self.data_weights is None else np.asarray(self.data_weights, np.float64)
        return float(np.sum(w * d * d))


@dataclass
class EngineSystem:
    box_coords: np.ndarray
    real_coords: np.ndarray
    el: np.ndarray
    mol: np.ndarray
    basis: np.ndarray
    rbasis: np.ndarray
    isPBC: bool
    model: PDFModel
    tolerance: float = 0.0
    keep: list = field(default_factory=list, repr=False)
    sq: SQModel | None = None
    group_size: int = 1              # atoms per move (molecule groups: their size)
    groups: np.ndarray | None = None  # (n_groups, group_size) atom indexes, for group moves

    def chi2_fp64(self, intra, inter):
        """chi2 of the engine's constraints from oriented counts (FP64)."""
        c = self.model.chi2_fp64(intra, inter)
        if self.sq is not None:
            c += self.sq.sd_fp64(intra, inter) / self.sq.variance_squared
        return c


def translation_moves(rng: np.random.Generator, n_atoms: int, count: int, amplitude: float):
    """Single-atom random translations: atom uniform in [0, n), direction
    uniform, length uniform in [0, amplitude) (the distribution of
    TranslationGenerator, Generators/Translations.py:171-190 with
    Core/Collection.py:674-700), plus one uniform per step for the tolerance
    test.  float32, like fullrmc's move vectors."""
    atoms = rng.integers(0, n_atoms, size=count).astype(np.int32)
    v = (1.0 - 2.0 * rng.random((count, 3))).astype(F32)
    norm = np.sqrt((v.astype(np.float64) ** 2).sum(axis=1)).astype(F32)
    norm[norm == 0] = F32(1.0)
    v = v / norm[:, None]
    v = (v * (rng.random(count) * amplitude).astype(F32)[:, None]).astype(F32)
    u = rng.random(count).astype(F32)
    return atoms, np.ascontiguousarray(v), u


def group_moves(rng: np.random.Generator, groups, count: int, amplitude: float, angle: float,
                p_rotation: float = 0.5):
    """Moves of whole groups (molecules), like fullrmc's TranslationGenerator
    (Generators/Translations.py:171-190) and RotationGenerator
    (Generators/Rotations.py:141-178) on molecule groups: a uniformly chosen
    group, then with probability `p_rotation` a rotation about the group's
    centroid by an angle uniform in [-angle, angle] degrees about a uniform
    random axis, else a translation of length uniform in [0, amplitude) in a
    uniform direction.  Returns (atoms (count, G), kinds (count,), params
    (count, 9), u (count,)): params holds the translation vector (first three)
    or the row-vector rotation matrix (x -> x R), float32."""
    groups = np.asarray(groups, np.int32)
    pick = rng.integers(0, groups.shape[0], size=count)
    atoms = np.ascontiguousarray(groups[pick])
    kinds = (rng.random(count) < p_rotation).astype(np.int32)
    params = np.zeros((count, 9), F32)
    for k in range(count):
        if kinds[k]:
            axis = 1.0 - 2.0 * rng.random(3)
            axis /= np.linalg.norm(axis)
            th = np.radians((1.0 - 2.0 * rng.random()) * angle)
            x, y, z = axis
            c, s_, C = np.cos(th), np.sin(th), 1.0 - np.cos(th)
            Rcol = np.array([[c + x * x * C, x * y * C - z * s_, x * z * C + y * s_],
                             [y * x * C + z * s_, c + y * y * C, y * z * C - x * s_],
                             [z * x * C - y * s_, z * y * C + x * s_, c + z * z * C]])
            params[k] = Rcol.T.astype(F32).ravel()   # row-vector convention: x R = (Rcol x)^T
        else:
            v = 1.0 - 2.0 * rng.random(3)
            v /= np.linalg.norm(v)
            params[k, :3] = (v * rng.random() * amplitude).astype(F32)
    u = rng.random(count).astype(F32)
    return atoms, kinds, params, u


def group_new_real(real, kind, params):
    """New real coordinates of a group (float32, the engine's operation
    order): translation real + v, or rotation (x - c) R + c about the
    centroid c (atoms added in group order, divided by the group size)."""
    real = np.asarray(real, F32)
    p = np.asarray(params, F32)
    if kind == 0:
        return (real + p[:3]).astype(F32)
    c = real[0].copy()
    for k in range(1, real.shape[0]):
        c = (c + real[k]).astype(F32)
    c = (c / F32(real.shape[0])).astype(F32)
    R = p.reshape(3, 3)
    d = (real - c).astype(F32)
    out = np.empty_like(real)
    for k in range(3):
        out[:, k] = ((d[:, 0] * R[0, k] + d[:, 1] * R[1, k]) + d[:, 2] * R[2, k]) + c[k]
    return out.astype(F32)


def make_spec(system, move_cap, sq_table=-1):
    """ctypes spec of one system; returns (spec, arrays that must stay alive).
    `sq_table` is the set's table id for the system's S(Q) term."""
    s = system
    m = s.model
    arrs = dict(box=np.ascontiguousarray(s.box_coords, F32), real=np.ascontiguousarray(s.real_coords, F32),
                el=np.ascontiguousarray(s.el, np.int32), mol=np.ascontiguousarray(s.mol, np.int32),
                B=np.ascontiguousarray(s.basis, F32), RB=np.ascontiguousarray(s.rbasis, F32),
                pi=np.ascontiguousarray(m.pair_i), pj=np.ascontiguousarray(m.pair_j),
                pc=np.ascontiguousarray(m.pair_coef), rfac=np.ascontiguousarray(m.rfac),
                iv=np.ascontiguousarray(1.0 / m.shell_volumes),
                ex=np.ascontiguousarray(np.asarray(m.exp_dev, np.float64)),
                dw=None if m.data_weights is None else np.ascontiguousarray(m.data_weights, np.float64))
    sp = _Spec()
    sp.n = arrs["box"].shape[0]
    sp.ne = len(m.elements_count)
    sp.hs = m.hs
    sp.isPBC = int(bool(s.isPBC))
    sp.box_coords = arrs["box"].ctypes.data_as(F32P)
    sp.real_coords = arrs["real"].ctypes.data_as(F32P)
    sp.el = arrs["el"].ctypes.data_as(I32P)
    sp.mol = arrs["mol"].ctypes.data_as(I32P)
    sp.basis = arrs["B"].ctypes.data_as(F32P)
    sp.rbasis = arrs["RB"].ctypes.data_as(F32P)
    sp.minDistance, sp.maxDistance, sp.bin = m.minDistance, m.maxDistance, m.bin
    sp.npairs = len(m.pair_i)
    sp.pair_i = arrs["pi"].ctypes.data_as(I32P)
    sp.pair_j = arrs["pj"].ctypes.data_as(I32P)
    sp.pair_coef = arrs["pc"].ctypes.data_as(F64P)
    sp.rfac = arrs["rfac"].ctypes.data_as(F64P)
    sp.inv_shell_volume = arrs["iv"].ctypes.data_as(F64P)
    sp.experimental = arrs["ex"].ctypes.data_as(F64P)
    sp.data_weights = arrs["dw"].ctypes.data_as(F64P) if arrs["dw"] is not None else None
    sp.variance_squared = float(m.variance_squared)
    sp.tolerance = float(s.tolerance)
    sp.move_cap = int(move_cap)
    sp.group_size = int(getattr(s, "group_size", 1) or 1)
    sp.scale_factor = float(m.scale_factor)
    if m.dense:
        arrs.update(fnum=np.ascontiguousarray(m.fit_num, np.float64),
                    fden=None if m.fit_den is None else np.ascontiguousarray(m.fit_den, np.float64),
                    win=None if m.window_fp64 is None else np.ascontiguousarray(m.window_fp64))
        sp.fit_frequency = m.fit_frequency
        sp.fit_min, sp.fit_max = m.fit_min, m.fit_max
        sp.fit_num = arrs["fnum"].ctypes.data_as(F64P)
        sp.fit_den = arrs["fden"].ctypes.data_as(F64P) if arrs["fden"] is not None else None
        if arrs["win"] is not None:
            sp.window_len = len(arrs["win"])
            sp.window = arrs["win"].ctypes.data_as(F64P)
    sp.sq_table = -1
    if s.sq is not None:
        q = s.sq
        arrs.update(sq_rfac=np.ascontiguousarray(q.rfac), sq_iv=np.ascontiguousarray(1.0 / q.shell_volumes),
                    sq_exp=np.ascontiguousarray(np.asarray(q.S_exp, np.float64) + (1.0 if q.reduced else 0.0)))
        sp.sq_table = int(sq_table)
        sp.nq = q.nq
        sp.sq_rfac = arrs["sq_rfac"].ctypes.data_as(F64P)
        sp.sq_inv_shell_volume = arrs["sq_iv"].ctypes.data_as(F64P)
        sp.sq_experimental = arrs["sq_exp"].ctypes.data_as(F64P)
        sp.sq_variance_squared = float(q.variance_squared)
        sp.sq_rho0 = float(s.model.rho0)
    return sp, arrs


def footprint(system, move_cap):
    """Device bytes an engine of this system occupies (without the S(Q) table
    it shares with other engines on the same grids)."""
    sp, _keep = make_spec(system, move_cap, sq_table=0)
    b = ctypes.c_int64()
    check(load().frmc_engine_footprint(ctypes.byref(sp), ctypes.byref(b)))
    return b.value


def cell_metric(basis, isPBC):
    """(w, lam, mode) of the column grids' distance bound for a basis (host
    only): |g B| >= |g_k| w_k and |g B|^2 >= lam |g|^2 (mode 1), or
    |g B|^2 >= sum (g_k w_k)^2 (mode 0)."""
    B = np.ascontiguousarray(basis, F32)
    w = np.empty(3, np.float64)
    lam, mode = ctypes.c_double(), _i32()
    check(load().frmc_cell_metric(B.ctypes.data_as(F32P), int(bool(isPBC)), w.ctypes.data_as(F64P),
                                  ctypes.byref(lam), ctypes.byref(mode)))
    return w, lam.value, mode.value


class EngineSet:
    """A set of device-resident engines stepped together or one at a time."""

    def __init__(self, systems=(), move_cap: int = 4096, tune=None, cells: bool = True):
        """cells: give engines a column grid where it pays (the one-CTA step
        then sweeps only the cells a moved atom may reach; results are
        identical either way)."""
        load()
        self.move_cap = int(move_cap)
        self.systems = {}
        self._stage_E = [None, None]
        self.tables = {}
        h = ctypes.c_void_p()
        systems = list(systems)
        if not cells or any(s.sq is not None for s in systems):
            # S(Q) tables must exist before their engines: add one by one
            check(load().frmc_engines_new(ctypes.byref(h)))
            self.handle = h
            check(load().frmc_engines_set_cells(h, 1 if cells else 0))
            for s in systems:
                self.add(s)
        elif systems:
            specs = (_Spec * len(systems))()
            keep = []
            for k, s in enumerate(systems):
                sp, arrs = make_spec(s, self.move_cap)
                specs[k] = sp
                keep.append(arrs)
            check(load().frmc_engines_create(specs, len(systems), ctypes.byref(h)))
            self.systems = {k: s for k, s in enumerate(systems)}
        else:
            check(load().frmc_engines_new(ctypes.byref(h)))
        self.handle = h
        if tune is not None:
            self.set_tune(*tune)

    def sq_table(self, sq):
        """Id of the device table of an SQModel's grids (created once per set)."""
        key = sq.key()
        t = self.tables.get(key)
        if t is None:
            w = None if sq.data_weights is None else np.ascontiguousarray(sq.data_weights, np.float64)
            M = np.ascontiguousarray(sq.M, np.float64)
            r0 = np.ascontiguousarray(sq.r0fac, np.float64)
            i = ctypes.c_int32()
            check(load().frmc_engines_sq_table(self.handle, sq.hs, sq.nq, M.ctypes.data_as(F64P),
                                               None if w is None else w.ctypes.data_as(F64P),
                                               r0.ctypes.data_as(F64P), ctypes.byref(i)))
            t = self.tables[key] = i.value
        return t

    @property
    def E(self):
        return len(self.systems)

    def add(self, system, move_cap=None):
        """Add (and initialise) one engine; returns its id."""
        tid = self.sq_table(system.sq) if system.sq is not None else -1
        sp, _keep = make_spec(system, move_cap or self.move_cap, tid)
        i = ctypes.c_int32()
        check(load().frmc_engines_add(self.handle, ctypes.byref(sp), ctypes.byref(i)))
        self.systems[i.value] = system
        return i.value

    def remove(self, e):
        check(load().frmc_engines_remove(self.handle, int(e)))
        self.systems.pop(int(e), None)

    def live(self):
        ids = np.empty(max(1, len(self.systems)), np.int32)
        c = ctypes.c_int32()
        check(load().frmc_engines_live(self.handle, ids.ctypes.data_as(I32P), len(ids), ctypes.byref(c)))
        return ids[:c.value].copy()

    def step_host(self, atoms, vecs, u):
        """One batched step of all live engines from host arrays (live-id order);
        returns (chi2_new, accepted)."""
        E = len(self.systems)
        atoms = np.ascontiguousarray(atoms, np.int32)
        vecs = np.ascontiguousarray(vecs, F32)
        u = np.ascontiguousarray(u, F32)
        if atoms.size != E or vecs.size != 3 * E or u.size != E:
            raise ValueError("step_host: need %d atoms, (%d, 3) vectors and %d numbers, got %s, %s, %s"
                             % (E, E, E, atoms.shape, vecs.shape, u.shape))
        c2 = np.empty(E, np.float64)
        acc = np.empty(E, np.int32)
        check(load().frmc_engines_step_host(self.handle, atoms.ctypes.data_as(I32P), vecs.ctypes.data_as(F32P),
                                            u.ctypes.data_as(F32P), c2.ctypes.data_as(F64P),
                                            acc.ctypes.data_as(I32P)))
        return c2, acc

    def step_host_submit(self, atoms, vecs, u, slot):
        """Submit one batched step from host arrays into staging slot 0 or 1
        (step_host in two halves: a host may submit step k + 1 before it
        collects step k)."""
        E = len(self.systems)
        atoms = np.ascontiguousarray(atoms, np.int32)
        vecs = np.ascontiguousarray(vecs, F32)
        u = np.ascontiguousarray(u, F32)
        if atoms.size != E or vecs.size != 3 * E or u.size != E:
            raise ValueError("step_host_submit: need %d atoms, (%d, 3) vectors and %d numbers, got %s, %s, %s"
                             % (E, E, E, atoms.shape, vecs.shape, u.shape))
        check(load().frmc_engines_step_host_submit(self.handle, atoms.ctypes.data, vecs.ctypes.data,
                                                   u.ctypes.data, int(slot)))
        self._stage_E[int(slot)] = E

    def step_host_collect(self, slot, out=None):
        """Wait for the step in `slot`; returns (chi2_new, accepted) in live-id
        order, into `out` = (float64 array, int32 array) of the live-engine
        count when given.  Engines cannot be added or removed while a step is
        in flight (the library refuses), so the count is the submitted one."""
        E = self._stage_E[int(slot)] if slot in (0, 1) and self._stage_E[int(slot)] is not None else len(self.systems)
        if out is None:
            c2, acc = np.empty(E, np.float64), np.empty(E, np.int32)
        else:
            c2, acc = out
            if (c2.dtype != np.float64 or acc.dtype != np.int32 or c2.size != E or acc.size != E
                    or not c2.flags.c_contiguous or not acc.flags.c_contiguous):
                raise ValueError("step_host_collect: out must be contiguous float64 and int32 arrays of %d" % E)
        check(load().frmc_engines_step_host_collect(self.handle, int(slot), c2.ctypes.data, acc.ctypes.data))
        self._stage_E[int(slot)] = None
        return c2, acc

    # ------------------------------------------------------------ control
    def set_tune(self, tile, threads, ctas_per_sm):
        check(load().frmc_engines_set_tune(self.handle, int(tile), int(threads), int(ctas_per_sm)))

    def cells(self, e):
        """Number of cells of engine e's column grid (0: no grid)."""
        v = _i32()
        check(load().frmc_engines_cells(self.handle, int(e), ctypes.byref(v), None))
        return v.value

    def regrid(self, e):
        """Rebuild engine e's column grid from its current coordinates."""
        check(load().frmc_engines_regrid(self.handle, int(e)))

    def swept(self, e):
        """Columns engine e's one-CTA steps swept since init (all its atoms
        per step without a grid, the selected cells' atoms with one)."""
        v, w = _i32(), _i64()
        check(load().frmc_engines_cells(self.handle, int(e), ctypes.byref(v), ctypes.byref(w)))
        return w.value

    def set_mode(self, fused):
        check(load().frmc_engines_set_mode(self.handle, int(bool(fused))))

    def set_sq_gemm_limit(self, limit):
        """Largest element-pair delta the S(Q) product takes through the
        tensor cores (default 2048; a column must also change at most 2^13
        unit counts); 0 forces the exact sum over the list of deltas and -1
        the dense integer loop (all three give the same integers)."""
        check(load().frmc_engines_set_sq_gemm_limit(self.handle, int(limit)))

    def set_sq_splits(self, max_splits):
        """At most `max_splits` K splits per 128-row block of the S(Q)
        product (0, the default: enough to fill the SMs).  The products are
        exact integers, so this changes a step's time, not its result."""
        check(load().frmc_engines_set_sq_splits(self.handle, int(max_splits)))

    TUNE_CANDIDATES = ((1024, 256, 2), (1024, 512, 1), (2048, 512, 1), (1024, 384, 1), (512, 128, 4),
                       (1024, 256, 4), (2048, 256, 2))

    def autotune(self, candidates=None, steps=6, warmup=2):
        """Choose the work-list configuration -- atoms per tile of split
        engines, threads per CTA, CTAs per SM -- with the shortest batched
        step for the live engines, by timing `steps` steps after `warmup`
        steps of each candidate, and keep it.  Results do not depend on the
        choice, but the timed steps advance every chain, so moves for
        len(candidates) * (warmup + steps) steps must be pushed.  Returns the
        chosen (tile, threads, ctas_per_sm)."""
        import time
        best = None
        for tn in candidates or self.TUNE_CANDIDATES:
            self.set_tune(*tn)
            self.step(warmup, graph=False)
            t0 = time.perf_counter()
            self.step(steps, graph=False)
            dt = time.perf_counter() - t0
            if best is None or dt < best[0]:
                best = (dt, tn)
        self.set_tune(*best[1])
        return best[1]

    @staticmethod
    def place_positions(sm, took):
        """The ordering `place` applies (host only): CTA b ran on SM sm[b] and
        its item took took[b]; returns the item each CTA gets."""
        sm = np.ascontiguousarray(sm, np.int32)
        took = np.ascontiguousarray(took, np.float64)
        if sm.shape != took.shape or sm.ndim != 1:
            raise ValueError("place_positions: sm and took must be 1-D arrays of one length")
        pos = np.empty(sm.size, np.int32)
        check(load().frmc_engines_place_positions(int(sm.size), sm.ctypes.data_as(I32P),
                                                  took.ctypes.data_as(F64P), pos.ctypes.data_as(I32P)))
        return pos

    def place(self, steps=3):
        """Measured placement of the batched launch: `steps` batched steps
        (they advance every chain) record which engines' CTAs share an SM
        and how long each engine took; the work list then gives the CTAs
        that hold an SM alone the longest engines and pairs the rest longest
        with shortest.  Results do not depend on the placement."""
        check(load().frmc_engines_place(self.handle, int(steps)))

    def get_tune(self):
        v = [ctypes.c_int() for _ in range(4)]
        check(load().frmc_engines_get_tune(self.handle, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def init(self):
        check(load().frmc_engines_init(self.handle))

    def push_group_moves(self, e, atoms, kinds, params, u, first_step):
        """Group moves (see group_moves) for steps [first_step, first_step + count)."""
        atoms = np.ascontiguousarray(atoms, np.int32)
        kinds = np.ascontiguousarray(kinds, np.int32)
        params = np.ascontiguousarray(params, F32)
        u = np.ascontiguousarray(u, F32)
        check(load().frmc_engines_push_group_moves(self.handle, int(e), atoms.ctypes.data_as(I32P),
                                                   kinds.ctypes.data_as(I32P), params.ctypes.data_as(F32P),
                                                   u.ctypes.data_as(F32P), len(kinds), int(first_step)))

    def push_moves(self, e, atoms, vecs, u, first_step):
        atoms = np.ascontiguousarray(atoms, np.int32)
        vecs = np.ascontiguousarray(vecs, F32)
        u = np.ascontiguousarray(u, F32)
        check(load().frmc_engines_push_moves(self.handle, int(e), atoms.ctypes.data_as(I32P),
                                             vecs.ctypes.data_as(F32P), u.ctypes.data_as(F32P), len(atoms),
                                             int(first_step), 0))

    def step(self, steps=1, engine=-1, graph=True, sync=True, stream=None):
        check(load().frmc_engines_step(self.handle, int(engine), int(steps), int(bool(graph)), stream))
        if sync:
            self.sync()

    def sync(self):
        check(load().frmc_engines_sync(self.handle))

    # ------------------------------------------------------------ queries
    def state(self, e):
        c2, st, acc = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        check(load().frmc_engines_state(self.handle, int(e), ctypes.byref(c2), ctypes.byref(st), ctypes.byref(acc)))
        return c2.value, st.value, acc.value

    def terms(self, e):
        """(sd of the G(r) term, sd of the S(Q) term) of engine e."""
        a, b = ctypes.c_double(), ctypes.c_double()
        check(load().frmc_engines_terms(self.handle, int(e), ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def sq(self, e):
        """S(Q) of engine e's current counts (FP64)."""
        out = np.empty(self.systems[e].sq.nq, np.float64)
        check(load().frmc_engines_sq(self.handle, int(e), out.ctypes.data_as(F64P)))
        return out

    def results(self, e, first_step, count):
        c = np.empty(count, np.float64)
        a = np.empty(count, np.int32)
        at = np.empty(count, np.int32)
        check(load().frmc_engines_results(self.handle, int(e), int(first_step), int(count), c.ctypes.data_as(F64P),
                                          a.ctypes.data_as(I32P), at.ctypes.data_as(I32P)))
        return c, a, at

    def counts(self, e):
        s = self.systems[e]
        ne, hs = len(s.model.elements_count), s.model.hs
        out = np.empty((2, ne, ne, hs), np.int32)
        check(load().frmc_engines_counts(self.handle, int(e), out.ctypes.data_as(I32P)))
        return out[0], out[1]

    def coords(self, e):
        n = self.systems[e].box_coords.shape[0]
        b = np.empty((n, 3), F32)
        r = np.empty((n, 3), F32)
        check(load().frmc_engines_coords(self.handle, int(e), b.ctypes.data_as(F32P), r.ctypes.data_as(F32P)))
        return b, r

    def info(self):
        E, a, b = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        check(load().frmc_engines_info(self.handle, ctypes.byref(E), ctypes.byref(a), ctypes.byref(b)))
        return {"engines": E.value, "atoms": a.value, "device_bytes": b.value}

    def close(self):
        if getattr(self, "handle", None):
            check(load().frmc_engines_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
