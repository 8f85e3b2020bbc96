"""Cases of ``atomic_coordination`` shared by the golden-vector generator and
the tests.

``make_inputs`` builds a seeded system with the definitions
AtomicCoordinationNumberConstraint would make from it
(``Constraints/AtomicCoordinationConstraints.py:242-415``: core and shell
atoms of each definition, and for every atom the definitions it is a core of
and a shell atom of); the golden file stores these inputs.  ``calls`` lists
every function of the module on those inputs, and ``run`` calls one on a
module (the compiled reference, the oracle or the GPU drop-in) and returns
its result as an array: the returned value, or ``coordNumData`` after an
in-place call.
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _triclinic(a, b, c, alpha, beta, gamma):
    al, be, ga = np.radians([alpha, beta, gamma])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(c * c - cx * cx - cy * cy)
    B = np.array([[a, 0, 0], [b * np.cos(ga), b * np.sin(ga), 0], [cx, cy, cz]], np.float64)
    B[np.abs(B) < 1e-9] = 0.0
    return B.astype(F)


def _flat(lists):
    off = np.zeros(len(lists) + 1, np.int64)
    off[1:] = np.cumsum([len(x) for x in lists])
    flat = np.concatenate(lists).astype(np.int32) if lists else np.zeros(0, np.int32)
    return flat, off


def _unflat(flat, off):
    return [np.ascontiguousarray(flat[off[k]:off[k + 1]], dtype=np.int32) for k in range(len(off) - 1)]


def definitions(el, ne_defs):
    """(cores, shells, lower, upper, asCore, inShell) for definitions given as
    (core element, shell element, lower, upper)."""
    n = el.shape[0]
    cores, shells, lower, upper = [], [], [], []
    for ce, se, lo, up in ne_defs:
        cores.append(np.flatnonzero(el == ce).astype(np.int32))
        shells.append(np.flatnonzero(el == se).astype(np.int32))
        lower.append(F(lo))
        upper.append(F(up))
    asCore = [[] for _ in range(n)]
    inShell = [[] for _ in range(n)]
    for d, (c, s) in enumerate(zip(cores, shells)):
        for a in c:
            asCore[a].append(d)
        for a in s:
            inShell[a].append(d)
    asCore = [np.array(x, np.int32) for x in asCore]
    inShell = [np.array(x, np.int32) for x in inShell]
    return cores, shells, lower, upper, asCore, inShell


def make_inputs(seed=909, n=420, ne=3):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)).astype(F)
    B = _triclinic(17.0, 16.0, 18.0, 84.0, 96.0, 104.0)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    defs = [(0, 1, 1.4, 2.9), (1, 2, 1.1, 3.3), (0, 0, 0.9, 2.6), (2, 1, 2.0, 4.1), (1, 1, 0.0, 2.2)]
    cores, shells, lower, upper, asCore, inShell = definitions(el, defs)
    g = dict(coords=c, basis=B, el=el, lower=np.array(lower, F), upper=np.array(upper, F))
    g["cores"], g["cores_off"] = _flat(cores)
    g["shells"], g["shells_off"] = _flat(shells)
    g["ascore"], g["ascore_off"] = _flat(asCore)
    g["inshell"], g["inshell_off"] = _flat(inShell)
    g["indexes"] = np.array([3, 17, 250, 17, 0, 419, 88], np.int32)
    # non-integer and near-2^24 starting values: float32 additions in order
    g["data0"] = (rng.random(len(defs)) * 50).astype(F)
    g["data_big"] = np.array([16777215.0, 16777210.0, 3.5, 16777216.0, 1e-30], F)
    g["neg_list"] = np.array([-1, -7, 5, 11, -420, 419], np.int32)
    return g


def unpack(g):
    cores = _unflat(g["cores"], g["cores_off"])
    shells = _unflat(g["shells"], g["shells_off"])
    asCore = _unflat(g["ascore"], g["ascore_off"])
    inShell = _unflat(g["inshell"], g["inshell_off"])
    lower = [F(x) for x in g["lower"]]
    upper = [F(x) for x in g["upper"]]
    return cores, shells, lower, upper, asCore, inShell


def distance_rows(pd, g, idx, isPBC=True):
    """Distance row of every atom in idx (fullrmc's pairs_distances_to_indexcoords)."""
    return [pd.pairs_distances_to_indexcoords(int(a), g["coords"], g["basis"], isPBC, True, 1) for a in idx]


def calls(g, rows):
    """(key, function name, positional args, start data or None).  rows are the
    distance rows of g["indexes"] (stored in the golden file)."""
    c, B, idx = g["coords"], g["basis"], g["indexes"]
    cores, shells, lower, upper, asCore, inShell = unpack(g)
    L = (cores, shells, lower, upper, asCore, inShell)
    cibc = (c * F(17.0)).astype(F)
    out = [
        ("all_pbc", "all_atoms_coord_number_coords", (c, B, True) + L, np.zeros(len(lower), F)),
        ("all_ibc", "all_atoms_coord_number_coords", (cibc, B, False) + L, np.zeros(len(lower), F)),
        ("multi_pbc", "multi_atoms_coord_number_coords", (idx, c, B, True) + L, g["data0"]),
        ("multi_ibc", "multi_atoms_coord_number_coords", (idx, cibc, B, False) + L, g["data0"]),
        ("multi_big", "multi_atoms_coord_number_coords", (np.arange(c.shape[0], dtype=np.int32), c, B, True) + L,
         g["data_big"]),
        ("multi_empty", "multi_atoms_coord_number_coords", (np.zeros(0, np.int32), c, B, True) + L, g["data0"]),
        ("multi_tot", "multi_atoms_coord_number_totdists", (idx, list(rows)) + L, g["data0"]),
        ("single_coords", "single_atom_coord_number_coords", (int(idx[2]), c, B, True) + L, g["data0"]),
        ("single_tot", "single_atom_coord_number_totdists", (int(idx[0]), rows[0]) + L, g["data0"]),
        ("ss_sub", "single_atom_single_shell_subdists", (rows[1], lower[1], upper[1]), None),
        ("ss_tot", "single_atom_single_shell_totdists", (rows[1], shells[1], lower[1], upper[1]), None),
        ("ss_tot_neg", "single_atom_single_shell_totdists", (rows[1], g["neg_list"], F(0.0), F(30.0)), None),
        ("ss_coords", "single_atom_single_shell_coords", (int(idx[1]), shells[1], c, B, True, lower[1], upper[1]),
         None),
        ("ss_coords_neg", "single_atom_single_shell_coords", (int(idx[1]), g["neg_list"], c, B, True, F(1.0),
                                                               F(9.0)), None),
        ("ms_tot", "single_atom_multi_shells_totdists", (rows[3], shells, g["lower"], g["upper"]), None),
        ("ms_coords", "single_atom_multi_shells_coords", (int(idx[3]), shells, c, B, True, g["lower"], g["upper"]),
         None),
        ("ms_coords_ibc", "single_atom_multi_shells_coords", (int(idx[3]), cores, cibc, B, False, g["lower"],
                                                              g["upper"]), None),
    ]
    return out


def run(module, name, args, data):
    """Result of one call as a float32 array."""
    fn = getattr(module, name)
    if data is not None:
        d = np.array(data, F, copy=True)
        fn(*(args + (d,)))
        return d
    return np.asarray(fn(*args), F).reshape(-1)
