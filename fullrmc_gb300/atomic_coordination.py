"""Drop-in replacement of ``fullrmc.Core.atomic_coordination`` on the GPU.

Same function names, positional order, keyword names, defaults and return
conventions as ``Extensions/atomic_coordination.pyx`` (used by
AtomicCoordinationNumberConstraint,
``Constraints/AtomicCoordinationConstraints.py:476-580``).  Every function is
turned into a sequence of terms -- (row, index list, definition) -- and the
terms run on the device in one call of ``frmc_coordination_terms``: the
window counts are integers, and the float32 additions into ``coordNumData``
keep the reference's term order, so the results equal the reference's
``ncores=1`` results bit for bit.  ``ncores`` is accepted and ignored.

Two reference behaviours are kept on purpose:

* ``single_atom_coord_number_totdists`` walks ``asCoreDefIdxs[atomIndex]``
  twice, the second time against ``coresIndexes``
  (``atomic_coordination.pyx:192-198``); it never reads ``inShellDefIdxs``.
* ``all_atoms_coord_number_totdists`` passes its 2-D ``distances`` array on
  to a function typed ``list distances`` (``atomic_coordination.pyx:317-347``)
  and therefore always raises ``TypeError``.

Where the reference reads outside a list or buffer without a check (it is
compiled with ``boundscheck(False)`` and ``wraparound(False)``: a negative
or too large atom index, definition index or shell-window index), these
functions raise ``IndexError`` and leave ``coordNumData`` unchanged.
"""
from __future__ import annotations

import operator

import numpy as np

from . import _args as A
from ._native import I32P, I64P, call, ptr
from .pairs_distances import pairs_distances_to_point  # noqa: F401  (the reference module imports it too)

NUMPY_FLOAT32 = np.float32
NUMPY_INT32 = np.int32


def _list_arg(name, v):
    """A ``list`` typed argument: a list or None (None fails when used)."""
    if v is not None and not isinstance(v, list):
        raise TypeError("Argument '%s' has incorrect type (expected list, got %s)" % (name, type(v).__name__))
    return v


def _item(seq, name, k):
    """seq[k] for an index the reference does not check."""
    if seq is None:
        raise TypeError("'NoneType' object is not subscriptable")
    if k < 0 or k >= len(seq):
        raise IndexError("%s index %d out of range" % (name, k))
    return seq[k]


def _window(v):
    """A C_FLOAT32 conversion of a window bound."""
    if isinstance(v, (str, bytes, bytearray)) or v is None:
        raise TypeError("must be real number, not %s" % type(v).__name__)
    return np.float32(float(v))


def _def_array(a):
    """Definition indexes of one atom (an array or list of integers)."""
    d = np.asarray(a)
    if d.ndim != 1:
        d = d.reshape(-1)
    if d.size == 0:
        return np.zeros(0, np.int64)
    if d.dtype.kind not in "iu":
        raise TypeError("list indices must be integers or slices, not %s" % d.dtype.name)
    return d.astype(np.int64)


def _coords(boxCoords, basis, isPBC):
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    if c.shape[1] != 3:
        raise ValueError("boxCoords must be (n, 3)")
    B = A.memview("basis", basis, np.float32, 2)
    if B.shape != (3, 3):
        raise ValueError("basis must be (3, 3)")
    return c, B, int(A.bint(isPBC))


def _data_arg(coordNumData):
    """``C_FLOAT32[:] coordNumData``: a writable float32 1-D buffer."""
    if coordNumData is None:
        raise TypeError("Argument 'coordNumData' must not be None")
    if not isinstance(coordNumData, np.ndarray):
        coordNumData = np.asarray(coordNumData)
    if coordNumData.ndim != 1:
        raise ValueError("Buffer has wrong number of dimensions (expected 1, got %d)" % coordNumData.ndim)
    if coordNumData.dtype != np.float32:
        raise ValueError("Buffer dtype mismatch, expected 'C_FLOAT32' but got '%s'" % coordNumData.dtype.name)
    if not coordNumData.flags.writeable:
        raise ValueError("buffer source array is read-only")
    return coordNumData


class _Terms:
    """Terms, their index lists and windows, run by one device call."""

    def __init__(self, ndata):
        self.ndata = ndata
        self.lists = []
        self.keys = {}
        self.rows, self.lids, self.defs = [], [], []
        self.lower = np.zeros(ndata, np.float32)
        self.upper = np.zeros(ndata, np.float32)
        self.window_set = np.zeros(ndata, bool)

    def list_id(self, key, arr, name):
        lid = self.keys.get(key)
        if lid is None:
            lid = len(self.lists)
            self.lists.append(A.memview(name, arr, np.int32, 1))
            self.keys[key] = lid
        return lid

    def window(self, d, lo, up):
        if d < 0 or d >= self.ndata:
            raise IndexError("coordNumData index %d out of range for %d entries" % (d, self.ndata))
        if not self.window_set[d]:
            self.lower[d] = _window(lo)
            self.upper[d] = _window(up)
            self.window_set[d] = True

    def add(self, row, lid, d):
        self.rows.append(row)
        self.lids.append(lid)
        self.defs.append(d)

    def add_many(self, rows, lids, defs):
        self.rows.append(np.asarray(rows, np.int32))
        self.lids.append(np.asarray(lids, np.int32))
        self.defs.append(np.asarray(defs, np.int32))

    def _flat(self, parts):
        arrs = [np.atleast_1d(np.asarray(p, np.int32)) for p in parts]
        return np.ascontiguousarray(np.concatenate(arrs) if arrs else np.zeros(0, np.int32), dtype=np.int32)

    def run(self, data, coords=None, basis=None, isPBC=0, drows=None):
        rows, lids, defs = self._flat(self.rows), self._flat(self.lids), self._flat(self.defs)
        if rows.shape[0] == 0:
            return
        lens = np.array([a.shape[0] for a in self.lists], np.int64)
        off = np.zeros(len(self.lists) + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        pool = np.ascontiguousarray(np.concatenate(self.lists) if self.lists else np.zeros(0, np.int32), np.int32)
        buf = np.ascontiguousarray(data) if data.flags.c_contiguous else data.copy()
        if coords is not None:
            call("frmc_coordination_terms", ptr(coords), coords.shape[0], ptr(basis), isPBC, None, None, None, 0,
                 ptr(pool, I32P), ptr(off, I64P), len(self.lists), ptr(rows, I32P), ptr(lids, I32P),
                 ptr(defs, I32P), rows.shape[0], ptr(self.lower), ptr(self.upper), ptr(buf), self.ndata)
        else:
            dl = np.array([r.shape[0] for r in drows], np.int32)
            do = np.zeros(len(drows), np.int64)
            if len(drows) > 1:
                np.cumsum(dl[:-1], out=do[1:])
            dpool = np.ascontiguousarray(np.concatenate(drows) if drows else np.zeros(0, np.float32), np.float32)
            call("frmc_coordination_terms", None, 0, None, 0, ptr(dpool), ptr(do, I64P), ptr(dl, I32P), len(drows),
                 ptr(pool, I32P), ptr(off, I64P), len(self.lists), ptr(rows, I32P), ptr(lids, I32P),
                 ptr(defs, I32P), rows.shape[0], ptr(self.lower), ptr(self.upper), ptr(buf), self.ndata)
        if buf is not data:
            data[...] = buf


def _atom_defs(seq, idx):
    """seq[a] for every atom a of idx (a Python list of ints already checked
    against len(seq)), concatenated: (counts per atom, definition indexes)."""
    K = len(idx)
    got = operator.itemgetter(*idx)(seq) if K > 1 else (seq[idx[0]],)
    counts = np.fromiter(map(len, got), np.int64, K)
    D = np.concatenate(got) if K else np.zeros(0, np.int64)
    if D.size and D.dtype.kind not in "iu":  # an empty float list widens the dtype: check one by one
        D = np.concatenate([_def_array(a) for a in got])
    return counts, np.asarray(D, np.int64).reshape(-1)


def _atoms_terms(T, indexes, rows, coresIndexes, shellsIndexes, lowerShells, upperShells, first, second):
    """The terms of the atoms ``indexes`` (row k for atom indexes[k]):
    first[atom]'s definitions against their shells, then second[atom]'s
    against their cores (``atomic_coordination.pyx:207-240``)."""
    K = len(indexes)
    if K == 0:
        return
    idx = np.asarray(indexes, np.int64)
    for seq in (first, second):
        if seq is None:
            raise TypeError("'NoneType' object is not subscriptable")
        if idx.min() < 0 or idx.max() >= len(seq):
            bad = int(idx[(idx < 0) | (idx >= len(seq))][0])
            raise IndexError("list index %d out of range" % bad)
    il = idx.tolist()
    c1, D1 = _atom_defs(first, il)
    c2, D2 = _atom_defs(second, il)
    # windows and lists of the definitions used
    lids = []
    for kind, D, lists in ((0, D1, shellsIndexes), (1, D2, coresIndexes)):
        if D.shape[0] == 0:
            lids.append(D)
            continue
        used = np.unique(D)
        lut = np.empty(int(used[-1]) + 1 - min(0, int(used[0])), np.int64)
        for d in used.tolist():
            T.window(d, _item(lowerShells, "list", d), _item(upperShells, "list", d))
            lut[d] = T.list_id((kind, d), _item(lists, "list", d), "shellIndexes")
        lids.append(lut[D])
    start = np.zeros(K, np.int64)
    np.cumsum((c1 + c2)[:-1], out=start[1:])
    total = int((c1 + c2).sum())
    t_row = np.empty(total, np.int32)
    t_lid = np.empty(total, np.int32)
    t_def = np.empty(total, np.int32)
    rows = np.asarray(rows, np.int64)
    for c, D, lid, base in ((c1, D1, lids[0], start), (c2, D2, lids[1], start + c1)):
        if D.shape[0] == 0:
            continue
        o = np.zeros(K, np.int64)
        np.cumsum(c[:-1], out=o[1:])
        pos = np.repeat(base, c) + (np.arange(D.shape[0]) - np.repeat(o, c))
        t_row[pos] = np.repeat(rows, c)
        t_lid[pos] = lid
        t_def[pos] = D
    T.add_many(t_row, t_lid, t_def)


# ----------------------------------------------------------- single shells
def single_atom_single_shell_subdists(distances, lowerShell, upperShell, ncores=1):
    """Number of distances inside [lowerShell, upperShell], as a float
    (``atomic_coordination.pyx:55-65``)."""
    d = A.memview("distances", distances, np.float32, 1)
    lo, up = A.float32("lowerShell", lowerShell), A.float32("upperShell", upperShell)
    A.int32("ncores", ncores)
    T = _Terms(1)
    T.window(0, lo, up)
    T.add(0, T.list_id("all", np.arange(d.shape[0], dtype=np.int32), "shellIndexes"), 0)
    out = np.zeros(1, np.float32)
    T.run(out, drows=[d])
    return float(out[0])


def single_atom_single_shell_totdists(distances, shellIndexes, lowerShell, upperShell, ncores=1):
    """The same over distances[shellIndexes] (``atomic_coordination.pyx:71-80``)."""
    d = A.array("distances", distances, np.float32, 1)
    s = A.memview("shellIndexes", shellIndexes, np.int32, 1)
    lo, up = A.float32("lowerShell", lowerShell), A.float32("upperShell", upperShell)
    A.int32("ncores", ncores)
    T = _Terms(1)
    T.window(0, lo, up)
    T.add(0, T.list_id("s", s, "shellIndexes"), 0)
    out = np.zeros(1, np.float32)
    T.run(out, drows=[d])
    return float(out[0])


def single_atom_single_shell_coords(coreIndex, shellIndexes, boxCoords, basis, isPBC, lowerShell, upperShell,
                                    ncores=1):
    """The same over the distances of atom coreIndex to the atoms shellIndexes
    (``atomic_coordination.pyx:89-108``)."""
    core = A.int32("coreIndex", coreIndex)
    s = A.memview("shellIndexes", shellIndexes, np.int32, 1)
    c, B, pbc = _coords(boxCoords, basis, isPBC)
    lo, up = A.float32("lowerShell", lowerShell), A.float32("upperShell", upperShell)
    A.int32("ncores", ncores)
    T = _Terms(1)
    T.window(0, lo, up)
    T.add(core, T.list_id("s", s, "shellIndexes"), 0)
    out = np.zeros(1, np.float32)
    T.run(out, coords=c, basis=B, isPBC=pbc)
    return float(out[0])


def _multi_shells(n_shells, shellsIndexes, lowerShells, upperShells, row):
    lo = A.memview("lowerShells", lowerShells, np.float32, 1)
    up = A.memview("upperShells", upperShells, np.float32, 1)
    T = _Terms(n_shells)
    for i in range(n_shells):
        T.window(i, _item(lo, "lowerShells", i), _item(up, "upperShells", i))
        T.add(row, T.list_id(i, shellsIndexes[i], "shellIndexes"), i)
    return T


def single_atom_multi_shells_totdists(distances, shellsIndexes, lowerShells, upperShells, ncores=1):
    """One count per shell i over distances[shellsIndexes[i]]
    (``atomic_coordination.pyx:116-133``); float32 array."""
    d = A.array("distances", distances, np.float32, 1)
    _list_arg("shellsIndexes", shellsIndexes)
    A.int32("ncores", ncores)
    ns = len(shellsIndexes)
    T = _multi_shells(ns, shellsIndexes, lowerShells, upperShells, 0)
    out = np.zeros(ns, NUMPY_FLOAT32)
    T.run(out, drows=[d])
    return out


def single_atom_multi_shells_coords(coreIndex, shellsIndexes, boxCoords, basis, isPBC, lowerShells, upperShells,
                                    ncores=1):
    """One count per shell i over the distances of atom coreIndex to
    shellsIndexes[i] (``atomic_coordination.pyx:139-166``); float32 array."""
    core = A.int32("coreIndex", coreIndex)
    _list_arg("shellsIndexes", shellsIndexes)
    c, B, pbc = _coords(boxCoords, basis, isPBC)
    A.int32("ncores", ncores)
    ns = len(shellsIndexes)
    T = _multi_shells(ns, shellsIndexes, lowerShells, upperShells, core)
    out = np.zeros(ns, NUMPY_FLOAT32)
    T.run(out, coords=c, basis=B, isPBC=pbc)
    return out


# ----------------------------------------------------- coordination numbers
def _lists(coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs):
    for name, v in (("coresIndexes", coresIndexes), ("shellsIndexes", shellsIndexes), ("lowerShells", lowerShells),
                    ("upperShells", upperShells), ("asCoreDefIdxs", asCoreDefIdxs),
                    ("inShellDefIdxs", inShellDefIdxs)):
        _list_arg(name, v)


def single_atom_coord_number_totdists(atomIndex, distances, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                      asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """Adds atom atomIndex's coordination terms from its distance row to
    coordNumData in place (``atomic_coordination.pyx:171-198``; both loops
    walk asCoreDefIdxs, as in the reference)."""
    a = A.int32("atomIndex", atomIndex)
    d = A.array("distances", distances, np.float32, 1)
    _lists(coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    data = _data_arg(coordNumData)
    A.int32("ncores", ncores)
    T = _Terms(data.shape[0])
    _atoms_terms(T, [a], [0], coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, asCoreDefIdxs)
    T.run(data, drows=[d])


def single_atom_coord_number_coords(atomIndex, boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells,
                                    upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """Adds atom atomIndex's coordination terms to coordNumData in place
    (``atomic_coordination.pyx:207-240``)."""
    a = A.int32("atomIndex", atomIndex)
    c, B, pbc = _coords(boxCoords, basis, isPBC)
    _lists(coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    data = _data_arg(coordNumData)
    A.int32("ncores", ncores)
    T = _Terms(data.shape[0])
    _atoms_terms(T, [a], [a], coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    T.run(data, coords=c, basis=B, isPBC=pbc)


def multi_atoms_coord_number_totdists(indexes, distances, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                      asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """single_atom_coord_number_totdists for every indexes[i] with the
    distance row distances[i] (``atomic_coordination.pyx:249-278``)."""
    idx = A.memview("indexes", indexes, np.int32, 1)
    _list_arg("distances", distances)
    _lists(coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    data = _data_arg(coordNumData)
    A.int32("ncores", ncores)
    K = idx.shape[0]
    rows = [A.array("distances", _item(distances, "list", k), np.float32, 1) for k in range(K)]
    T = _Terms(data.shape[0])
    _atoms_terms(T, idx, np.arange(K), coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs,
                 asCoreDefIdxs)
    T.run(data, drows=rows)


def multi_atoms_coord_number_coords(indexes, boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells,
                                    upperShells, asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """single_atom_coord_number_coords for every indexes[i], in order
    (``atomic_coordination.pyx:280-309``): the constraint's before- and
    after-move data (AtomicCoordinationConstraints.py:520-573)."""
    idx = A.memview("indexes", indexes, np.int32, 1)
    c, B, pbc = _coords(boxCoords, basis, isPBC)
    _lists(coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    data = _data_arg(coordNumData)
    A.int32("ncores", ncores)
    T = _Terms(data.shape[0])
    _atoms_terms(T, idx, idx, coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs, inShellDefIdxs)
    T.run(data, coords=c, basis=B, isPBC=pbc)


def all_atoms_coord_number_totdists(distances, coresIndexes, shellsIndexes, lowerShells, upperShells, asCoreDefIdxs,
                                    inShellDefIdxs, coordNumData, ncores=1):
    """Raises TypeError, as the reference does (``atomic_coordination.pyx:317-347``
    passes the 2-D array to a ``list`` argument)."""
    if distances is not None:
        A.array("distances", distances, np.float32, 2)
    raise TypeError("Argument 'distances' has incorrect type (expected list, got %s)"
                    % ("numpy.ndarray" if isinstance(distances, np.ndarray) else type(distances).__name__))


def all_atoms_coord_number_coords(boxCoords, basis, isPBC, coresIndexes, shellsIndexes, lowerShells, upperShells,
                                  asCoreDefIdxs, inShellDefIdxs, coordNumData, ncores=1):
    """multi_atoms_coord_number_coords over every atom 0..n-1
    (``atomic_coordination.pyx:349-377``): the constraint's compute_data
    (AtomicCoordinationConstraints.py:476-518)."""
    c = A.array("boxCoords", boxCoords, np.float32, 2)
    indexes = np.arange(c.shape[0], dtype=NUMPY_INT32)
    multi_atoms_coord_number_coords(indexes=indexes, boxCoords=c, basis=basis, isPBC=isPBC,
                                    coresIndexes=coresIndexes, shellsIndexes=shellsIndexes, lowerShells=lowerShells,
                                    upperShells=upperShells, asCoreDefIdxs=asCoreDefIdxs,
                                    inShellDefIdxs=inShellDefIdxs, coordNumData=coordNumData, ncores=ncores)
