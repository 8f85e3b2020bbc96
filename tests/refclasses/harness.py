"""Run fullrmc's own constraint classes, unmodified, on a histogram backend.

Test infrastructure.  ``load_classes()`` imports fullrmc's
``Constraints/PairDistributionConstraints.py``,
``Constraints/StructureFactorConstraints.py`` and
``Constraints/PairCorrelationConstraints.py`` from the reference checkout as
they are: the ``fullrmc`` package object is made here (its ``__init__.py``
would import the whole Engine, which needs the repository and PDB packages
that are not installed), the shims under ``shims/`` stand in for
``pysimplelog`` and ``pdbparser``, ``fullrmc.Engine`` is a stub module whose
``Engine`` class is the stub engine below (``Core/Constraint.py:87-91``
checks ``isinstance(engine, Engine)``), and ``fullrmc.Core.pairs_histograms``
is a switch that forwards every call to the backend selected with
``use_backend`` -- the compiled reference, the C oracle or the GPU drop-in --
and feeds a running digest of each call's inputs and outputs.

``run_chain()`` drives one constraint through fullrmc's plain step
(``Engine.py:3278-3344``): ``compute_data``, then per move
``compute_before_move``, ``compute_after_move`` with the moved box
coordinates (``transform_coordinates`` of the moved real coordinates,
``Engine.py:3222-3223``), the total standard error
(``Engine.py:3000-3029``) against the current one with fullrmc's rule
(reject iff larger and ``u > tolerance``, ``Engine.py:3300-3317``), then
``accept_move`` (and the engine's coordinates updated) or ``reject_move``.

``replay_calls()`` issues the same histogram calls from a recorded chain
(the moves, decisions and call arguments) on any backend without the
classes, so that the GPU drop-in can be checked against a chain of the
reference classes where the reference checkout is absent.
"""
from __future__ import annotations

import hashlib
import importlib
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHIMS = os.path.join(HERE, "shims")
F32 = np.float32

_BACKEND = {"ph": None, "bcc": None}
_RECORD = {"digest": None, "calls": 0}


# ----------------------------------------------------------- the switch
def _feed(kind, kw, out):
    h = _RECORD["digest"]
    if h is None:
        return
    _RECORD["calls"] += 1
    h.update(kind.encode())
    for key in ("indexes", "boxCoords", "moleculeIndex", "elementIndex"):
        if key in kw:
            h.update(np.ascontiguousarray(kw[key]).tobytes())
    h.update(np.array([kw["minDistance"], kw["maxDistance"], kw["bin"]], F32).tobytes())
    h.update(np.array([kw["histSize"], kw["numberOfElements"], int(bool(kw.get("allAtoms", False)))],
                      np.int64).tobytes())
    for a in out:
        h.update(np.ascontiguousarray(a, F32).tobytes())


def multiple_pairs_histograms_coords(**kw):
    out = _BACKEND["ph"].multiple_pairs_histograms_coords(**kw)
    _feed("M", kw, out)
    return out


def full_pairs_histograms_coords(**kw):
    out = _BACKEND["ph"].full_pairs_histograms_coords(**kw)
    _feed("F", kw, out)
    return out


def use_backend(pairs_histograms, boundary_conditions_collection):
    _BACKEND["ph"] = pairs_histograms
    _BACKEND["bcc"] = boundary_conditions_collection


def start_digest():
    _RECORD["digest"] = hashlib.blake2b(digest_size=16)
    _RECORD["calls"] = 0


def digest():
    return _RECORD["digest"].hexdigest()


# ----------------------------------------------------------- stub engine
class _NoneCollected(object):
    """The engine's atoms collector with no atom removed."""
    indexes = []

    def __len__(self):
        return 0


class StubEngine(object):
    """The engine attributes fullrmc's PDF, S(Q) and g(r) constraints read,
    with fullrmc's types: float32 coordinates and basis, int32 indexes,
    ``volume`` and ``numberDensity`` as float32 (``Engine.py:2246-2274``),
    sorted element names and per-element counts (``Engine.py:2435-2446``),
    one normal frame and no repository."""

    def __init__(self, system, names):
        self.realCoordinates = np.array(system.real_coords, F32, copy=True)
        self.boxCoordinates = np.array(system.box_coords, F32, copy=True)
        self.basisVectors = np.ascontiguousarray(system.basis, F32)
        self.reciprocalBasisVectors = np.ascontiguousarray(system.rbasis, F32)
        self.isPBC = bool(system.isPBC)
        self.moleculesIndex = np.ascontiguousarray(system.mol, np.int32)
        self.allElements = [names[i] for i in system.el]
        self.elements = sorted(set(self.allElements))
        lut = {e: i for i, e in enumerate(self.elements)}
        self.elementsIndex = np.array([lut[e] for e in self.allElements], np.int32)
        self.numberOfAtomsPerElement = {}
        for e in self.allElements:
            self.numberOfAtomsPerElement[e] = self.numberOfAtomsPerElement.get(e, 0) + 1
        # the box volume comes from pdbparser in fullrmc (Engine.py:2248),
        # which is not installed: both sides of every comparison take the
        # system model's volume
        self.volume = F32(system.model.volume)
        self.numberDensity = F32(self.numberOfAtoms) / F32(self.volume)
        self._runtime_ncores = np.int32(1)
        self.usedFrame = "0"
        self.frames = {"0": {"frames_name": None}}
        self.constraints = []
        self.accepted = 0
        self.tried = 0
        self.totalStandardError = None
        self._atomsCollector = _NoneCollected()

    @property
    def numberOfAtoms(self):
        return self.realCoordinates.shape[0]

    @property
    def numberOfElements(self):
        return len(self.elements)

    def get_frame_category(self, frame):
        return True, False, False

    def _get_repository(self):
        return None


# ----------------------------------------------------------- loading
def load_classes(reference_root, switch=True):
    """Import the three constraint modules from the reference checkout as
    they are; returns (PairDistributionConstraint, StructureFactorConstraint,
    PairCorrelationConstraint).  With switch=False,
    ``fullrmc.Core.pairs_histograms`` is left to whatever import hook is
    installed (``fullrmc_gb300.install()``).  Idempotent within a process."""
    done = sys.modules.get("fullrmc.Constraints.PairCorrelationConstraints")
    if done is not None:
        return (sys.modules["fullrmc.Constraints.PairDistributionConstraints"].PairDistributionConstraint,
                sys.modules["fullrmc.Constraints.StructureFactorConstraints"].StructureFactorConstraint,
                done.PairCorrelationConstraint)
    if SHIMS not in sys.path:
        sys.path.insert(0, SHIMS)
    # a compiled reference imported earlier (oracle/_ref/fullrmc) stays usable
    # through the module objects its caller holds; the names go to the tree
    for key in [k for k in sys.modules if k == "fullrmc" or k.startswith("fullrmc.")]:
        del sys.modules[key]
    pkg = types.ModuleType("fullrmc")
    pkg.__path__ = [reference_root]
    sys.modules["fullrmc"] = pkg
    eng = types.ModuleType("fullrmc.Engine")
    eng.Engine = StubEngine
    sys.modules["fullrmc.Engine"] = eng
    pkg.Engine = eng
    core = importlib.import_module("fullrmc.Core")
    if switch:
        this = sys.modules[__name__]
        sys.modules["fullrmc.Core.pairs_histograms"] = this
        core.pairs_histograms = this
    pdc = importlib.import_module("fullrmc.Constraints.PairDistributionConstraints")
    sfc = importlib.import_module("fullrmc.Constraints.StructureFactorConstraints")
    pcf = importlib.import_module("fullrmc.Constraints.PairCorrelationConstraints")
    return pdc.PairDistributionConstraint, sfc.StructureFactorConstraint, pcf.PairCorrelationConstraint


# ----------------------------------------------------------- chains
def chain_definitions():
    """The recorded chains: name -> dict(system, kind, options, steps, ...)."""
    from fullrmc_gb300 import synthetic
    return {
        # 5,000-atom binary alloy, cubic 38.2 A, r 0-15 A; single-atom
        # translations up to 0.1 A; 10^4 steps
        "pdc_alloy_5000": dict(system=lambda: synthetic.alloy_5000(seed=1), kind="pdc", steps=10000, amp=0.1,
                               group=1, options={}),
        # the same constraint with a fitted scale factor every 10 accepted
        # moves and a 5-point window function, 2,000 atoms of the alloy
        "pdc_scaled_window": dict(system=lambda: synthetic.alloy_5000(seed=2, n=2000), kind="pdc", steps=1000,
                                  amp=0.3, group=1,
                                  options=dict(adjustScaleFactor=(10, 0.8, 1.2), window=5)),
        # PairDistributionConstraint with 13-atom groups of a molecular system
        # (translations of whole molecules)
        "pdc_groups_13": dict(system=lambda: synthetic.ring_molecules(seed=3, nmol=300), kind="pdc", steps=600,
                              amp=0.2, group=13, options={}),
        # StructureFactorConstraint on Q 0.5-12, its own r grid 0-10 A (0.02)
        "sfc_alloy_2000": dict(system=lambda: synthetic.alloy_5000(seed=4, n=2000), kind="sfc", steps=800, amp=0.3,
                               group=1, options=dict(q=(0.5, 12.0, 0.05), rmin=0.0, rmax=10.0, dr=0.02)),
        # PairCorrelationConstraint g(r), three species, triclinic box
        "pcf_triclinic_3000": dict(system=lambda: synthetic.triclinic_100k(seed=5, n=3000), kind="pcf", steps=800,
                                   amp=0.3, group=1, options={}),
    }


NAMES = ["Cu", "Ni", "Ti", "Zr"]


def make_moves(system, steps, amp, group, seed=91):
    """(indexes (steps, group), vectors (steps, 3), u (steps,)): atom or
    molecule picked uniformly, translation direction uniform, length
    uniform in [0, amp), float32 (the distribution of fullrmc's
    TranslationGenerator).  Always generated for the chain's full length,
    so that a shorter run uses a prefix of the same moves."""
    from fullrmc_gb300.engine import translation_moves
    rng = np.random.default_rng(seed)
    n = system.box_coords.shape[0]
    if group == 1:
        a, v, u = translation_moves(rng, n, steps, amp)
        return a.reshape(-1, 1), v, u
    a, v, u = translation_moves(rng, n // group, steps, amp)
    idx = (a[:, None] * group + np.arange(group)[None, :]).astype(np.int32)
    return idx, v, u


def make_constraint(classes, d, system, engine):
    PDC, SFC, PCF = classes
    m = system.model
    ne = len(m.elements_count)
    aw = {NAMES[i]: float(1.0 + 0.25 * i) for i in range(ne)}
    opts = d["options"]
    if d["kind"] == "sfc":
        q0, q1, dq = opts["q"]
        q = (q0 + dq * np.arange(int(round((q1 - q0) / dq)) + 1)).astype(F32)
        rng = np.random.default_rng(11)
        S = (1.0 + 0.3 * np.sin(q) * np.exp(-0.2 * q) + rng.normal(0, 0.01, q.size)).astype(F32)
        c = SFC(experimentalData=np.column_stack([q, S]).astype(F32), weighting="atomicNumber", atomsWeight=aw,
                rmin=opts["rmin"], rmax=opts["rmax"], dr=opts["dr"])
    else:
        G = np.asarray(m.G_exp, F32)
        if d["kind"] == "pcf":
            r = np.asarray(m.r, np.float64)
            G = (1.0 + G / np.where(r > 0, 4 * np.pi * r * float(m.rho0), 1.0)).astype(F32)
        exp = np.column_stack([np.asarray(m.r, F32), G]).astype(F32)
        kw = dict(experimentalData=exp, weighting="atomicNumber", atomsWeight=aw)
        if "adjustScaleFactor" in opts:
            kw["adjustScaleFactor"] = opts["adjustScaleFactor"]
        if opts.get("window"):
            w = np.hanning(opts["window"] + 2)[1:-1].astype(F32)
            kw["windowFunction"] = w
        c = (PCF if d["kind"] == "pcf" else PDC)(**kw)
    c._set_engine(engine)
    engine.constraints.append(c)
    c.listen("engine set")
    c._runtime_initialize()
    return c


def call_arguments(c):
    """The histogram grid a constraint passes to its histogram calls."""
    return dict(minDistance=F32(c.minimumDistance), maxDistance=F32(c.maximumDistance), bin=F32(c.bin),
                histSize=int(c.histogramSize))


def run_chain(classes, name, steps=None, record_every=100):
    """One chain of fullrmc's own class on the current backend.  Returns a
    dict: decisions, total standard error after each move, digest
    checkpoints of all histogram calls every `record_every` steps, the final
    data arrays, and what a replay needs (grid, weights, system)."""
    d = chain_definitions()[name]
    system = d["system"]()
    steps = d["steps"] if steps is None else steps
    names = NAMES
    engine = StubEngine(system, names)
    c = make_constraint(classes, d, system, engine)
    start_digest()
    c.compute_data()
    total = np.sum([c.standardError / c.varianceSquared])
    engine.totalStandardError = total
    idx, vec, u = (x[:steps] for x in make_moves(system, d["steps"], d["amp"], d["group"]))
    accepted = np.zeros(steps, bool)
    errors = np.zeros(steps, F32)
    checkpoints = []
    bcc = _BACKEND["bcc"]
    for k in range(steps):
        rel = np.ascontiguousarray(idx[k], np.int32)
        c._runtime_on_step()
        moved_real = (engine.realCoordinates[rel] + vec[k]).astype(F32)
        moved_box = bcc.transform_coordinates(transMatrix=engine.reciprocalBasisVectors, coords=moved_real) \
            if engine.isPBC else moved_real
        engine.tried += 1
        c.compute_before_move(realIndexes=rel, relativeIndexes=rel)
        c.compute_after_move(realIndexes=rel, relativeIndexes=rel, movedBoxCoordinates=moved_box)
        new = np.sum([c.afterMoveStandardError / c.varianceSquared])
        errors[k] = new
        reject = False
        if new > total:
            if u[k] > 0.0:   # tolerance 0: fullrmc's default
                reject = True
            else:
                total = new
        else:
            total = new
        if reject:
            c.reject_move(realIndexes=rel, relativeIndexes=rel)
        else:
            engine.accepted += 1
            c.accept_move(realIndexes=rel, relativeIndexes=rel)
            engine.realCoordinates[rel] = moved_real
            engine.boxCoordinates[rel] = moved_box
            accepted[k] = True
        engine.totalStandardError = total
        if (k + 1) % record_every == 0:
            checkpoints.append(digest())
    ws = {}
    scheme = c.weightingScheme
    for i, a in enumerate(engine.elements):
        for j, b in enumerate(engine.elements):
            w = scheme.get("%s-%s" % (a, b), scheme.get("%s-%s" % (b, a)))
            ws[(i, j)] = F32(w)
    ne = len(engine.elements)
    return dict(accepted=accepted, errors=errors, checkpoints=np.array(checkpoints), calls=_RECORD["calls"],
                intra=np.asarray(c.data["intra"], F32), inter=np.asarray(c.data["inter"], F32),
                box=engine.boxCoordinates.copy(), grid=call_arguments(c),
                weights=np.array([[ws[(i, j)] for j in range(ne)] for i in range(ne)], F32), system=system,
                moves=(idx, vec, u))


def replay_calls(ph, bcc, system, moves, accepted, grid, record_every=100):
    """The histogram calls of a recorded chain, issued on `ph` in the
    classes' order (``compute_data``: F on all atoms; each move: M and F of
    the group before the move, then with the moved coordinates written in,
    ``PairDistributionConstraints.py:1001-1129`` and the same in the S(Q) and
    g(r) classes), with the recorded decisions.  Returns the digest
    checkpoints, the call count and the final data arrays (updated as the
    classes do: data - before + after on acceptance)."""
    box = np.array(system.box_coords, F32, copy=True)
    real = np.array(system.real_coords, F32, copy=True)
    rbasis = np.ascontiguousarray(system.rbasis, F32)
    basis = np.ascontiguousarray(system.basis, F32)
    mol = np.ascontiguousarray(system.mol, np.int32)
    el = np.ascontiguousarray(system.el, np.int32)
    ne = len(system.model.elements_count)
    kw = dict(basis=basis, isPBC=bool(system.isPBC), numberOfElements=ne, ncores=np.int32(1), **grid)
    use_backend(ph, bcc)
    start_digest()
    switch = sys.modules[__name__]
    intra, inter = switch.full_pairs_histograms_coords(boxCoords=box, moleculeIndex=mol, elementIndex=el, **kw)
    idx, vec, u = moves
    checkpoints = []

    def delta(rel):
        iM, eM = switch.multiple_pairs_histograms_coords(indexes=rel, boxCoords=box, moleculeIndex=mol,
                                                         elementIndex=el, allAtoms=True, **kw)
        iF, eF = switch.full_pairs_histograms_coords(boxCoords=box[rel], moleculeIndex=mol[rel],
                                                     elementIndex=el[rel], **kw)
        return iM - iF, eM - eF

    for k in range(len(accepted)):
        rel = np.ascontiguousarray(idx[k], np.int32)
        moved_real = (real[rel] + vec[k]).astype(F32)
        moved_box = bcc.transform_coordinates(transMatrix=rbasis, coords=moved_real) if system.isPBC else moved_real
        before = delta(rel)
        saved = np.array(box[rel], F32)
        box[rel] = moved_box
        after = delta(rel)
        box[rel] = saved
        if accepted[k]:
            intra = intra - before[0] + after[0]
            inter = inter - before[1] + after[1]
            real[rel] = moved_real
            box[rel] = moved_box
        if (k + 1) % record_every == 0:
            checkpoints.append(digest())
    return dict(checkpoints=np.array(checkpoints), calls=_RECORD["calls"], intra=intra, inter=inter, box=box)


def save_chain(path, name, res):
    idx, vec, u = res["moves"]
    np.savez_compressed(path, name=np.array(name), accepted=np.packbits(res["accepted"]),
                        steps=np.int64(len(res["accepted"])), errors=res["errors"],
                        checkpoints=res["checkpoints"], calls=np.int64(res["calls"]), intra=res["intra"],
                        inter=res["inter"], weights=res["weights"],
                        minDistance=res["grid"]["minDistance"], maxDistance=res["grid"]["maxDistance"],
                        bin=res["grid"]["bin"], histSize=np.int32(res["grid"]["histSize"]),
                        moves_sha256=np.array(hashlib.sha256(idx.tobytes() + vec.tobytes() + u.tobytes()).hexdigest()),
                        box_sha256=np.array(hashlib.sha256(np.ascontiguousarray(res["box"]).tobytes()).hexdigest()))


def load_chain(path):
    with np.load(path) as z:
        g = {k: z[k] for k in z.files}
    g["accepted"] = np.unpackbits(g["accepted"])[:int(g["steps"])].astype(bool)
    g["grid"] = dict(minDistance=F32(g["minDistance"]), maxDistance=F32(g["maxDistance"]), bin=F32(g["bin"]),
                     histSize=int(g["histSize"]))
    return g


def chain_inputs(name, steps):
    """System and moves of a recorded chain, regenerated from its seeds."""
    d = chain_definitions()[name]
    system = d["system"]()
    return system, tuple(x[:steps] for x in make_moves(system, d["steps"], d["amp"], d["group"]))
