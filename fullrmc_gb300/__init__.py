"""GB300-native pair-distance and histogram path for fullrmc.

The package provides drop-in replacements of fullrmc's Cython modules
``fullrmc.Core.pairs_distances``, ``fullrmc.Core.pairs_histograms``,
``fullrmc.Core.reciprocal_space``, ``fullrmc.Core.boundary_conditions_collection``,
``fullrmc.Core.atomic_distances`` and ``fullrmc.Core.atomic_coordination``
(same signatures, bit-identical float32 results), backed by
``libfrmc_gpu.so`` (CUDA, sm_103a; C ABI in ``include/frmc_gpu.h``), plus
device-resident RMC engines (``fullrmc_gb300.engine``) and a serving loop
(``fullrmc_gb300.serve``).

``install()`` makes ``import fullrmc.Core.pairs_histograms`` (and the other
five) resolve to these modules, so fullrmc's constraints run unmodified.
"""
from __future__ import annotations

import importlib
import importlib.abc
import importlib.util
import sys

from . import (atomic_coordination, atomic_distances, boundary_conditions_collection, pairs_distances,  # noqa: F401
               pairs_histograms, reciprocal_space)
from ._native import NativeError, device_info, load  # noqa: F401

__version__ = "0.1.0"

DROPIN_MODULES = {
    "pairs_distances": pairs_distances,
    "pairs_histograms": pairs_histograms,
    "reciprocal_space": reciprocal_space,
    "boundary_conditions_collection": boundary_conditions_collection,
    "atomic_distances": atomic_distances,
    "atomic_coordination": atomic_coordination,
}


class _DropInFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    """Resolves ``<package>.Core.<module>`` to this package's modules."""

    def __init__(self, package: str):
        self.package = package
        self.targets = {"%s.Core.%s" % (package, n): m for n, m in DROPIN_MODULES.items()}

    def find_spec(self, fullname, path, target=None):
        if fullname in self.targets:
            return importlib.util.spec_from_loader(fullname, self)
        return None

    def create_module(self, spec):
        return self.targets[spec.name]

    def exec_module(self, module):
        return None


def install(package: str = "fullrmc") -> None:
    """Route ``<package>.Core.{pairs_distances, pairs_histograms, reciprocal_space,
    boundary_conditions_collection}`` to the GPU modules.

    Call it before importing fullrmc; names already bound by loaded fullrmc
    modules are rebound as well."""
    load()  # fail loudly now if the library is missing
    for f in sys.meta_path:
        if isinstance(f, _DropInFinder) and f.package == package:
            break
    else:
        sys.meta_path.insert(0, _DropInFinder(package))
    for name, mod in DROPIN_MODULES.items():
        full = "%s.Core.%s" % (package, name)
        old = sys.modules.get(full)
        sys.modules[full] = mod
        core = sys.modules.get(package + ".Core")
        if core is not None:
            setattr(core, name, mod)
        if old is not None and old is not mod:
            for mname, m in list(sys.modules.items()):
                if m is None or not mname.startswith(package + "."):
                    continue
                for attr, val in list(vars(m).items()):
                    if getattr(val, "__module__", None) == getattr(old, "__name__", None) and hasattr(mod, attr):
                        setattr(m, attr, getattr(mod, attr))
