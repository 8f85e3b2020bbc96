"""Build recipe for the compiled reference (test infrastructure only).

This script compiles fullrmc's own Cython sources for the pair-distance and
histogram path -- ``Extensions/pairs_distances.pyx``,
``Extensions/pairs_histograms.pyx``, ``Extensions/reciprocal_space.pyx``,
``Extensions/boundary_conditions_collection.pyx``,
``Extensions/atomic_distances.pyx`` and ``Extensions/atomic_coordination.pyx``
-- exactly as they are, into
``oracle/_ref/fullrmc/Core/``, so that ``import fullrmc.Core.pairs_histograms``
(with ``oracle/_ref`` first on ``sys.path``) loads the reference itself.  The
reference's own ``Extensions/setup.py:63-121`` builds the same four modules
with ``include_dirs=[numpy.get_include()]`` and ``-fopenmp``.

Two stages, so that the result can be rebuilt on a machine that has neither
the reference checkout nor Cython:

1. ``cythonize``: when the reference checkout and Cython are both present,
   each ``.pyx`` is translated to C under ``oracle/_ref/src/``.
2. ``compile``: every ``oracle/_ref/src/*.c`` is compiled with ``gcc`` against
   this interpreter's headers and numpy's headers.

``-ffp-contract=off`` is added to the reference's own flags: on x86-64 (no FMA
in the baseline ISA) gcc never contracts ``a*b+c``, while on aarch64 gcc
contracts by default.  With the flag the reference gives the same float32
results on both machines.

Nothing in the product imports this module or its output.  ``oracle/_ref`` is
listed in ``.gitignore`` and nothing from it is committed.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_OUT, "src")
PKG_DIR = os.path.join(REF_OUT, "fullrmc", "Core")
# Where the reference checkout lies: the FRMC_REFERENCE_ROOT environment
# variable or `--reference-root` on the command line; the default is this
# recipe's checkout location.  Without the checkout, stage 2 still compiles
# the C of an earlier stage 1.
REFERENCE_ROOT = os.environ.get("FRMC_REFERENCE_ROOT", "/root/reference")
MODULES = ("pairs_distances", "pairs_histograms", "reciprocal_space",
           "boundary_conditions_collection", "atomic_distances", "atomic_coordination")


def _cythonize() -> bool:
    ext_dir = os.path.join(REFERENCE_ROOT, "Extensions")
    if not os.path.isdir(ext_dir):
        return False
    try:
        import Cython  # noqa: F401
    except ImportError:
        return False
    os.makedirs(SRC_DIR, exist_ok=True)
    for name in MODULES:
        pyx = os.path.join(ext_dir, name + ".pyx")
        out = os.path.join(SRC_DIR, name + ".c")
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(pyx):
            continue
        cmd = [sys.executable, "-m", "cython", "-3", "--module-name",
               "fullrmc.Core." + name, "-o", out, pyx]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
    return True


def _compile_one(csrc: str) -> str:
    import numpy as np
    name = os.path.splitext(os.path.basename(csrc))[0]
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(PKG_DIR, name + suffix)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(csrc):
        return out
    cmd = ["gcc", "-shared", "-fPIC", "-O2", "-fwrapv", "-fno-strict-aliasing",
           "-ffp-contract=off", "-fopenmp", "-DNDEBUG", "-w",
           "-I" + sysconfig.get_paths()["include"], "-I" + np.get_include(),
           "-o", out, csrc]
    subprocess.run(cmd, check=True)
    return out


def build() -> bool:
    """Build ``oracle/_ref``; returns True when all four modules exist."""
    _cythonize()
    sources = sorted(glob.glob(os.path.join(SRC_DIR, "*.c")))
    if len(sources) < len(MODULES):
        return False
    os.makedirs(PKG_DIR, exist_ok=True)
    for d in (os.path.join(REF_OUT, "fullrmc"), PKG_DIR):
        init = os.path.join(d, "__init__.py")
        if not os.path.exists(init):
            with open(init, "w") as fh:
                fh.write("")
    with ThreadPoolExecutor(max_workers=len(sources)) as pool:
        list(pool.map(_compile_one, sources))
    return True


def available() -> bool:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return all(os.path.exists(os.path.join(PKG_DIR, m + suffix)) for m in MODULES)


def import_reference():
    """Import the compiled reference modules; raises ImportError when absent."""
    if not available():
        raise ImportError("compiled reference not built (run oracle/build_ref.py)")
    if REF_OUT not in sys.path:
        sys.path.insert(0, REF_OUT)
    import importlib
    mods = {m: importlib.import_module("fullrmc.Core." + m) for m in MODULES}
    return mods


if __name__ == "__main__":
    if "--reference-root" in sys.argv:
        REFERENCE_ROOT = sys.argv[sys.argv.index("--reference-root") + 1]
    ok = build()
    print("reference built" if ok else "reference sources unavailable")
