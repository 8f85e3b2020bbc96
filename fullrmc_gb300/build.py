"""Build ``libfrmc_gpu.so`` in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` file is compiled in parallel into ``_build/`` and linked
into ``fullrmc_gb300/_lib/libfrmc_gpu.so``.  The library is rebuilt only when a
source or header is newer than it.

The library links only the static CUDA runtime: every kernel is the
library's own.

Flags that matter for parity: ``--fmad=false`` (no contraction of a*b+c; the
kernels also use explicit round-to-nearest intrinsics), IEEE division and
square root (the defaults without --use_fast_math).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libfrmc_gpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler",
            "-fvisibility=hidden", "-I" + INCLUDE, "-I" + CSRC, *extra]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        if not ptxas_info and not _stale(obj, [src, *hdrs]):
            return obj
        cmd = [cc, *_flags(["-Xptxas", "-v"] if ptxas_info else []), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose or ptxas_info:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as pool:
        objs = list(pool.map(compile_one, srcs))
    lib_changed = _stale(LIB, objs)
    if lib_changed:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [cc, ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    build_fastcall(force=lib_changed)
    return LIB


def build_fastcall(force=False):
    """The CPython fast path of the per-move drop-in calls (csrc/fastcall.c),
    compiled with the host C compiler against this interpreter's headers and
    linked to the library beside it."""
    import sysconfig
    src = os.path.join(CSRC, "fastcall.c")
    out = os.path.join(LIBDIR, "_fastcall" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))
    if not force and not _stale(out, [src, LIB, os.path.join(INCLUDE, "frmc_gpu.h")]):
        return out
    cc = os.environ.get("CC", "gcc")
    tmp = out + ".tmp%d" % os.getpid()
    cmd = [cc, "-shared", "-fPIC", "-O2", "-std=c11", "-I" + sysconfig.get_paths()["include"], "-I" + INCLUDE, src,
           "-L" + LIBDIR, "-lfrmc_gpu", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("fastcall build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
