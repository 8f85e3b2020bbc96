"""C-ABI library checks that need no GPU: it loads, exports every declared
symbol, and its host-only helpers are exact."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


@pytest.fixture(scope="module")
def lib():
    from fullrmc_gb300 import build
    build.build()
    from fullrmc_gb300 import _native
    return _native.load()


def declared_symbols():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(frmc_[a-zA-Z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("frmc_full_pairs_histograms_coords", "frmc_multiple_pairs_histograms_coords",
              "frmc_single_pairs_histograms", "frmc_pairs_distances_to_indexcoords", "frmc_gr_to_sq"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_exports(lib):
    from fullrmc_gb300 import _native
    from fullrmc_gb300 import engine  # noqa: F401  (registers the engine-module entry points)
    for n in declared_symbols():
        if n.startswith("frmc_engine") or n.startswith("frmc_serve") or n.startswith("frmc_batch"):
            continue
        assert n in _native.SIGNATURES, n


def _limits(lib, mn, mx):
    lo, hi = ctypes.c_float(), ctypes.c_float()
    assert lib.frmc_sq_limits(np.float32(mn), np.float32(mx), ctypes.byref(lo), ctypes.byref(hi)) == 0
    return np.float32(lo.value), np.float32(hi.value)


@pytest.mark.parametrize("mn,mx", [(-0.005, 15.005), (0.995, 12.005), (2.5, 20.005), (0.0, 1.0), (-1.0, 0.0),
                                   (1e-20, 3.0), (7.123, 7.124)])
def test_sq_limits_are_exact(lib, mn, mx):
    """s >= s_lo  <=>  sqrtf(s) >= min  and  s < s_hi  <=>  sqrtf(s) < max,
    checked on every float32 in a window around both thresholds."""
    mn, mx = np.float32(mn), np.float32(mx)
    lo, hi = _limits(lib, mn, mx)
    for thr, lim, pred in ((lo, mn, lambda d: d >= mn), (hi, mx, lambda d: d < mx)):
        if not np.isfinite(thr) or thr == 0:
            continue
        bits = np.arange(-2000, 2000, dtype=np.int64) + np.array(thr, np.float32).view(np.int32)
        s = bits.astype(np.int32).view(np.float32)
        s = s[s >= 0]
        d = np.sqrt(s)  # correctly rounded float32 sqrt
        if lim is mn:
            assert np.array_equal(s >= lo, pred(d))
        else:
            assert np.array_equal(s < hi, pred(d))


def test_sq_limits_degenerate(lib):
    lo, hi = _limits(lib, -0.005, 0.0)
    assert lo == 0 and hi == 0  # nothing accepted
    lo, hi = _limits(lib, 0.0, np.inf)
    assert lo == 0 and np.isinf(hi)


def test_basis_modes(lib):
    from fullrmc_gb300._native import F32P

    def mode(B, pbc=1):
        B = np.ascontiguousarray(B, np.float32)
        return lib.frmc_basis_mode(B.ctypes.data_as(F32P), pbc)
    assert mode(np.eye(3), 0) == 0
    assert mode(np.diag([3, 4, 5])) == 1
    assert mode([[103, 0, 0], [-51.5, 89.2, 0], [0, 0, 103]]) == 2
    assert mode([[10, 0, 0], [2, 9, 0], [1, 2, 8]]) == 3
    assert mode([[10, 1, 0], [2, 9, 0], [1, 2, 8]]) == 4


def test_place_positions_orders_lone_and_shared_sms(lib):
    """The measured placement's ordering (host only): CTAs alone on an SM
    take the longest items; on a shared SM the first CTA takes the longest
    remaining item and the others the shortest."""
    from fullrmc_gb300.engine import EngineSet
    sm = [0, 1, 1, 2, 2, 3]            # CTAs 0 and 5 hold SMs 0 and 3 alone
    took = [1.0, 5.0, 3.0, 6.0, 2.0, 4.0]
    # items by time: 3, 1, 5, 2, 4, 0; lone CTAs 0, 5 get 3, 1; SM 1: 5 and
    # the shortest, 0; SM 2: 2 and 4
    assert EngineSet.place_positions(sm, took).tolist() == [3, 5, 0, 2, 4, 1]
    rng = np.random.default_rng(4)
    for n in (1, 7, 256):
        sm = rng.integers(0, max(1, n // 2), n)
        took = rng.random(n)
        pos = EngineSet.place_positions(sm, took)
        assert sorted(pos.tolist()) == list(range(n))  # every item once
        lone = [b for b in range(n) if (sm == sm[b]).sum() == 1]
        if lone:
            longest = set(np.argsort(-took, kind="stable")[:len(lone)].tolist())
            assert {int(pos[b]) for b in lone} == longest
    assert EngineSet.place_positions([], []).tolist() == []
