"""The all-pairs histogram entry point that allocates no device memory.

It exists for callers that cannot let the library call cudaMalloc -- a host
framework that owns all device memory through its own pool, or a stepping
loop that must not stall on an allocation.  Its counts live in one fixed
device array shared by every call, so these tests check that two calls in a
row (including a second, different system) give exactly the histograms of the
existing full_pairs_histograms_coords entry point, and that a histogram too
large for the array is refused with FRMC_E_ARG before any work is queued.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(torch, native, system):
    from fullrmc_gb300._native import F32P
    m = system.model
    n = system.box_coords.shape[0]
    ne = len(m.elements_count)
    dev = torch.device("cuda", 0)
    coords = torch.from_numpy(np.ascontiguousarray(system.box_coords)).to(dev)
    el = torch.from_numpy(np.ascontiguousarray(system.el)).to(dev)
    mol = torch.from_numpy(np.ascontiguousarray(system.mol)).to(dev)
    atoms4 = torch.empty((n, 4), dtype=torch.float32, device=dev)
    hintra = torch.full((ne, ne, m.hs), -1.0, dtype=torch.float32, device=dev)
    hinter = torch.full((ne, ne, m.hs), -1.0, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    native.call("frmc_dev_pack_atoms", coords.data_ptr(), el.data_ptr(), n, atoms4.data_ptr(), stream)
    B = np.ascontiguousarray(system.basis, np.float32)
    rc = native.load().frmc_dev_full_pairs_histograms_noalloc(
        atoms4.data_ptr(), mol.data_ptr(), n, B.ctypes.data_as(F32P), int(bool(system.isPBC)), ne, m.minDistance,
        m.maxDistance, m.bin, m.hs, hintra.data_ptr(), hinter.data_ptr(), stream)
    native.check(rc)
    return hintra.cpu().numpy(), hinter.cpu().numpy()


def _existing(system):
    from fullrmc_gb300 import pairs_histograms
    m = system.model
    return pairs_histograms.full_pairs_histograms_coords(
        system.box_coords, system.basis, system.isPBC, system.mol, system.el, len(m.elements_count), m.minDistance,
        m.maxDistance, m.bin, m.hs)


def test_two_calls_match_existing_entry_point():
    torch = pytest.importorskip("torch")
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300 import synthetic
    native.load()
    first = synthetic.triclinic_100k(seed=4, n=12000)
    second = synthetic.alloy_5000(seed=5, n=3000)
    for system in (first, second, first):
        got = _noalloc(torch, native, system)
        want = _existing(system)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        assert want[1].sum() > 0


def test_too_large_histogram_is_refused():
    torch = pytest.importorskip("torch")
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300._native import F32P
    lib = native.load()
    B = np.eye(3, dtype=np.float32) * 10
    dev = torch.device("cuda", 0)
    atoms4 = torch.zeros((4, 4), dtype=torch.float32, device=dev)
    mol = torch.zeros(4, dtype=torch.int32, device=dev)
    out = torch.zeros(16, dtype=torch.float32, device=dev)
    # 2 * 8 * 8 * 8193 = 1,048,704 counts > 1,048,576
    rc = lib.frmc_dev_full_pairs_histograms_noalloc(atoms4.data_ptr(), mol.data_ptr(), 4, B.ctypes.data_as(F32P), 1,
                                                    8, np.float32(0.0), np.float32(5.0), np.float32(0.01), 8193,
                                                    out.data_ptr(), out.data_ptr(), None)
    assert rc == native.FRMC_E_ARG
    assert "exceed" in native.last_error()
    assert torch.count_nonzero(out).item() == 0
