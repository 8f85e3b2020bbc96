"""The all-pairs histogram entry point that allocates no device memory.

It exists for callers that cannot let the library call cudaMalloc -- a host
framework that owns all device memory through its own pool, or a stepping
loop that must not stall on an allocation.  Its counts live in one fixed
device array shared by every call, so these tests check that two calls in a
row (including a second, different system) give exactly the histograms of the
existing full_pairs_histograms_coords entry point, that calls after the first
leave the device's free memory unchanged, that small, free-boundary and empty
cases agree too, and that a histogram too large for the array is refused with
FRMC_E_ARG before any work is queued.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _Call:
    """Device inputs and outputs of one call, allocated up front (so that the
    calls themselves can be checked for allocating nothing)."""

    def __init__(self, torch, native, box, el, mol, basis, isPBC, ne, minD, maxD, binw, hs):
        dev = torch.device("cuda", 0)
        n = box.shape[0]
        self.native, self.n, self.ne, self.hs = native, n, ne, hs
        self.args = (np.ascontiguousarray(basis, np.float32), int(bool(isPBC)), np.float32(minD),
                     np.float32(maxD), np.float32(binw))
        self.atoms4 = torch.empty((max(n, 1), 4), dtype=torch.float32, device=dev)
        self.mol = torch.from_numpy(np.ascontiguousarray(mol, np.int32).reshape(-1)).to(dev) if n else \
            torch.zeros(4, dtype=torch.int32, device=dev)
        self.hintra = torch.full((ne, ne, hs), -1.0, dtype=torch.float32, device=dev)
        self.hinter = torch.full((ne, ne, hs), -1.0, dtype=torch.float32, device=dev)
        self.stream = torch.cuda.current_stream().cuda_stream
        if n:
            coords = torch.from_numpy(np.ascontiguousarray(box, np.float32)).to(dev)
            elt = torch.from_numpy(np.ascontiguousarray(el, np.int32)).to(dev)
            native.call("frmc_dev_pack_atoms", coords.data_ptr(), elt.data_ptr(), n, self.atoms4.data_ptr(),
                        self.stream)

    def run(self):
        from fullrmc_gb300._native import F32P
        B, pbc, minD, maxD, binw = self.args
        self.hintra.fill_(-1.0)
        self.hinter.fill_(-1.0)
        rc = self.native.load().frmc_dev_full_pairs_histograms_noalloc(
            self.atoms4.data_ptr(), self.mol.data_ptr(), self.n, B.ctypes.data_as(F32P), pbc, self.ne, minD, maxD,
            binw, self.hs, self.hintra.data_ptr(), self.hinter.data_ptr(), self.stream)
        self.native.check(rc)

    def result(self):
        return self.hintra.cpu().numpy(), self.hinter.cpu().numpy()


def _call(torch, native, system):
    m = system.model
    return _Call(torch, native, system.box_coords, system.el, system.mol, system.basis, system.isPBC,
                 len(m.elements_count), m.minDistance, m.maxDistance, m.bin, m.hs)


def _noalloc(torch, native, system):
    c = _call(torch, native, system)
    c.run()
    return c.result()


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


def test_calls_allocate_no_device_memory():
    """After a first call on the device (its set-up), further calls leave the
    device's free memory unchanged: no cudaMalloc, no allocating library
    routine.  Inputs and outputs are allocated before the first reading."""
    torch = pytest.importorskip("torch")
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300 import synthetic
    native.load()
    calls = [_call(torch, native, synthetic.alloy_5000(seed=8, n=4000)),
             _call(torch, native, synthetic.triclinic_100k(seed=9, n=6000))]
    calls[0].run()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for c in calls:
            c.run()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_small_free_boundary_and_empty_cases():
    """0 and 1 atom (only the conversion kernels run), free boundaries
    (isPBC = 0) and an empty histogram (ne = 0) agree with the existing entry
    point, called twice in a row."""
    torch = pytest.importorskip("torch")
    from fullrmc_gb300 import _native as native
    from fullrmc_gb300 import pairs_histograms
    native.load()
    rng = np.random.default_rng(21)
    B = (np.eye(3) * 20.0).astype(np.float32)
    cases = []
    for n, ne, pbc in ((0, 2, True), (1, 2, True), (1500, 3, False), (1200, 2, True), (0, 0, True)):
        box = rng.random((n, 3)).astype(np.float32)
        if not pbc:
            box = (box * 20.0).astype(np.float32)
        el = rng.integers(0, max(ne, 1), n).astype(np.int32)
        mol = (np.arange(n) // 4).astype(np.int32)
        cases.append((box, el, mol, pbc, ne))
    for _ in range(2):
        for box, el, mol, pbc, ne in cases:
            c = _Call(torch, native, box, el, mol, B, pbc, ne, -0.005, 8.005, 0.01, 801)
            c.run()
            got = c.result()
            want = pairs_histograms.full_pairs_histograms_coords(
                box, B, pbc, mol, el, ne, np.float32(-0.005), np.float32(8.005), np.float32(0.01), 801)
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


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
