"""Sharding over ranks, on the CPU.

The partition functions are checked directly.  The multi-rank path runs as
two `gloo` processes: each rank computes the integer counts of its share of
the all-pairs work with the oracle (its rows of the i < j triangle, which is
what a rank's GPU produces for its item range), and
``full_pairs_histograms_sharded`` must return, on every rank, exactly the
oracle's full_pairs_histograms_coords.
"""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from fullrmc_gb300 import sharding


def test_item_range_covers_disjointly_and_balances():
    for nitems in (0, 1, 7, 64, 1000, 12345):
        for world in (1, 2, 3, 8):
            ranges = [sharding.item_range(nitems, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == nitems
            for (b0, e0), (b1, e1) in zip(ranges, ranges[1:]):
                assert e0 == b1
            lens = [e - b for b, e in ranges]
            assert max(lens) - min(lens) <= 1
    with pytest.raises(ValueError):
        sharding.item_range(10, 2, 2)


def test_deal_assigns_every_engine_once_and_balances():
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(20000), size=256)).astype(int)
    for world in (1, 2, 4, 8):
        parts = sharding.deal(sizes, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(256))
        loads = [sum(sizes[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)
        assert parts == sharding.deal(sizes, world)  # deterministic


def test_counts_to_histograms_saturates_like_float32():
    c = np.zeros((2, 1, 1, 3), np.int64)
    c[0, 0, 0] = [5, (1 << 24) + 7, 1 << 30]
    hi, _ = sharding.counts_to_histograms(c)
    assert np.float32(np.float32(1 << 24) + np.float32(1)) == np.float32(1 << 24)
    assert hi[0, 0, 0] == 5.0 and hi[0, 0, 1] == np.float32(1 << 24) and hi[0, 0, 2] == np.float32(1 << 24)


def _system(seed=3, n=700, ne=3):
    rng = np.random.default_rng(seed)
    L = 22.0
    box = rng.random((n, 3)).astype(np.float32)
    el = rng.integers(0, ne, size=n).astype(np.int32)
    mol = (np.arange(n) // 5).astype(np.int32)
    B = np.diag([L, L, L]).astype(np.float32)
    return box, B, mol, el, ne


def _rows_for_rank(n, world, rank):
    """Row split of the i < j triangle with equal pair counts per rank."""
    pairs = np.cumsum(np.arange(n - 1, -1, -1, dtype=np.int64))
    total = pairs[-1]
    cut = [0] + [int(np.searchsorted(pairs, total * k / world)) + 1 for k in range(1, world)] + [n]
    return cut[rank], cut[rank + 1]


def _worker(rank, world, port, q):
    try:
        import torch.distributed as dist
        import oracle
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
        box, B, mol, el, ne = _system()
        args = (box, B, True, mol, el, ne, np.float32(-0.005), np.float32(9.995), np.float32(0.01), 1000)

        def partial(b, e):
            assert (b, e) == sharding.item_range(world, world, rank)
            r0, r1 = _rows_for_rank(box.shape[0], world, rank)
            idx = np.arange(r0, r1, dtype=np.int32)
            hi, he = oracle.multiple_pairs_histograms_coords(idx, box, B, True, mol, el, ne, *args[6:], allAtoms=False)
            return np.stack([hi, he]).astype(np.int64)

        hi, he = sharding.full_pairs_histograms_sharded(*args, partial=partial, nitems=world)
        want = oracle.full_pairs_histograms_coords(*args)
        q.put((rank, bool(np.array_equal(hi, want[0]) and np.array_equal(he, want[1])), float(want[1].sum())))
        dist.destroy_process_group()
    except Exception as exc:  # reported to the parent
        q.put((rank, False, repr(exc)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_all_pairs_histogram_over_two_gloo_ranks(oracle_mod):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    env_root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    old = os.environ.get("PYTHONPATH", "")
    os.environ["PYTHONPATH"] = os.pathsep.join([env_root, os.path.join(env_root, "oracle"), old])
    try:
        procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
        for p in procs:
            p.start()
        out = [q.get(timeout=120) for _ in procs]
        for p in procs:
            p.join(timeout=60)
    finally:
        os.environ["PYTHONPATH"] = old
    assert sorted(r for r, _, _ in out) == [0, 1]
    for rank, ok, info in out:
        assert ok, (rank, info)
        assert info > 0
