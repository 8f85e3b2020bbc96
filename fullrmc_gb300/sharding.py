"""Sharding the path over ranks (one process per GPU).

* All-pairs histogram: the tiled kernel's work items (pairs of atom tiles of
  the upper triangle, ``frmc_full_items``) are split into contiguous balanced
  ranges, one per rank.  Each rank counts the pairs of its items on its own
  GPU (``frmc_dev_full_hist_counts_range``) into integer counts
  [2][ne][ne][hs]; one sum all-reduce of those counts is the whole exchange.
  Integer sums do not depend on their order, so the result is bit-identical
  to a single GPU's, and the float32 histograms follow from the summed counts
  exactly as on one GPU (sequential float32 additions of 1.0 saturate at
  2^24).
* Engines and served fits are independent chains: they are dealt to ranks
  with no exchange at all (``deal``).
* A single chain's step is too small to shard: replicas only.
"""
from __future__ import annotations

import numpy as np

F32_SATURATION = 1 << 24  # float32 + 1.0 stops growing here


def item_range(nitems: int, world: int, rank: int):
    """Contiguous [begin, end) of `nitems` work items for `rank` of `world`;
    the ranges of all ranks are disjoint, cover every item and differ in
    length by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    q, r = divmod(int(nitems), world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def deal(sizes, world: int):
    """Assign independent engines (sizes = their atom counts, the per-step
    cost) to `world` ranks: largest first, each to the least-loaded rank
    (ties to the lowest rank).  Returns one list of engine indexes per rank,
    each in increasing order."""
    sizes = [int(s) for s in sizes]
    load = [0] * world
    out = [[] for _ in range(world)]
    for k in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda j: (load[j], j))
        out[r].append(k)
        load[r] += sizes[k]
    return [sorted(x) for x in out]


def counts_to_histograms(counts):
    """(hintra, hinter) float32 from summed integer counts [2][ne][ne][hs],
    equal to the float32 accumulation of unit increments."""
    c = np.minimum(np.asarray(counts, np.int64), F32_SATURATION)
    return c[0].astype(np.float32), c[1].astype(np.float32)


def device_partial_counts(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements, minDistance,
                          maxDistance, bin, histSize, item_begin, item_end, device=None):
    """Counts [2][ne][ne][hs] (int64) of work items [item_begin, item_end) of
    the all-pairs histogram, computed on this rank's GPU."""
    import torch
    from . import _native as native
    from ._native import F32P
    n = boxCoords.shape[0]
    ne, hs = int(numberOfElements), int(histSize)
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    c = torch.from_numpy(np.ascontiguousarray(boxCoords, np.float32)).to(dev)
    el = torch.from_numpy(np.ascontiguousarray(elementIndex, np.int32)).to(dev)
    mol = torch.from_numpy(np.ascontiguousarray(moleculeIndex, np.int32)).to(dev)
    a4 = torch.empty((n, 4), dtype=torch.float32, device=dev)
    cnt = torch.zeros(2 * ne * ne * hs, dtype=torch.int32, device=dev)
    B = np.ascontiguousarray(basis, np.float32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    native.call("frmc_dev_pack_atoms", c.data_ptr(), el.data_ptr(), n, a4.data_ptr(), stream)
    native.call("frmc_dev_full_hist_counts_range", a4.data_ptr(), mol.data_ptr(), n, B.ctypes.data_as(F32P),
                int(bool(isPBC)), ne, np.float32(minDistance), np.float32(maxDistance), np.float32(bin), hs,
                int(item_begin), int(item_end), cnt.data_ptr(), stream)
    out = cnt.cpu().numpy().view(np.uint32).astype(np.int64)
    return out.reshape(2, ne, ne, hs)


def full_items(n: int) -> int:
    """Work items of the tiled all-pairs kernel for n atoms."""
    import ctypes
    from . import _native as native
    v = ctypes.c_int64()
    native.call("frmc_full_items", int(n), ctypes.byref(v))
    return v.value


def full_pairs_histograms_sharded(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                                  minDistance, maxDistance, bin, histSize, group=None, partial=None, nitems=None):
    """full_pairs_histograms_coords over the ranks of a torch.distributed
    group (the default group when initialised, else this process alone).

    `partial(begin, end)` returns the int64 counts [2][ne][ne][hs] of work
    items [begin, end) (default: this rank's GPU); `nitems` the item count
    (default: the tiled kernel's for n atoms).  Every rank returns the full
    (hintra, hinter)."""
    import torch
    import torch.distributed as dist
    on = dist.is_available() and dist.is_initialized()
    world = dist.get_world_size(group) if on else 1
    rank = dist.get_rank(group) if on else 0
    n = int(np.asarray(boxCoords).shape[0])
    if nitems is None:
        nitems = full_items(n)
    b, e = item_range(nitems, world, rank)
    if partial is None:
        def partial(b0, e0):
            return device_partial_counts(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
                                         minDistance, maxDistance, bin, histSize, b0, e0)
    counts = np.ascontiguousarray(partial(b, e), np.int64)
    if world > 1:
        t = torch.from_numpy(counts.copy())
        if dist.get_backend(group) == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        counts = t.cpu().numpy()
    return counts_to_histograms(counts)
