"""Item ranges of the all-pairs kernel on the device: the counts of disjoint
ranges that cover every work item add up, bit for bit, to the full counts,
which is what makes the one-all-reduce sharding over GPUs exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3, 7])
def test_item_ranges_sum_to_full_histogram(world):
    from fullrmc_gb300 import pairs_histograms, sharding, synthetic
    s = synthetic.triclinic_100k(seed=2, n=20000)
    m = s.model
    ne = len(m.elements_count)
    args = (s.box_coords, s.basis, True, s.mol, s.el, ne, m.minDistance, m.maxDistance, m.bin, m.hs)
    nitems = sharding.full_items(s.box_coords.shape[0])
    assert nitems >= world
    total = np.zeros((2, ne, ne, m.hs), np.int64)
    for r in range(world):
        b, e = sharding.item_range(nitems, world, r)
        total += sharding.device_partial_counts(*args, b, e)
    hi, he = sharding.counts_to_histograms(total)
    want = pairs_histograms.full_pairs_histograms_coords(*args)
    assert np.array_equal(hi, want[0]) and np.array_equal(he, want[1])
    one = sharding.full_pairs_histograms_sharded(*args)  # no process group: this rank alone
    assert np.array_equal(one[0], want[0]) and np.array_equal(one[1], want[1])
    assert want[1].sum() > 0
