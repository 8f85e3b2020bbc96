"""The compiled fast path of the per-move drop-in calls declines every
argument it does not handle itself (None, lists, other dtypes, other ranks,
non-contiguous arrays, floats given for integers, None for floats), so that
the Python wrappers run their full checks and raise fullrmc's exception
types; no device is needed for these cases."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def fast():
    from fullrmc_gb300 import _native
    f = _native.fastcall()
    if f is None:
        pytest.skip("fast path not built")
    return f


def _args():
    rng = np.random.default_rng(0)
    n = 50
    return dict(idx=np.array([3, 7], np.int32), box=rng.random((n, 3)).astype(np.float32),
                B=(np.eye(3) * 10).astype(np.float32), mol=np.arange(n, dtype=np.int32),
                el=(np.arange(n) % 2).astype(np.int32))


def _multiple(fast, a, **over):
    v = dict(indexes=a["idx"], box=a["box"], B=a["B"], pbc=True, mol=a["mol"], el=a["el"], ne=2,
             mn=np.float32(0.0), mx=np.float32(5.0), bw=np.float32(0.01), hs=500, all=True, nc=1)
    v.update(over)
    return fast.multiple(v["indexes"], v["box"], v["B"], v["pbc"], v["mol"], v["el"], v["ne"], v["mn"], v["mx"],
                         v["bw"], v["hs"], v["all"], v["nc"])


@pytest.mark.parametrize("over", [
    dict(indexes=[3, 7]), dict(indexes=np.array([3, 7], np.int64)), dict(box=None),
    dict(box=np.zeros((50, 3), np.float64)), dict(box=np.zeros(150, np.float32)),
    dict(box=np.zeros((50, 6), np.float32)[:, ::2]), dict(mol=np.arange(50, dtype=np.float32)),
    dict(ne=2.0), dict(hs=np.float32(500)), dict(mn=None), dict(nc=1.5), dict(ne=2 ** 31), dict(hs=-1),
    dict(el=np.zeros(10, np.int32)), dict(box=np.zeros((50, 4), np.float32))])
def test_multiple_declines_unusual_arguments(fast, over):
    assert _multiple(fast, _args(), **over) is None


def test_full_and_transform_decline_unusual_arguments(fast):
    a = _args()
    assert fast.full(a["box"].tolist(), a["B"], True, a["mol"], a["el"], 2, 0.0, 5.0, 0.01, 500, 1) is None
    assert fast.full(a["box"], a["B"], True, a["mol"], a["el"], 2.0, 0.0, 5.0, 0.01, 500, 1) is None
    assert fast.transform(a["B"], a["box"].astype(np.float64)) is None
    assert fast.transform(a["B"].tolist(), a["box"]) is None
    assert fast.transform(a["B"], a["box"][:, :2].copy()) is None


def test_wrappers_raise_reference_exception_types_through_the_fast_path():
    from fullrmc_gb300 import pairs_histograms as ph
    a = _args()
    kw = dict(basis=a["B"], isPBC=True, moleculeIndex=a["mol"], elementIndex=a["el"], numberOfElements=2,
              minDistance=0.0, maxDistance=5.0, bin=0.01, histSize=500)
    with pytest.raises(ValueError):
        ph.multiple_pairs_histograms_coords(a["idx"], a["box"].astype(np.float64), **kw)
    with pytest.raises(TypeError):
        ph.multiple_pairs_histograms_coords(a["idx"], None, **kw)
    with pytest.raises(TypeError):
        ph.full_pairs_histograms_coords(a["box"], **dict(kw, numberOfElements=2.0))
