"""The launch order (emt6_test_order): before every chunk of steps the
simulations are sorted on the device by the region their next step
diffuses, largest first, simulations already at their target step (or
horizon) last.  Checked: the order is a permutation of the simulations and
its keys never decrease; the keys are the (rows, columns) of each stored ROI
plus its ring.  Results never depend on the order (every draw is keyed by
the simulation): the bit-exact whole-simulation tests run through it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = 4096


def _keys(roi, step, horizon, t_end):
    h, w = roi[:, 2], roi[:, 3]
    nr = np.clip(h + 2, 0, 62)
    nc = np.clip(w + 2, 0, 63)
    key = (KEYS - 2) - (nr * 64 + nc)
    stop = np.minimum(t_end, horizon) if horizon is not None else np.full_like(step, t_end)
    return np.where(step >= stop, KEYS - 1, key)


@pytest.mark.parametrize("n,with_horizon", [(1, False), (7, True), (1000, False), (40_000, True)])
def test_order_is_a_sorted_permutation(n, with_horizon):
    from emt6ro import _native as N
    rng = np.random.default_rng(n)
    roi = np.zeros((n, 8), np.int32)
    roi[:, 2] = rng.integers(0, 52, n)
    roi[:, 3] = np.where(rng.random(n) < 0.8, roi[:, 2], rng.integers(0, 52, n))
    roi[rng.random(n) < 0.05, 2:4] = 0  # no living cell: empty ROI
    step = rng.integers(0, 1300, n).astype(np.uint32)
    horizon = rng.integers(600, 2000, n).astype(np.uint32) if with_horizon else None
    t_end = 1200
    order = np.zeros(n, np.int64)
    N.check(N.lib().emt6_test_order(N.ptr(roi), N.ptr(step),
                                    N.ptr(horizon) if horizon is not None else None, n, t_end,
                                    N.ptr(order), 0))
    assert np.array_equal(np.sort(order), np.arange(n))
    k = _keys(roi, step, horizon, t_end)[order]
    assert (np.diff(k) >= 0).all()
    if n > 1:
        assert k[0] < k[-1] or len(np.unique(k)) == 1
