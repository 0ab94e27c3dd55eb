"""Surrogate MLP on the CPU: the float64 oracle's gradients against central
finite differences (pins the oracle), the BF16-rounding oracle against the
float64 one, BF16 rounding itself, and the feature extraction."""
import numpy as np
import pytest


def _mo():
    from oracle import mlp_oracle
    return mlp_oracle


def test_bf16_rounding_is_nearest_even():
    mo = _mo()
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -2.5, 3.0e-3],
                 np.float32)
    got = mo.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1) wins;
    # 1 + 3*2^-8 ties between 1 + 2^-7 and 1 + 2^-6: even (1 + 2^-6) wins
    assert got.tolist()[:5] == [1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, -2.5]
    assert abs(got[5] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_exact_gradients_match_finite_differences():
    mo = _mo()
    rng = np.random.default_rng(3)
    params = [p.astype(np.float64) for p in mo.init_params(5)]
    x = rng.normal(size=(6, mo.IN))
    t = rng.normal(size=6)
    g = mo.exact_gradients(params, x, t)
    h = 1e-6
    for k in range(8):
        p = params[k]
        flat = p.reshape(-1)
        idxs = rng.choice(flat.size, size=min(4, flat.size), replace=False)
        if k == 0:
            idxs = [i for i in idxs if i % mo.IN_PAD < mo.IN] or [0]
        for i in idxs:
            old = flat[i]
            flat[i] = old + h
            lp = mo.exact_loss(params, x, t)
            flat[i] = old - h
            lm = mo.exact_loss(params, x, t)
            flat[i] = old
            fd = (lp - lm) / (2 * h)
            an = g[k].reshape(-1)[i]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (k, i, fd, an)


def test_mixed_precision_oracle_tracks_exact():
    mo = _mo()
    rng = np.random.default_rng(4)
    params = mo.init_params(6)
    x = rng.normal(size=(256, mo.IN)).astype(np.float32)
    t = rng.normal(size=256).astype(np.float32)
    ge = mo.exact_gradients(params, x, t)
    gm, _ = mo.mixed_gradients(params, x, t)
    for a, b in zip(gm, ge):
        assert np.linalg.norm(a - b) <= 0.05 * np.linalg.norm(b) + 1e-12
    ye, _ = mo.exact_forward(params, x)
    ym, _ = mo.mixed_forward(params, x)
    assert np.linalg.norm(ym - ye) <= 0.02 * np.linalg.norm(ye)


def test_features(params):
    from emt6ro import surrogate as s, workloads as wl
    v = s.dose_vector([(0, 1.0), (300, 2.0), (599, 0.25), (28_799, 0.5), (30_000, 9.0)])
    assert v.shape == (96,) and v[0] == 1.0 and v[1] == 2.25 and v[95] == 0.5 and v.sum() == 3.75
    f = s.tumour_features(wl.disc_tumor(params, 10, seed=0))
    assert f[0] == 317 and f[1] == pytest.approx(10.0, abs=0.5) and 0 < f[2] < 1
    x = s.features([[(0, 2.0)], []], [wl.disc_tumor(params, 5, seed=1)], [0, 1], [0, 0])
    assert x.shape == (2, 100) and x[0, 0] == 2.0 and x[1, :96].sum() == 0
