"""Surrogate MLP on the GPU through the C ABI: the tcgen05 BF16 GEMM against
float64 products of the same BF16 inputs, the forward pass, gradients and one
Adam step against the CPU oracle (oracle/mlp_oracle.py), and training on
simulator output: held-out accuracy and what pre-screening with the trained
network gains over pre-screening without it (a random subset)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(a):
    from oracle import mlp_oracle as mo
    return (mo.bf16(a).view(np.uint32) >> 16).astype(np.uint16)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 128), (512, 512, 4096),
                                   (4096, 512, 512), (512, 128, 1024)])
def test_tcgen05_gemm_matches_float64(M, N, K):
    import torch
    from emt6ro import _native as Nat
    from oracle import mlp_oracle as mo
    rng = np.random.default_rng(M + N + K)
    a = rng.normal(size=(M, K)).astype(np.float32)
    b = rng.normal(size=(N, K)).astype(np.float32)
    da = torch.from_numpy(_bf16_bits(a).view(np.int16)).cuda()
    db = torch.from_numpy(_bf16_bits(b).view(np.int16)).cuda()
    dc = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    Nat.check(Nat.lib().emt6_test_mlp_gemm(da.data_ptr(), db.data_ptr(), dc.data_ptr(), M, N, K,
                                           None))
    c = dc.cpu().numpy().astype(np.float64)
    ref = mo.bf16(a).astype(np.float64) @ mo.bf16(b).astype(np.float64).T
    scale = np.abs(mo.bf16(a)).astype(np.float64) @ np.abs(mo.bf16(b)).astype(np.float64).T
    assert np.max(np.abs(c - ref) / scale) < 1e-5


def test_gemm_rejects_unaligned_shapes():
    from emt6ro import _native as Nat
    with pytest.raises(Nat.NativeError, match="multiples"):
        Nat.check(Nat.lib().emt6_test_mlp_gemm(1, 1, 1, 100, 128, 64, None))


def _net(seed=0, max_batch=1024):
    from emt6ro.surrogate import Surrogate
    from oracle import mlp_oracle as mo
    net = Surrogate(max_batch=max_batch, seed=seed)
    params = mo.init_params(seed)
    net.set_params(params)
    return net, params


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30)


def test_params_roundtrip_and_forward_matches_oracle():
    from oracle import mlp_oracle as mo
    net, params = _net(1)
    back = net.get_params()
    for p, q in zip(params, back):
        assert np.array_equal(p, q)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(640, 100)).astype(np.float32)   # 5 x 128 rows
    y = net.predict_std(x)
    ym, _ = mo.mixed_forward(params, x)
    ye, _ = mo.exact_forward(params, x)
    assert _rel(y, ym) < 5e-3
    assert _rel(y, ye) < 3e-2
    # rows that are not a multiple of 128 are padded and dropped
    assert np.allclose(net.predict_std(x[:200]), y[:200], rtol=0, atol=1e-6)


def test_gradients_match_oracle():
    from oracle import mlp_oracle as mo
    net, params = _net(3)
    rng = np.random.default_rng(4)
    x = rng.normal(size=(1024, 100)).astype(np.float32)
    t = rng.normal(size=1024).astype(np.float32)
    g, loss = net.gradients(x, t)
    gm, loss_m = mo.mixed_gradients(params, x, t)
    ge = mo.exact_gradients(params, x, t)
    assert loss == pytest.approx(loss_m, rel=1e-3)
    names = ["W1", "b1", "W2", "b2", "W3", "b3", "w4", "b4"]
    for name, a, b, c in zip(names, g, gm, ge):
        assert _rel(a, b) < 3e-2, (name, _rel(a, b))
        assert _rel(a, c) < 8e-2, (name, _rel(a, c))
    assert np.all(g[0][:, 100:] == 0)          # padded inputs get no gradient


def test_adam_step_matches_oracle():
    from oracle import mlp_oracle as mo
    net, params = _net(5)
    rng = np.random.default_rng(6)
    x = rng.normal(size=(512, 100)).astype(np.float32)
    t = rng.normal(size=512).astype(np.float32)
    gm, _ = mo.mixed_gradients(params, x, t)
    lr = 1e-3
    net.train_step(x, t, lr)
    after = net.get_params()
    zeros = [np.zeros_like(p) for p in params]
    want, _, _ = mo.adam(params, gm, zeros, [z.copy() for z in zeros], 1, lr)
    for k, (a, w, p) in enumerate(zip(after, want, params)):
        moved, expect = a - p, w - p
        # the first Adam step moves each weight by about +-lr; entries whose
        # gradient sign differs under rounding are rare
        agree = np.isclose(moved, expect, rtol=1e-3, atol=2e-6)
        assert agree.mean() > 0.98, (k, agree.mean())
    assert np.all(after[0][:, 100:] == 0)


@pytest.fixture(scope="module")
def small_dataset():
    """2,000 (protocol, tumour) pairs of the GA workload: 20 tumours x 100
    protocols, mean of 4 replicates at a 48-h horizon (28,800 steps)."""
    from emt6ro import workloads as wl, surrogate as s
    params = wl.default_parameters()
    tumors = wl.ga_tumors(params, 20)
    protocols = wl.ga_protocols(100, seed=77)
    pp = np.repeat(np.arange(100), 20)
    pt = np.tile(np.arange(20), 100)
    y = s.simulate_means(params, tumors, protocols, pp, pt, replicates=4, steps=28_800, seed=5)
    x = s.features(protocols, tumors, pp, pt)
    return params, tumors, protocols, pp, pt, x, y


def test_training_beats_mean_predictor(small_dataset):
    from emt6ro.surrogate import Surrogate
    _, _, _, pp, pt, x, y = small_dataset
    train = pp < 80                       # hold out 20 protocols entirely
    net = Surrogate(max_batch=512, seed=1)
    hist = net.fit(x[train], y[train], epochs=150, lr=2e-3, batch=512)
    assert hist[-1] < 0.5 * hist[0]
    pred = net.predict(x[~train])
    rmse = np.sqrt(np.mean((pred - y[~train]) ** 2))
    base = np.sqrt(np.mean((y[train].mean() - y[~train]) ** 2))
    assert rmse < 0.6 * base, (rmse, base)


def test_prescreening_beats_random_subset(small_dataset):
    """What the trained network gains: among held-out protocols, the tenth it
    ranks best has a lower simulated mean count than a random tenth."""
    from emt6ro.surrogate import Surrogate, prescreen
    params, tumors, protocols, pp, pt, x, y = small_dataset
    train = pp < 80
    net = Surrogate(max_batch=512, seed=2)
    net.fit(x[train], y[train], epochs=150, lr=2e-3, batch=512)
    held = list(range(80, 100))
    sim_mean = y.reshape(100, 20).mean(1)[held]
    elite, pred = prescreen(net, [protocols[i] for i in held], tumors, keep=4)
    rng = np.random.default_rng(0)
    random_means = [sim_mean[rng.choice(20, 4, replace=False)].mean() for _ in range(2000)]
    assert sim_mean[elite].mean() < np.percentile(random_means, 10)
    rho = np.corrcoef(np.argsort(np.argsort(pred)), np.argsort(np.argsort(sim_mean)))[0, 1]
    assert rho > 0.5, rho
