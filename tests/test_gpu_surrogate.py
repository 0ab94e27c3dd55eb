"""Surrogate MLP on the GPU through the C ABI: the tcgen05 BF16 GEMM against
float64 products of the same BF16 inputs, the forward pass, gradients and one
Adam step against the CPU oracle (oracle/mlp_oracle.py), and training on
simulator output: held-out accuracy and what pre-screening with the trained
network gains over pre-screening without it (a random subset)."""
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


@pytest.mark.parametrize("K", [128, 1024])
def test_gemm_pipeline_wait_timeout_returns_an_error_and_leaves_the_gpu_usable(K):
    """The failure path of the bounded mbarrier waits, made to happen: the
    test hook has the MMA issuer wait 200 us on a barrier nothing arrives on.
    It gives up, the producer stops issuing, the CTA waits for the loads it
    issued, frees its tensor memory and returns; the call reports
    EMT6_ERR_DEVICE.  The same GEMM then runs normally on the same inputs
    (with K = 128 every load is issued before the issuer gives up, with
    K = 1024 the producer is stopped mid-way)."""
    import torch
    from emt6ro import _native as Nat
    from oracle import mlp_oracle as mo
    M = N = 256
    rng = np.random.default_rng(K)
    a = rng.normal(size=(M, K)).astype(np.float32)
    b = rng.normal(size=(N, K)).astype(np.float32)
    da = torch.from_numpy(_bf16_bits(a).view(np.int16)).cuda()
    db = torch.from_numpy(_bf16_bits(b).view(np.int16)).cuda()
    dc = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L = Nat.lib()
    rc = L.emt6_test_mlp_gemm_timeout(da.data_ptr(), db.data_ptr(), dc.data_ptr(), M, N, K, 200,
                                      None)
    assert rc == Nat.EMT6_ERR_DEVICE
    assert "timed out" in L.emt6_last_error().decode()
    Nat.check(L.emt6_test_mlp_gemm(da.data_ptr(), db.data_ptr(), dc.data_ptr(), M, N, K, None))
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


def test_split_k_weight_gradients_agree():
    """The weight-gradient GEMMs with the batch dimension split over 2, 4 or 8
    CTAs (partial tiles reduced in a fixed order) agree with the unsplit
    kernel, and one Adam step through the split path (reduce kernel) agrees
    with the fused Adam epilogue."""
    from emt6ro import _native as Nat
    net, _ = _net(7)
    rng = np.random.default_rng(8)
    x = rng.normal(size=(1024, 100)).astype(np.float32)
    t = rng.normal(size=1024).astype(np.float32)
    grads = {}
    for sp in (1, 2, 4, 0):
        Nat.check(Nat.lib().emt6_mlp_set_splitk(net._h, sp))
        grads[sp], _ = net.gradients(x, t)
    for sp in (2, 4, 0):
        for a, b in zip(grads[sp], grads[1]):
            assert _rel(a, b) < 1e-5
    stepped = {}
    for sp in (1, 4):
        fresh, _ = _net(7)          # fresh Adam state
        Nat.check(Nat.lib().emt6_mlp_set_splitk(fresh._h, sp))
        fresh.train_step(x, t, 1e-3)
        stepped[sp] = fresh.get_params()
    for a, b in zip(stepped[1], stepped[4]):
        assert np.mean(np.isclose(a, b, rtol=1e-4, atol=1e-6)) > 0.995
    with pytest.raises(Nat.NativeError, match="splits"):
        Nat.check(Nat.lib().emt6_mlp_set_splitk(net._h, 3))


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
def dataset_48h():
    """3,072 (protocol, tumour) pairs of the GA workload, one simulation each
    at a 48-h horizon (28,800 steps): 3,072 distinct 10-Gy protocols, each
    with one of the 20 GA tumours."""
    from emt6ro import workloads as wl, surrogate as s
    params = wl.default_parameters()
    tumors = wl.ga_tumors(params, 20)
    protocols = wl.ga_protocols(3072, seed=77)
    pp = np.arange(3072)
    pt = np.random.default_rng(3).integers(0, 20, 3072)
    y = s.simulate_means(params, tumors, protocols, pp, pt, replicates=1, steps=28_800, seed=5)
    x = s.features(protocols, tumors, pp, pt)
    return x, y


def _spearman(a, b):
    return np.corrcoef(np.argsort(np.argsort(a)), np.argsort(np.argsort(b)))[0, 1]


@pytest.fixture(scope="module")
def trained(dataset_48h):
    from emt6ro.surrogate import Surrogate
    x, y = dataset_48h
    net = Surrogate(max_batch=512, seed=1)
    net.fit(x[:2560], y[:2560], epochs=100, lr=1e-3, batch=512)
    return net


def test_training_beats_mean_predictor(dataset_48h, trained):
    x, y = dataset_48h
    hist = trained.history
    assert hist[-1] < 0.7 * hist[0]
    pred = trained.predict(x[2560:])
    rmse = np.sqrt(np.mean((pred - y[2560:]) ** 2))
    base = np.sqrt(np.mean((y[:2560].mean() - y[2560:]) ** 2))
    assert rmse < 0.85 * base, (rmse, base)
    assert _spearman(pred, y[2560:]) > 0.5


def test_prescreening_beats_random_subset(dataset_48h, trained):
    """What the trained network gains: among 512 held-out pairs, the tenth it
    ranks best has a lower simulated mean count than 99% of random tenths
    (pre-screening without the network)."""
    x, y = dataset_48h
    pred = trained.predict(x[2560:])
    held = y[2560:]
    keep = len(held) // 10
    elite = np.argsort(pred)[:keep]
    rng = np.random.default_rng(0)
    random_means = [held[rng.choice(len(held), keep, replace=False)].mean() for _ in range(5000)]
    assert held[elite].mean() < np.percentile(random_means, 1)


def test_validation_keeps_best_epoch(dataset_48h):
    from emt6ro.surrogate import Surrogate
    x, y = dataset_48h
    net = Surrogate(max_batch=512, seed=4)
    net.fit(x[:1280], y[:1280], epochs=30, lr=1e-3, batch=256, val_frac=0.2)
    assert len(net.val_history) == 30
    xv_err = min(net.val_history)
    # the kept parameters reproduce the best validation error
    order = np.random.default_rng(1).permutation(1280)
    nv = 256
    xv, yv = x[:1280][order[:nv]], y[:1280][order[:nv]]
    assert np.mean((net.predict(xv) - yv) ** 2) == pytest.approx(xv_err, rel=1e-5)


def test_screened_model_simulates_only_the_elites(params, trained):
    """ScreenedModel.predict: the drop-in for EMT6RoModel.predict that scores
    every protocol with the surrogate and simulates only the best fraction;
    elites carry their simulated fitness, the rest the predicted one."""
    from emt6ro import workloads as wl
    from emt6ro.ga_model import ScreenedModel, EMT6RoModel
    tumors = wl.ga_tumors(params, 20)[:2]
    protocols = wl.ga_protocols(12, seed=5)
    model = ScreenedModel(params, tumors, trained, num_tests=2, keep_frac=0.25, num_steps=28_800,
                          seed=3)
    fit = model.predict(protocols)
    assert fit.shape == (12,)
    elite = model.last["elite"]
    assert len(elite) == 3
    assert np.allclose(fit[elite], 1500 - model.last["simulated"])
    rest = np.setdiff1d(np.arange(12), elite)
    from emt6ro.surrogate import prescreen
    _, pred = prescreen(trained, protocols, tumors, 3)
    assert np.allclose(fit[rest], 1500 - pred[rest])
    # the elites' simulated fitness is what the plain model gives them
    plain = EMT6RoModel(params, tumors, 3, 2, num_steps=28_800, seed=3)
    assert np.allclose(plain.predict([protocols[i] for i in elite]), fit[elite])


def test_ensemble_averages_its_members(dataset_48h):
    from emt6ro.surrogate import SurrogateEnsemble
    x, y = dataset_48h
    ens = SurrogateEnsemble(k=2, max_batch=512, seed=9)
    ens.fit(x[:2560], y[:2560], epochs=20, lr=1e-3, batch=512)
    members = [net.predict(x[2560:]) for net in ens.nets]
    assert not np.allclose(members[0], members[1])           # independent members
    assert np.allclose(ens.predict(x[2560:]), np.mean(members, axis=0))
