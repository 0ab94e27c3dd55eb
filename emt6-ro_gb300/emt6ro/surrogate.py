"""Learned surrogate of the simulator for GA pre-screening.

An MLP (100 -> 512 -> 512 -> 512 -> 1, GELU) maps a protocol's dose-time
vector (96 bins of 30 min over the first 48 h, Gy per bin) plus four summary
features of the initial tumour (living cells, radius, fraction of cells in
G1, mean oxygen over occupied sites) to the mean final living-cell count of
that (protocol, tumour) pair.  It is trained only on simulator output, on the
GPU, by the library's own BF16 tensor-core kernels (include/emt6ro_surrogate.h;
forward, backward and Adam); a GA scores a whole population with it and
re-simulates only the best fraction (`ScreenedModel`), so full simulation still
decides the fitness of every protocol it keeps.

The reference has no surrogate: its GA scores every protocol by simulation
(python/emt6ro/ga_model/model.py:33-54).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _native as N

DOSE_BINS = 96
BIN_STEPS = 300           # 30 min of 6-s steps
N_FEATURES = DOSE_BINS + 4
HIDDEN = 512


def dose_vector(protocol) -> np.ndarray:
    """Gy per 30-min bin over the first 48 h; later doses are ignored."""
    v = np.zeros(DOSE_BINS, np.float32)
    for step, dose in protocol:
        b = int(step) // BIN_STEPS
        if 0 <= b < DOSE_BINS:
            v[b] += np.float32(dose)
    return v


def tumour_features(tumor) -> np.ndarray:
    """(living cells, radius, fraction in G1, mean O2 over occupied sites)."""
    s = np.asarray(getattr(tumor, "sites", tumor))
    occ = s["state"] == 1
    n = int(occ.sum())
    if n == 0:
        return np.zeros(4, np.float32)
    r, c = np.nonzero(occ)
    radius = float(np.sqrt(((r - r.mean()) ** 2 + (c - c.mean()) ** 2).max()))
    g1 = float((s["phase"][occ] == 0).mean())
    o2 = float(s["ox"][occ].mean())
    return np.array([n, radius, g1, o2], np.float32)


def features(protocols, tumors, pair_protocol, pair_tumor) -> np.ndarray:
    """Raw feature rows [n_pairs, 100] for (protocol, tumour) index pairs."""
    dv = np.stack([dose_vector(p) for p in protocols]) if len(protocols) else \
        np.zeros((0, DOSE_BINS), np.float32)
    tf = np.stack([tumour_features(t) for t in tumors])
    return np.concatenate([dv[np.asarray(pair_protocol)], tf[np.asarray(pair_tumor)]],
                          axis=1).astype(np.float32)


def simulate_means(params, tumors, protocols, pair_protocol, pair_tumor, replicates, steps,
                   seed=1, device=0, chunk=40_000):
    """Mean final living-cell count of each (protocol, tumour) pair over
    `replicates` simulations of `steps` steps (the GPU simulator)."""
    from .batch import Batch
    pp = np.asarray(pair_protocol, np.int32)
    pt = np.asarray(pair_tumor, np.int32)
    n_pairs = len(pp)
    out = np.zeros(n_pairs, np.float64)
    per = max(1, chunk // replicates)
    for lo in range(0, n_pairs, per):
        hi = min(n_pairs, lo + per)
        st = np.repeat(pt[lo:hi], replicates)
        sp = np.repeat(pp[lo:hi], replicates)
        b = Batch(params, tumors, protocols, st, sp, device=device, seed=seed + lo)
        b.run(steps)
        out[lo:hi] = b.counts().reshape(hi - lo, replicates).mean(1)
        del b
    return out


class Surrogate:
    """The MLP on one GPU.  Inputs are raw feature rows (see `features`);
    the network sees them standardised with statistics of the training set,
    and its output is de-standardised to living cells."""

    def __init__(self, max_batch: int = 4096, seed: int = 0, device: int = 0):
        import torch
        self._torch = torch
        if max_batch % 128:
            raise ValueError("max_batch must be a multiple of 128")
        self.max_batch = max_batch
        self.device = device
        h = ctypes.c_void_p()
        N.check(N.lib().emt6_mlp_create(max_batch, seed, device, ctypes.byref(h)))
        self._h = h
        self.x_mean = np.zeros(N_FEATURES, np.float32)
        self.x_std = np.ones(N_FEATURES, np.float32)
        self.y_mean = 0.0
        self.y_std = 1.0
        self.history: list[float] = []

    def close(self):
        if getattr(self, "_h", None):
            N.lib().emt6_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # ---- parameters -------------------------------------------------------
    SHAPES = [(HIDDEN, 128), (HIDDEN,), (HIDDEN, HIDDEN), (HIDDEN,), (HIDDEN, HIDDEN), (HIDDEN,),
              (HIDDEN,), (1,)]

    def get_params(self) -> list[np.ndarray]:
        out = [np.zeros(s, np.float32) for s in self.SHAPES]
        arr = (ctypes.c_void_p * 8)(*[a.ctypes.data for a in out])
        N.check(N.lib().emt6_mlp_get_params(self._h, arr))
        return out

    def set_params(self, params) -> None:
        ps = [np.ascontiguousarray(p, np.float32).reshape(s) for p, s in zip(params, self.SHAPES)]
        arr = (ctypes.c_void_p * 8)(*[a.ctypes.data for a in ps])
        N.check(N.lib().emt6_mlp_set_params(self._h, arr))

    # ---- device helpers -----------------------------------------------------
    def _stream(self):
        return self._torch.cuda.ExternalStream(N.lib().emt6_mlp_stream(self._h),
                                               device=self.device)

    def _to_dev(self, a: np.ndarray):
        torch = self._torch
        with torch.cuda.stream(self._stream()):
            return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(
                f"cuda:{self.device}", non_blocking=False)

    def _norm_x(self, x):
        return (np.asarray(x, np.float32) - self.x_mean) / self.x_std

    # ---- raw (standardised) interface used by tests ---------------------------
    def gradients(self, x_std, t_std):
        """Gradients of the MSE on one batch (standardised inputs/targets)."""
        B = len(x_std)
        xd, td = self._to_dev(x_std), self._to_dev(t_std)
        out = [np.zeros(s, np.float32) for s in self.SHAPES]
        arr = (ctypes.c_void_p * 8)(*[a.ctypes.data for a in out])
        loss = ctypes.c_float()
        N.check(N.lib().emt6_mlp_gradients(self._h, xd.data_ptr(), td.data_ptr(), B, arr,
                                           ctypes.byref(loss)))
        return out, loss.value

    def train_step(self, x_std, t_std, lr):
        B = len(x_std)
        xd, td = self._to_dev(x_std), self._to_dev(t_std)
        loss = ctypes.c_float()
        N.check(N.lib().emt6_mlp_train_step(self._h, xd.data_ptr(), td.data_ptr(), B, lr,
                                            ctypes.byref(loss)))
        return loss.value

    def predict_std(self, x_std) -> np.ndarray:
        """Network output for standardised rows (any count; padded to 128)."""
        torch = self._torch
        x = np.ascontiguousarray(x_std, np.float32)
        n = len(x)
        out = np.zeros(n, np.float32)
        if n == 0:
            return out
        xd_all = self._to_dev(x)
        with torch.cuda.stream(self._stream()):
            yd = torch.empty(self.max_batch, dtype=torch.float32, device=f"cuda:{self.device}")
            pad = torch.zeros((self.max_batch, N_FEATURES), dtype=torch.float32,
                              device=f"cuda:{self.device}")
            for lo in range(0, n, self.max_batch):
                hi = min(n, lo + self.max_batch)
                rows = hi - lo
                B = (rows + 127) // 128 * 128
                if rows == B:
                    src = xd_all[lo:hi]
                else:
                    pad[:rows].copy_(xd_all[lo:hi])
                    pad[rows:B].zero_()
                    src = pad
                N.check(N.lib().emt6_mlp_predict(self._h, src.data_ptr(), B, yd.data_ptr()))
                out[lo:hi] = yd[:rows].cpu().numpy()
        return out

    # ---- training / inference in living cells -------------------------------
    def fit(self, x, y, epochs: int = 60, lr: float = 1e-3, batch: int = 4096, seed: int = 0,
            lr_final: float = 1e-5, val_frac: float = 0.0, verbose: bool = False):
        """Adam on the MSE of standardised targets, cosine learning-rate decay
        from lr to lr_final; drops the last partial batch of each epoch.
        With val_frac > 0 that share of the rows is held out and the
        parameters of the epoch with the lowest validation error are kept."""
        x = np.asarray(x, np.float32)
        y = np.asarray(y, np.float64)
        xv = yv = None
        if val_frac > 0:
            order = np.random.default_rng(seed + 1).permutation(len(x))
            nv = max(1, int(round(val_frac * len(x))))
            xv, yv = x[order[:nv]], y[order[:nv]]
            x, y = x[order[nv:]], y[order[nv:]]
        if batch > self.max_batch or batch % 128:
            raise ValueError("batch must be a multiple of 128 up to max_batch")
        # a training set smaller than one batch trains on all of it each step
        batch = min(batch, len(x) // 128 * 128)
        # Dose bins are sparse (a protocol doses at most a few of 96), so they
        # share one scale, the root mean square of all dose entries, and are
        # not centred: a bin that is rare in the training set is not
        # magnified for an unseen protocol.  The tumour features are
        # standardised one by one; a constant one keeps its raw scale.
        d = x[:, :DOSE_BINS]
        rms = float(np.sqrt(np.mean(d.astype(np.float64) ** 2))) or 1.0
        t = x[:, DOSE_BINS:]
        sd = t.std(0)
        self.x_mean = np.concatenate([np.zeros(DOSE_BINS), t.mean(0)]).astype(np.float32)
        self.x_std = np.concatenate([np.full(DOSE_BINS, rms),
                                     np.where(sd > 1e-3, sd, 1.0)]).astype(np.float32)
        self.y_mean = float(y.mean())
        self.y_std = float(max(y.std(), 1e-6))
        xs = self._norm_x(x)
        ts = ((y - self.y_mean) / self.y_std).astype(np.float32)
        rng = np.random.default_rng(seed)
        n = len(xs)
        steps_per_epoch = max(1, n // batch)
        if batch < 128:
            raise ValueError(f"need at least 128 training rows, have {n}")
        total = epochs * steps_per_epoch
        torch = self._torch
        xd, td = self._to_dev(xs), self._to_dev(ts)
        loss = ctypes.c_float()
        k = 0
        t0 = time.perf_counter()
        best, best_params = np.inf, None
        self.val_history: list[float] = []
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)[: steps_per_epoch * batch]).to(xd.device)
            with torch.cuda.stream(self._stream()):
                xe, te = xd[perm].contiguous(), td[perm].contiguous()
                ep_loss = 0.0
                for s in range(steps_per_epoch):
                    frac = k / max(1, total - 1)
                    lr_k = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * frac))
                    want = s == steps_per_epoch - 1
                    N.check(N.lib().emt6_mlp_train_step(
                        self._h, xe[s * batch:].data_ptr(), te[s * batch:].data_ptr(), batch,
                        float(lr_k), ctypes.byref(loss) if want else None))
                    k += 1
                ep_loss = loss.value
            self.history.append(ep_loss)
            if xv is not None:
                err = float(np.mean((self.predict(xv) - yv) ** 2))
                self.val_history.append(err)
                if err < best:
                    best, best_params = err, self.get_params()
            if verbose:
                print(f"epoch {ep}: loss {ep_loss:.4f} ({time.perf_counter() - t0:.1f}s)")
        N.check(N.lib().emt6_mlp_sync(self._h))
        if best_params is not None:
            self.set_params(best_params)
        return self.history

    def predict(self, x) -> np.ndarray:
        """Predicted mean final living-cell count per raw feature row."""
        return self.predict_std(self._norm_x(x)).astype(np.float64) * self.y_std + self.y_mean


class SurrogateEnsemble:
    """k independently initialised and shuffled surrogates whose predictions
    are averaged.  Pre-screening keeps the protocols with the lowest
    predicted counts, so it also keeps the protocols whose prediction errors
    happen to be lowest; averaging members cuts the share of that error that
    differs between them, which ranks protocols better and leaves less of a
    downward bias on the kept ones."""

    def __init__(self, k: int = 5, max_batch: int = 4096, seed: int = 0, device: int = 0):
        self.nets = [Surrogate(max_batch=max_batch, seed=seed + 101 * i, device=device)
                     for i in range(k)]

    def fit(self, x, y, seed: int = 0, **kw):
        for i, net in enumerate(self.nets):
            net.fit(x, y, seed=seed + 7 * i, **kw)
        return [net.history for net in self.nets]

    def predict(self, x) -> np.ndarray:
        return np.mean([net.predict(x) for net in self.nets], axis=0)

    def close(self):
        for net in self.nets:
            net.close()


def prescreen(surrogate, protocols, tumors, keep: int):
    """Indices of the `keep` protocols with the lowest predicted mean final
    count over the tumours (highest GA fitness), and all predicted means."""
    P, T = len(protocols), len(tumors)
    pp = np.repeat(np.arange(P), T)
    pt = np.tile(np.arange(T), P)
    pred = surrogate.predict(features(protocols, tumors, pp, pt)).reshape(P, T).mean(1)
    order = np.argsort(pred, kind="stable")
    return order[:keep], pred
