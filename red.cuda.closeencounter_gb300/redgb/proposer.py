"""Learned step proposer: dataset from the ensemble's attempt log, training and inference
through the library's own GPU kernels (rg_mlp_*).

Features of a step (rg_step_rec_t.feat): log10 min(d / mutual Hill radius), log10 max|a|,
log10 last accepted dt [day], log10 last error/tolerance, last attempt accepted, logs of the
last three ratios of consecutive ideal steps.  A step's ideal size is the one the
controller's error model says would have met the tolerance exactly,
dt_accepted * (tol / err_accepted)^(1/8) (the RKF7(8) error scales as dt^8).  Target:
log(ideal step / previous step's ideal step) -- the drift of the ideal step, a property of
the dynamics rather than of the controller that chose the steps.  Training logs come from
runs whose plain trial steps are dithered (rg_ens_set_dither), so that the error-ratio
feature covers the values it takes once the network chooses the steps.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib, types as T
from .api import RedError

N_PARAM = 4801
N_IN = 8


def _bind(L):
    if getattr(L, "_mlp_bound", False):
        return L
    vp, ci, cf, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint64
    sig = {
        "rg_mlp_create": [u64, ctypes.POINTER(vp)],
        "rg_mlp_destroy": [vp],
        "rg_mlp_set_normalisation": [vp, vp, vp],
        "rg_mlp_get_normalisation": [vp, vp, vp],
        "rg_mlp_get_params": [vp, vp, ci],
        "rg_mlp_set_params": [vp, vp, ci],
        "rg_mlp_forward": [vp, vp, ci, vp],
        "rg_mlp_gradient": [vp, vp, vp, ci, vp, ctypes.POINTER(cf)],
        "rg_mlp_train": [vp, vp, vp, ci, ci, ci, cf, cf, u64, ctypes.POINTER(cf)],
        "rg_ens_set_proposer": [vp, vp, ctypes.c_double, ci],
        "rg_ens_set_dither": [vp, ctypes.c_double, u64],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ci
    L._mlp_bound = True
    return L


class Proposer:
    """The 8 -> 64 -> 64 -> 1 SiLU network (BF16 weights, FP32 accumulation) on the GPU."""

    def __init__(self, seed=0):
        self._lib = _bind(lib.load())
        self.handle = ctypes.c_void_p()
        self._call("rg_mlp_create", int(seed), ctypes.byref(self.handle))

    def _call(self, name, *args):
        rc = getattr(self._lib, name)(*args)
        if rc != 0:
            raise RedError(name, rc, self._lib.rg_last_error().decode())

    def close(self):
        if self.handle:
            self._lib.rg_mlp_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_normalisation(self, mean, std):
        mean = np.ascontiguousarray(mean, np.float32)
        std = np.ascontiguousarray(std, np.float32)
        self._call("rg_mlp_set_normalisation", self.handle, T.ptr(mean), T.ptr(std))

    def normalisation(self):
        mean = np.zeros(N_IN, np.float32)
        std = np.zeros(N_IN, np.float32)
        self._call("rg_mlp_get_normalisation", self.handle, T.ptr(mean), T.ptr(std))
        return mean, std

    def params(self):
        w = np.zeros(N_PARAM, np.float32)
        self._call("rg_mlp_get_params", self.handle, T.ptr(w), N_PARAM)
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == N_PARAM
        self._call("rg_mlp_set_params", self.handle, T.ptr(w), N_PARAM)

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_IN)
        y = np.zeros(len(x), np.float32)
        self._call("rg_mlp_forward", self.handle, T.ptr(x), len(x), T.ptr(y))
        return y

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_IN)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(N_PARAM, np.float32)
        loss = ctypes.c_float()
        self._call("rg_mlp_gradient", self.handle, T.ptr(x), T.ptr(y), len(x), T.ptr(g), ctypes.byref(loss))
        return g, loss.value

    def train(self, x, y, epochs=20, batch=512, lr=2e-3, weight_decay=1e-4, seed=0):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_IN)
        y = np.ascontiguousarray(y, np.float32)
        loss = ctypes.c_float()
        self._call("rg_mlp_train", self.handle, T.ptr(x), T.ptr(y), len(x), int(epochs), int(batch), float(lr),
                   float(weight_decay), int(seed), ctypes.byref(loss))
        return loss.value

    def attach(self, ensemble, safety=None, cooldown=16):
        """Use this network for the ensemble's trial steps (see rg_ens_set_proposer); the
        default safety factor is the one fit() chose from held-out residuals."""
        if safety is None:
            safety = getattr(self, "safety", 0.9)
        self._call("rg_ens_set_proposer", ensemble.handle, self.handle, float(safety), int(cooldown))
        ensemble._proposer = self

    @staticmethod
    def detach(ensemble):
        L = _bind(lib.load())
        rc = L.rg_ens_set_proposer(ensemble.handle, None, 1.0, 0)
        if rc:
            raise RedError("rg_ens_set_proposer", rc, L.rg_last_error().decode())
        ensemble._proposer = None


def set_dither(ensemble, sigma, seed=0):
    """Dither the ensemble's plain trial steps for training-data collection (rg_ens_set_dither)."""
    L = _bind(lib.load())
    rc = L.rg_ens_set_dither(ensemble.handle, float(sigma), int(seed))
    if rc:
        raise RedError("rg_ens_set_dither", rc, L.rg_last_error().decode())


def dataset_from_log(log, tol, min_step=4, with_groups=False):
    """(X, Y) training pairs from an attempt log: one sample per accepted step, the target
    being log(ideal step / the previous accepted step's ideal step).  with_groups: also the
    disk of every sample."""
    X, Y, G = [], [], []
    order = np.argsort(log["sys"], kind="stable")
    log = log[order]
    for s in np.unique(log["sys"]):
        acc = log[(log["sys"] == s) & (log["accepted"] == 1)]
        if len(acc) < 2:
            continue
        with np.errstate(divide="ignore", invalid="ignore"):
            ideal = acc["dt"] * (tol / acc["err"]) ** (1.0 / 8.0)
            y = np.log(ideal[1:] / ideal[:-1])
        keep = (acc["step"][1:] >= min_step) & (acc["err"][1:] > 0) & (acc["err"][:-1] > 0)
        X.append(acc["feat"][1:][keep])
        Y.append(y[keep])
        G.append(np.full(int(keep.sum()), s, np.int32))
    X = np.concatenate(X).astype(np.float32).reshape(-1, N_IN) if X else np.zeros((0, N_IN), np.float32)
    Y = np.concatenate(Y).astype(np.float32) if Y else np.zeros(0, np.float32)
    G = np.concatenate(G) if G else np.zeros(0, np.int32)
    ok = np.isfinite(Y) & np.all(np.isfinite(X), axis=1)
    return (X[ok], Y[ok], G[ok]) if with_groups else (X[ok], Y[ok])


def best_safety(res, retry=0.9, grid=np.linspace(0.90, 1.0, 201)):
    """The safety factor s that minimises the expected attempts per unit of simulated time
    on held-out residuals res = y - prediction: a proposal s * ideal_last * exp(prediction)
    passes the error test when it does not exceed the ideal step, i.e. when log s <= res;
    a rejected proposal costs one more attempt, retried at about `retry` times the ideal
    step (the plain controller's rule).  Cost(s) = (1 + P) / (s (1 - P) + retry P),
    P = P(res < log s)."""
    res = np.sort(np.asarray(res, np.float64))
    best, best_cost = float(grid[0]), np.inf
    for s_ in grid:
        p = np.searchsorted(res, np.log(s_)) / max(len(res), 1)
        cost = (1.0 + p) / (s_ * (1.0 - p) + retry * p)
        if cost < best_cost:
            best, best_cost = float(s_), cost
    return best, best_cost


def fit(x, y, seed=0, epochs=30, batch=512, lr=2e-3, holdout=0.1, quantile=None, groups=None):
    """A new network standardised on (x, y)'s inputs and trained on the GPU.

    A `holdout` fraction is kept out of training -- whole disks when `groups` (the disk of
    each sample) is given, since the samples of one disk are correlated in time -- and, with
    groups, as many other disks for validation: the weights kept are those of the epoch with
    the smallest validation residual (the network fits disks it has seen better than new ones
    after a few epochs).  The returned network's `safety` minimises the expected attempts per
    unit time on the held-out residuals y - prediction (best_safety), or with `quantile` is
    exp(that quantile of them); `residual_std` is their spread and `holdout_drift_std` the
    targets' own spread on the held-out disks (the residual of predicting no drift);
    `best_epoch` is the epoch kept."""
    rng = np.random.RandomState(seed)
    val = np.zeros(0, np.int64)
    if groups is not None and len(np.unique(groups)) > 2:
        disks = np.unique(groups)
        k = max(1, int(round(len(disks) * holdout)))
        pick = rng.choice(disks, size=min(len(disks) - 1, 2 * k), replace=False)
        held, valid = pick[:k], pick[k:]
        is_hold, is_val = np.isin(groups, held), np.isin(groups, valid)
        hold, val = np.flatnonzero(is_hold), np.flatnonzero(is_val)
        train = np.flatnonzero(~is_hold & ~is_val)
    else:
        perm = rng.permutation(len(x))
        n_hold = int(len(x) * holdout)
        hold, train = perm[:n_hold], perm[n_hold:]
    p = Proposer(seed)
    mean = x[train].mean(axis=0)
    std = x[train].std(axis=0)
    std[std < 1e-6] = 1.0
    p.set_normalisation(mean, std)
    loss, best, best_w, p.best_epoch = float("nan"), np.inf, None, epochs - 1
    for ep in range(epochs):
        loss = p.train(x[train], y[train], epochs=1, batch=batch, lr=lr, seed=seed + ep)
        if len(val) > 0:
            rms = float(np.sqrt(np.mean((y[val] - p.forward(x[val])) ** 2)))
            if rms < best:
                best, best_w, p.best_epoch = rms, p.params(), ep
    if best_w is not None:
        p.set_params(best_w)
    if len(hold) > 0:
        res = y[hold] - p.forward(x[hold])
        p.residual_std = float(np.std(res))
        p.holdout_drift_std = float(np.std(y[hold]))  # the residual of predicting no drift
        if quantile is not None:
            p.safety = float(min(1.0, np.exp(np.quantile(res, quantile))))
        else:
            p.safety, p.expected_cost = best_safety(res)
    else:
        p.residual_std = float("nan")
        p.holdout_drift_std = float("nan")
        p.safety = 0.9
    return p, loss
