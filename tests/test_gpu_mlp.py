"""Learned step proposer: the GPU forward / backward kernels against the float64 oracle,
training, and what the trained network gains over the plain controller."""
import numpy as np
import pytest

import mlp_ref
from redgb import bodies, types as T
from redgb.ensemble import Ensemble
from redgb.proposer import Proposer, dataset_from_log, fit, set_dither

pytestmark = pytest.mark.gpu


def _random_net(seed=0):
    rng = np.random.RandomState(seed)
    w = (rng.randn(mlp_ref.N) * 0.3).astype(np.float32)
    p = Proposer(seed)
    p.set_params(w)
    p.set_normalisation(np.zeros(8), np.ones(8))
    return p, w, rng


def test_forward_matches_oracle(gpulib):
    p, w, rng = _random_net(1)
    x = rng.randn(1000, 8).astype(np.float32)
    got = p.forward(x)
    ref, _ = mlp_ref.forward(w, x.astype(np.float64))
    assert np.max(np.abs(got - ref)) <= 2e-4 * max(1.0, np.max(np.abs(ref)))


def test_gradient_matches_oracle(gpulib):
    """FP32 accumulation on the GPU vs float64 on the CPU, same bf16-rounded weights."""
    p, w, rng = _random_net(2)
    x = rng.randn(777, 8).astype(np.float32)
    y = rng.randn(777).astype(np.float32)
    g, loss = p.gradient(x, y)
    gr, lr = mlp_ref.gradient(w, x.astype(np.float64), y.astype(np.float64))
    assert abs(loss - lr) <= 1e-4 * lr
    scale = np.max(np.abs(gr))
    assert np.max(np.abs(g - gr)) <= 2e-4 * scale
    # every parameter block carries gradient
    for a, b in [(mlp_ref.OFF_W1, mlp_ref.OFF_B1), (mlp_ref.OFF_W2, mlp_ref.OFF_B2), (mlp_ref.OFF_W3, mlp_ref.OFF_B3)]:
        assert np.any(g[a:b] != 0)


def test_training_fits_a_smooth_target(gpulib):
    rng = np.random.RandomState(3)
    x = rng.randn(20000, 8).astype(np.float32)
    y = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3]).astype(np.float32)
    p = Proposer(3)
    p.set_normalisation(np.zeros(8), np.ones(8))
    before = float(np.mean((p.forward(x) - y) ** 2))
    p.train(x, y, epochs=15, batch=256, lr=3e-3)
    after = float(np.mean((p.forward(x) - y) ** 2))
    assert after < 0.1 * before, (before, after)


def _run(disks, years, proposer=None, log=False, dither=0.0):
    ens = Ensemble(disks, bodies.thresholds(collision_factor=0.0))
    ens.set_integrator(0.001, 1e-10)
    if log:
        ens.set_step_log(1 << 20)
    if dither:
        set_dither(ens, dither, seed=7)
    if proposer is not None:
        proposer.attach(ens)
    E0 = [ens.energy(s)[0] for s in range(len(disks))]
    ens.advance(years * T.YEAR)
    st = [ens.stats(s) for s in range(len(disks))]
    dE = max(abs((ens.energy(s)[0] - E0[s]) / E0[s]) for s in range(len(disks)))
    return ens, st, dE


def test_dither_spreads_error_ratios(gpulib):
    """Dithered plain steps (training-data collection) are still judged by the error estimate:
    the run keeps its accuracy and the logged error ratios spread out."""
    disks = [bodies.config_disk("ensemble_member", seed=s, n=256) for s in (1, 2)]
    e0, st0, dE0 = _run(disks, 2.0, log=True)
    e1, st1, dE1 = _run(disks, 2.0, log=True, dither=0.15)
    # past the start-up steps (which begin from the 0.001-day initial step)
    l0, l1 = e0.step_log(), e1.step_log()
    f0 = l0["feat"][l0["step"] >= 8, 3]
    f1 = l1["feat"][l1["step"] >= 8, 3]
    assert np.std(f1) > 3 * np.std(f0)
    assert dE1 <= 1e-10 and all(s["status"] == T.SYS_DONE for s in st1)
    assert sum(s["n_failed_step"] for s in st1) > 0


def test_trained_proposer_gain(gpulib):
    """Trained on dithered attempt logs of disks with seeds 1-16 (held-out residuals from whole
    disks choose the safety factor), evaluated on seeds 65-72: the proposer must keep the
    accuracy (|dE/E| <= 1e-10 over the interval), take fewer attempts than the plain
    controller, and deliver more simulated years per second of wall time on the same disks
    (each form's interval is one graph launch, timed after a warm-up interval; the forms are
    timed in turn three times each and each keeps its best rate, so that a slow moment of
    the machine does not decide a comparison of a few per cent)."""
    import time
    import torch
    train = [bodies.config_disk("ensemble_member", seed=s, n=512) for s in range(1, 17)]
    ens, _, _ = _run(train, 60.0, log=True, dither=0.15)
    x, y, grp = dataset_from_log(ens.step_log(), 1e-10, with_groups=True)
    assert len(x) > 5000
    net, loss = fit(x, y, seed=0, epochs=40, groups=grp)
    evald = [bodies.config_disk("ensemble_member", seed=s, n=512) for s in range(65, 73)]

    def timed(proposer):
        e = Ensemble(evald, bodies.thresholds(collision_factor=0.0))
        e.set_integrator(0.001, 1e-10)
        e.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=0.0)
        if proposer is not None:
            proposer.attach(e)
        e.advance(2.0 * T.YEAR)  # warm-up: the network needs a few steps of history
        E0 = [e.energy(s)[0] for s in range(len(evald))]
        st0 = [e.stats(s) for s in range(len(evald))]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.advance(12.0 * T.YEAR)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        st = [e.stats(s) for s in range(len(evald))]
        years = sum(a["t_day"] - b["t_day"] for a, b in zip(st, st0)) / T.YEAR
        dE = max(abs((e.energy(s)[0] - E0[s]) / E0[s]) for s in range(len(evald)))
        att = sum(a["n_tried_step"] - b["n_tried_step"] for a, b in zip(st, st0))
        return years / secs, att, dE, st

    timed(None)  # first use of this shape: graph capture, caches
    runs = {"plain": [], "learned": []}
    for _ in range(3):
        runs["plain"].append(timed(None))
        runs["learned"].append(timed(net))
    rate_plain = max(r[0] for r in runs["plain"])
    rate_learned = max(r[0] for r in runs["learned"])
    _, att_plain, dE_plain, _ = runs["plain"][0]
    _, att_learned, dE_learned, st_l = runs["learned"][0]
    print(f"sim-yr/s plain {rate_plain:.1f} learned {rate_learned:.1f} ({rate_learned / rate_plain:.3f}x); attempts "
          f"{att_plain} vs {att_learned} ({att_plain / att_learned:.3f}x); dE/E {dE_plain:.2e} vs {dE_learned:.2e}; "
          f"train loss {loss:.2e}; residual std {net.residual_std:.4f}; safety {net.safety:.4f}")
    assert all(s["status"] == T.SYS_DONE for s in st_l)
    assert dE_learned <= 1e-10
    assert att_learned < att_plain
    assert rate_learned > rate_plain
    assert sum(s["n_proposed"] for s in st_l) > 0
