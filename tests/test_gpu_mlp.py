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
    """Trained on dithered attempt logs of disks with seeds 1-16, evaluated on seeds 65-70:
    the proposer must keep the accuracy (|dE/E| <= 1e-10 over the interval) and take fewer
    attempts than the plain controller; the measured gain is printed."""
    train = [bodies.config_disk("ensemble_member", seed=s, n=512) for s in range(1, 17)]
    ens, _, _ = _run(train, 20.0, log=True, dither=0.15)
    x, y = dataset_from_log(ens.step_log(), 1e-10)
    assert len(x) > 5000
    net, loss = fit(x, y, seed=0, epochs=40)
    # the network explains part of the ideal step's drift
    assert net.residual_std < np.std(y)
    evald = [bodies.config_disk("ensemble_member", seed=s, n=512) for s in range(65, 71)]
    _, plain, dE_plain = _run(evald, 10.0)
    _, learned, dE_learned = _run(evald, 10.0, proposer=net)
    att_plain = sum(s["n_tried_step"] for s in plain)
    att_learned = sum(s["n_tried_step"] for s in learned)
    rej_plain = sum(s["n_failed_step"] for s in plain) / att_plain
    rej_learned = sum(s["n_failed_step"] for s in learned) / att_learned
    print(f"attempts plain {att_plain} learned {att_learned} ({att_plain / att_learned:.3f}x); rejected "
          f"{rej_plain:.3%} vs {rej_learned:.3%}; dE/E {dE_plain:.2e} vs {dE_learned:.2e}; train loss {loss:.2e}; "
          f"drift std {np.std(y):.4f} residual std {net.residual_std:.4f} safety {net.safety:.4f}")
    assert all(s["status"] == T.SYS_DONE for s in learned)
    assert dE_learned <= 1e-10
    assert att_learned < att_plain
    assert sum(s["n_proposed"] for s in learned) > 0
