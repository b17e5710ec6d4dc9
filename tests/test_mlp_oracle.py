"""The float64 network restatement used to check the GPU kernels: its gradient against
central finite differences (CPU only)."""
import numpy as np

import mlp_ref


def test_reference_gradient_matches_finite_differences():
    rng = np.random.RandomState(0)
    w = (rng.randn(mlp_ref.N) * 0.2).astype(np.float32)
    # exactly representable in bfloat16 so the perturbation is seen by the rounding
    w = mlp_ref.bf16(w).astype(np.float32)
    x = rng.randn(16, 8)
    y = rng.randn(16)
    g, _ = mlp_ref.gradient(w, x, y)
    for k in rng.choice(mlp_ref.N, 40, replace=False):
        # perturb along one weight in a way bf16 keeps: change the weight by a power of two
        base = float(w[k]) if w[k] != 0 else 1.0
        h = 2.0 ** (np.floor(np.log2(abs(base))) - 6)
        wp, wm = w.astype(np.float64).copy(), w.astype(np.float64).copy()
        wp[k] += h
        wm[k] -= h
        fp = np.mean((mlp_ref.forward(wp.astype(np.float32), x)[0] - y) ** 2)
        fm = np.mean((mlp_ref.forward(wm.astype(np.float32), x)[0] - y) ** 2)
        fd = (fp - fm) / (2 * h)
        assert abs(fd - g[k]) <= 2e-3 * max(1.0, abs(g[k])) + 1e-6, (k, fd, g[k])


def test_proposer_safety_minimises_expected_attempts():
    """best_safety: with no residual below log(0.9) the optimum is past the plain
    controller's 0.9; a wider residual spread calls for a smaller factor; the cost it reports
    is (1 + P) / (s (1 - P) + 0.9 P) at its choice."""
    from redgb.proposer import best_safety
    rng = np.random.RandomState(3)
    narrow = rng.normal(0.0, 0.004, 20000)
    wide = rng.normal(0.0, 0.02, 20000)
    s_n, c_n = best_safety(narrow)
    s_w, c_w = best_safety(wide)
    assert 0.97 < s_n < 1.0 and s_w < s_n and c_w > c_n
    p = np.mean(narrow < np.log(s_n))
    assert abs(c_n - (1 + p) / (s_n * (1 - p) + 0.9 * p)) < 1e-12
    assert c_n < 1.0 / 0.9  # better than the plain controller's fixed 0.9
