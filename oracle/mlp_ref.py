"""ORACLE (test infrastructure only): float64 numpy restatement of the learned step
proposer's network (red.cuda.closeencounter_gb300/csrc/mlp.cu) -- forward pass and the
gradient of the mean squared error -- used to check the GPU training kernels.  The
weights are rounded to bfloat16 first, as the GPU kernels read them."""
import numpy as np

H, I = 64, 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * I
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
N = OFF_B3 + 1


def bf16(w):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    u = np.asarray(w, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = bf16(w)
    return (w[OFF_W1:OFF_B1].reshape(H, I), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(H, H), w[OFF_B2:OFF_W3],
            w[OFF_W3:OFF_B3], w[OFF_B3])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, x):
    W1, b1, W2, b2, w3, b3 = unpack(w)
    z1 = x @ W1.T + b1
    z2 = silu(z1) @ W2.T + b2
    return silu(z2) @ w3 + b3, (z1, z2)


def gradient(w, x, y):
    """dL/dw of L = mean((f(x) - y)^2), and L; x already standardised."""
    W1, b1, W2, b2, w3, b3 = unpack(w)
    out, (z1, z2) = forward(w, x)
    n = len(x)
    r = out - y
    d = 2.0 * r / n
    g = np.zeros(N)
    h2 = silu(z2)
    g[OFF_W3:OFF_B3] = d @ h2
    g[OFF_B3] = d.sum()
    dz2 = np.outer(d, w3) * dsilu(z2)
    h1 = silu(z1)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * dsilu(z1)
    g[OFF_W1:OFF_B1] = (dz1.T @ x).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return g, float(np.mean(r * r))
