"""FP64 CPU restatement of the learned-rebuild network (pairs_gb300/csrc/mlp.cu).

TEST INFRASTRUCTURE: the gradient check compares the GPU forward/backward kernels
with this file.  The reference has no such network (it rebuilds on a fixed period,
sim/timestep.py:47); the restatement follows the kernel's stated mathematics:

  h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), o = W3 . h2 + b3     (per cell)
  P  = m - T log sum_c exp(-(o_c - m)/T),  m = min_c o_c             (soft minimum)
  e  = P - log R;  L = e^2, or min(e, 0)^2 for a censored sample.
"""
import numpy as np

H, IN = 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAMS = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, feat):
    """Per-cell outputs (inf for empty cells) and the cached activations."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(feat, dtype=np.float64)[:, :3]
    valid = np.asarray(feat)[:, 3] > 0
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    o = h2 @ W3 + b3
    o = np.where(valid, o, np.inf)
    return o, (x, h1, h2, valid)


def softmin(o, temperature):
    v = o[np.isfinite(o)]
    m = v.min()
    z = np.exp(-(v - m) / temperature).sum()
    return m - temperature * np.log(z)


def loss_and_grad(p, feat, target_log, censored, temperature):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    o, (x, h1, h2, valid) = forward(p, feat)
    P = softmin(o, temperature)
    e = P - target_log
    if censored:
        e = min(e, 0.0)
    L = e * e
    dP = 2.0 * e
    m = o[valid].min()
    w = np.where(valid, np.exp(-(np.where(valid, o, m) - m) / temperature), 0.0)
    w = w / w.sum()
    go = dP * w                                    # dL/do_c
    g = np.zeros(NPARAMS)
    g[OFF_B3] = go.sum()
    g[OFF_W3:OFF_B3] = go @ h2
    dz2 = (go[:, None] * W3[None, :]) * (1.0 - h2 * h2)
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    dh1 = dz2 @ W2
    dz1 = dh1 * (1.0 - h1 * h1)
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    g[OFF_W1:OFF_B1] = (dz1.T @ x).ravel()
    return L, g, P
