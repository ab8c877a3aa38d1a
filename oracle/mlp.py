"""FP64 reference of the warm-start MLP (test infrastructure).

Forward z_l = h_{l-1} W_l^T + b_l, h_l = gelu_tanh(z_l) for the three hidden
layers, y = z_4 (first 3 outputs), loss = mean((y - t)^2) over all rows and
the 3 outputs; gradients by back-propagation in FP64.  GELU uses the tanh
form 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) (Hendrycks & Gimpel
2016).  The GPU kernels compute the same network in BF16 with FP32
accumulation; this module is the checker for their gradients.
"""

from __future__ import annotations

import numpy as np

_K0 = np.sqrt(2.0 / np.pi)
_K1 = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_K0 * (x + _K1 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(_K0 * (x + _K1 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _K0 * (1.0 + 3.0 * _K1 * x * x)


def loss_and_grads(Ws, bs, X, T):
    """Ws[l]: (n_l, k_l), bs[l]: (n_l,), X: (M, k_0), T: (M, 3).  Returns loss, dWs, dbs."""
    hs, zs = [X], []
    h = X
    for l in range(3):
        z = h @ Ws[l].T + bs[l]
        zs.append(z)
        h = gelu(z)
        hs.append(h)
    y = h @ Ws[3].T + bs[3]
    M = X.shape[0]
    d = y[:, :3] - T
    loss = float(np.mean(d ** 2))
    dy = np.zeros_like(y)
    dy[:, :3] = 2.0 * d / (M * 3)
    dWs, dbs = [None] * 4, [None] * 4
    dWs[3] = dy.T @ hs[3]
    dbs[3] = dy.sum(0)
    dh = dy @ Ws[3]
    for l in (2, 1, 0):
        dz = dh * gelu_grad(zs[l])
        dWs[l] = dz.T @ hs[l]
        dbs[l] = dz.sum(0)
        dh = dz @ Ws[l]
    return loss, dWs, dbs
