"""CPU restatement of the learned-initial-density network (test
infrastructure): the per-atom descriptors and the multilayer perceptron's
forward pass, loss and gradient, in NumPy (FP64), against which the CUDA
kernels of ttdft_public_gb300/csrc/mlp.cu are checked.  The reference has no
learned guess; its superposition guess is dft/InitialGuess.cc:573-681."""
from __future__ import annotations

import numpy as np


def descriptors(pos, n_features, mu0, dmu, eta, rc):
    """D[a, m] = sum_{b != a} exp(-eta (r_ab - mu_m)^2) (cos(pi r_ab / rc) + 1) / 2, r_ab < rc."""
    pos = np.asarray(pos, np.float64)
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=-1)
    np.fill_diagonal(d, np.inf)
    mu = mu0 + dmu * np.arange(n_features)
    fc = np.where(d < rc, 0.5 * (np.cos(np.pi * np.minimum(d, rc) / rc) + 1.0), 0.0)
    g = np.exp(-eta * (d[:, :, None] - mu[None, None, :]) ** 2) * fc[:, :, None]
    return g.sum(axis=1)


def unpack(params, sizes):
    """Per layer (W in x out row-major, b out) from the packed vector."""
    out, off = [], 0
    for i, o in zip(sizes[:-1], sizes[1:]):
        W = params[off:off + i * o].reshape(i, o)
        off += i * o
        b = params[off:off + o]
        off += o
        out.append((W, b))
    return out


def forward(params, sizes, x):
    hs = [np.asarray(x, np.float64)]
    layers = unpack(np.asarray(params, np.float64), sizes)
    for li, (W, b) in enumerate(layers):
        z = hs[-1] @ W + b
        hs.append(z if li == len(layers) - 1 else np.tanh(z))
    return hs


def loss_and_grad(params, sizes, x, t):
    """Loss = mean over samples of sum_j (y_j - t_j)^2 and its gradient."""
    hs = forward(params, sizes, x)
    layers = unpack(np.asarray(params, np.float64), sizes)
    B = x.shape[0]
    r = hs[-1] - t
    loss = float(np.sum(r * r) / B)
    d = 2.0 * r / B
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        if li != len(layers) - 1:
            d = d * (1.0 - hs[li + 1] ** 2)
        grads.append((hs[li].T @ d, d.sum(axis=0)))
        d = d @ W.T
    g = []
    for gW, gb in reversed(grads):
        g.append(gW.ravel())
        g.append(gb)
    return loss, np.concatenate(g)
