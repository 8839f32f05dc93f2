"""ORACLE — test infrastructure only.

NumPy float64 restatement of the learned-guess MLP (5 -> 32 -> 32 -> 1, tanh)
forward pass and of the gradient of the mean squared error of its normalised
output, used to check the CUDA training kernels.  Parameter layout as in
include/trixiatmo_gpu.h (tag_set_mlp).
"""
import numpy as np

N_IN, N_H = 5, 32


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_H * N_IN].reshape(N_H, N_IN); o += N_H * N_IN
    b1 = p[o:o + N_H]; o += N_H
    W2 = p[o:o + N_H * N_H].reshape(N_H, N_H); o += N_H * N_H
    b2 = p[o:o + N_H]; o += N_H
    W3 = p[o:o + N_H]; o += N_H
    b3 = p[o]; o += 1
    mu = p[o:o + N_IN]; o += N_IN
    sc = p[o:o + N_IN]; o += N_IN
    om, osc = p[o], p[o + 1]
    return W1, b1, W2, b2, W3, b3, mu, sc, om, osc


def forward(p, X):
    W1, b1, W2, b2, W3, b3, mu, sc, om, osc = unpack(p)
    x = (np.asarray(X, dtype=np.float64) - mu) * sc
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return om + osc * (h2 @ W3 + b3)


def loss_grad(p, X, T):
    """Mean over samples of (y_norm - t_norm)^2 and its gradient w.r.t. the
    1281 trainable parameters (same order as the layout)."""
    W1, b1, W2, b2, W3, b3, mu, sc, om, osc = unpack(p)
    x = (np.asarray(X, dtype=np.float64) - mu) * sc
    t = (np.asarray(T, dtype=np.float64) - om) / osc
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    y = h2 @ W3 + b3
    n = x.shape[0]
    e = y - t
    loss = np.mean(e * e)
    dy = 2.0 * e / n
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    d2 = (dy[:, None] * W3[None, :]) * (1 - h2 * h2)
    gW2 = d2.T @ h1
    gb2 = d2.sum(axis=0)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    gW1 = d1.T @ x
    gb1 = d1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g
