"""Host-side LGL nodal basis (the arrays Trixi's `LobattoLegendreBasis` holds).

Nodes and weights by Newton iteration on q = L_{N+1} - L_{N-1} (Kopriva,
"Implementing Spectral Methods for PDEs", 2009, Alg. 25); derivative matrix
from barycentric weights (Alg. 37); D_split = 2 D - M^{-1} B.  These are the
`dg.basis` arrays TrixiAtmo's kernels read (derivative_split at
src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:140).
"""
from __future__ import annotations

import numpy as np


def _legendre(N, x):
    if N == 0:
        return 1.0, 0.0
    if N == 1:
        return x, 1.0
    L2, L1, d2, d1 = 1.0, x, 0.0, 1.0
    L, dL = L1, d1
    for k in range(2, N + 1):
        L = (2 * k - 1) / k * x * L1 - (k - 1) / k * L2
        dL = d2 + (2 * k - 1) * L1
        L2, L1, d2, d1 = L1, L, d1, dL
    return L, dL


def lgl_nodes_weights(polydeg: int):
    N = polydeg
    if N == 1:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    x = np.zeros(N + 1)
    w = np.zeros(N + 1)
    x[0], x[N] = -1.0, 1.0
    w[0] = w[N] = 2.0 / (N * (N + 1))
    for j in range(1, (N + 1) // 2):
        xj = -np.cos((j + 0.25) * np.pi / N - 3.0 / (8.0 * N * np.pi * (j + 0.25)))
        for _ in range(100):
            Lp, dLp = _legendre(N + 1, xj)
            Lm, dLm = _legendre(N - 1, xj)
            delta = -(Lp - Lm) / (dLp - dLm)
            xj += delta
            if abs(delta) <= 4e-16 * abs(xj):
                break
        LN, _ = _legendre(N, xj)
        x[j], x[N - j] = xj, -xj
        w[j] = w[N - j] = 2.0 / (N * (N + 1) * LN * LN)
    if N % 2 == 0:
        LN, _ = _legendre(N, 0.0)
        x[N // 2] = 0.0
        w[N // 2] = 2.0 / (N * (N + 1) * LN * LN)
    return x, w


def barycentric_weights(x):
    n = len(x)
    lam = np.ones(n)
    for j in range(1, n):
        for k in range(j):
            lam[k] *= x[k] - x[j]
            lam[j] *= x[j] - x[k]
    return 1.0 / lam


def derivative_matrix(x):
    n = len(x)
    lam = barycentric_weights(x)
    D = np.zeros((n, n))
    for i in range(n):
        diag = 0.0
        for j in range(n):
            if i != j:
                D[i, j] = lam[j] / lam[i] / (x[i] - x[j])
                diag -= D[i, j]
        D[i, i] = diag
    return D


def interpolation_matrix(x_from, x_to):
    lam = barycentric_weights(x_from)
    V = np.zeros((len(x_to), len(x_from)))
    for k, t in enumerate(x_to):
        hit = np.nonzero(x_from == t)[0]
        if len(hit):
            V[k, hit[0]] = 1.0
            continue
        r = lam / (t - x_from)
        V[k] = r / r.sum()
    return V


class LobattoLegendreBasis:
    """`Trixi.LobattoLegendreBasis(polydeg)` host arrays."""

    def __init__(self, polydeg: int):
        self.polydeg = polydeg
        self.nodes, self.weights = lgl_nodes_weights(polydeg)
        self.n = polydeg + 1
        D = derivative_matrix(self.nodes)
        self.derivative_matrix = D
        Ds = 2.0 * D
        Ds[0, 0] += 1.0 / self.weights[0]
        Ds[-1, -1] -= 1.0 / self.weights[-1]
        self.derivative_split = Ds
        self.derivative_hat = -(D.T * self.weights[None, :]) / self.weights[:, None]

    def nnodes(self):
        return self.n
