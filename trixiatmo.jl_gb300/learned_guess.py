"""Learned initial guess for the rainy saturation Newton solve.

The guess has two branches.  Where the unsaturated equilibrium is valid
(e_s(T_unsat) / (R_v T_unsat) >= rho_moist, with T_unsat = (e_int - rho_m L) /
(c_vd rho_d + c_vv rho_m + c_l rho_r)) it is exact and closed-form.  Elsewhere
a small FP32 MLP (5 -> 32 -> 32 -> 1, tanh) predicts the latent-heat offset
T* - T_unsat from (rho_dry, rho_moist, rho_rain, e_int, T_unsat), and vapour
and cloud follow from the saturation relation at that temperature.  The Newton
iteration (the reference's stage limiter, src/callbacks_stage/nonlinear_solve_dg2d.jl)
then starts from that guess with the reference's tolerance, and falls back to
the plain warm start when it has not converged after 8 updates.

Training pairs (state, converged temperature) come from the reference's Newton
algorithm run to the tolerance from the warm start (tag_newton_solve_states);
training and inference run in the library's own CUDA kernels (tag_mlp_train,
k_newton_rainy).  Parameter layout: include/trixiatmo_gpu.h (tag_set_mlp).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

N_IN, N_H = 5, 32
N_TRAIN = N_H * N_IN + N_H + N_H * N_H + N_H + N_H + 1
N_PARAMS = N_TRAIN + 2 * N_IN + 2
O_W1, O_B1 = 0, N_H * N_IN
O_W2 = O_B1 + N_H
O_B2 = O_W2 + N_H * N_H
O_W3 = O_B2 + N_H
O_B3 = O_W3 + N_H
O_IN_MEAN = O_B3 + 1
O_IN_SCALE = O_IN_MEAN + N_IN
O_OUT_MEAN = O_IN_SCALE + N_IN
O_OUT_SCALE = O_OUT_MEAN + 1

_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
C_VD, C_VV, C_L, L_VAP = 717.0, 1424.0, 4186.0, 2500000.0


def t_unsat(u):
    """Unsaturated-equilibrium temperature and internal energy of states u[..., 9]."""
    rho = u[..., 0] + u[..., 1] + u[..., 2]
    e_int = u[..., 5] - 0.5 * (u[..., 3] ** 2 + u[..., 4] ** 2) / rho
    return (e_int - u[..., 1] * L_VAP) / (C_VD * u[..., 0] + C_VV * u[..., 1] + C_L * u[..., 2]), e_int


def saturated(u, equations=None):
    """Nodes whose equilibrium is saturated (the network's branch)."""
    from .equations import CompressibleRainyEulerEquations2D
    eq = equations or CompressibleRainyEulerEquations2D()
    tu, _ = t_unsat(u)
    return ~((tu > 0) & (eq.saturation_vapour_pressure(tu) / (eq.R_v * tu) >= u[..., 1]))


def features(u):
    """Network inputs of rainy states u[..., 9] (same as mlp_inputs on the device)."""
    tu, e_int = t_unsat(u)
    return np.stack([u[..., 0], u[..., 1], u[..., 2], e_int, tu], axis=-1).astype(np.float32)


def init_params(seed=0):
    """Xavier-uniform weights, zero biases, identity normalisation."""
    rng = np.random.Generator(np.random.Philox(seed))
    p = np.zeros(N_PARAMS, dtype=np.float32)
    a1 = np.sqrt(6.0 / (N_IN + N_H))
    a2 = np.sqrt(6.0 / (2 * N_H))
    a3 = np.sqrt(6.0 / (N_H + 1))
    p[O_W1:O_B1] = rng.uniform(-a1, a1, N_H * N_IN)
    p[O_W2:O_B2] = rng.uniform(-a2, a2, N_H * N_H)
    p[O_W3:O_B3] = rng.uniform(-a3, a3, N_H)
    p[O_IN_SCALE:O_IN_SCALE + N_IN] = 1.0
    p[O_OUT_SCALE] = 1.0
    return p


def set_normalization(p, X, T):
    p[O_IN_MEAN:O_IN_MEAN + N_IN] = X.mean(axis=0)
    p[O_IN_SCALE:O_IN_SCALE + N_IN] = 1.0 / np.maximum(X.std(axis=0), 1e-30)
    p[O_OUT_MEAN] = T.mean()
    p[O_OUT_SCALE] = max(T.std(), 1e-30)
    return p


def newton_solve_states(u, mode=1, tol=1e-12, max_iterations=30, polish=0, params=None):
    """Newton solve on host states u[n, 9] (in place); returns (stats, iters)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    n = u.size // 9
    iters = np.zeros(n, dtype=np.int32)
    st = _lib.NewtonStats()
    pp = None
    if params is not None:
        params = np.ascontiguousarray(params, dtype=np.float32)
        pp = params.ctypes.data_as(_fp)
    _lib.check(_lib.load().tag_newton_solve_states(u.ctypes.data_as(_dp), n, int(mode),
                                                   float(tol), int(max_iterations), int(polish),
                                                   pp, iters.ctypes.data_as(_ip),
                                                   ctypes.byref(st)))
    return u, {"nodes": st.nodes, "updates": st.updates, "fallbacks": st.fallbacks,
               "not_converged": st.not_converged}, iters


def forward(params, X):
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.zeros(X.shape[0], dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    _lib.check(_lib.load().tag_mlp_forward(p.ctypes.data_as(_fp), X.ctypes.data_as(_fp),
                                           X.shape[0], y.ctypes.data_as(_fp)))
    return y


def loss_grad(params, X, T):
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    g = np.zeros(N_TRAIN, dtype=np.float32)
    loss = ctypes.c_float()
    _lib.check(_lib.load().tag_mlp_loss_grad(p.ctypes.data_as(_fp), X.ctypes.data_as(_fp),
                                             T.ctypes.data_as(_fp), X.shape[0],
                                             g.ctypes.data_as(_fp), ctypes.byref(loss)))
    return loss.value, g


def train(params, X, T, epochs=20, batch=4096, lr=3e-3, seed=0):
    """Adam on the GPU; returns (trained params, per-epoch loss)."""
    p = np.ascontiguousarray(params, dtype=np.float32).copy()
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    losses = np.zeros(epochs, dtype=np.float32)
    _lib.check(_lib.load().tag_mlp_train(p.ctypes.data_as(_fp), X.ctypes.data_as(_fp),
                                         T.ctypes.data_as(_fp), X.shape[0], int(epochs),
                                         int(batch), float(lr), int(seed),
                                         losses.ctypes.data_as(_fp)))
    return p, losses


def sample_states(n, seed=11, equations=None):
    """States from the benchmark's moist distribution at random heights in
    [0, 10 km] (training set)."""
    from .equations import CompressibleRainyEulerEquations2D
    from .initial_conditions import MoistBubbleRainy
    eq = equations or CompressibleRainyEulerEquations2D()
    rng = np.random.Generator(np.random.Philox(seed + 1000))
    x = np.stack([rng.uniform(0, 20000.0, n), rng.uniform(0, 10000.0, n)], axis=-1)
    return MoistBubbleRainy(seed=seed)(x, 0.0, eq)


def train_guess(n=1_000_000, epochs=20, seed=11, mode=1, tol=1e-12, batch=4096, lr=3e-3):
    """Generates n (state, T*) pairs with the Newton solve and trains the MLP on
    the offset T* - T_unsat of the saturated ones.  Returns (params, stats of
    the data generation, per-epoch losses)."""
    u = sample_states(n, seed)
    solved, st, _ = newton_solve_states(u.copy(), mode=mode, tol=tol, max_iterations=50, polish=1)
    tu, _ = t_unsat(u)
    ok = np.isfinite(solved[:, 8]) & saturated(u)
    X = features(u[ok])
    T = (solved[ok, 8] - tu[ok]).astype(np.float32)
    p = set_normalization(init_params(seed), X, T)
    p, losses = train(p, X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return p, st, losses
