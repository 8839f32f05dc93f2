"""ORACLE — test infrastructure only.

End-of-run error norms computed the way Trixi's AnalysisCallback reports
`l2` / `linf` (the quantities the reference's tests pin, e.g.
test/test_2d_euler_energy.jl:10-23): solution, node coordinates and the
Jacobian J = 1/inverse_jacobian are interpolated from the LGL nodes of degree
N to the LGL nodes of degree 2N (the default analysis polydeg); the exact
solution is evaluated there;
    l2   = sqrt( sum w_i w_j (w_k) J |u_exact - u|^2 / sum w_i w_j (w_k) J ),
    linf = max |u_exact - u|,
per variable.
"""
from __future__ import annotations

import numpy as np


def _lgl(N):
    import importlib
    import sys
    b = sys.modules.get("trixiatmo_gb300.basis") or importlib.import_module("trixiatmo_gb300.basis")
    return b


def error_norms(u, xyz, inv_jacobian, nodes, exact, ndims):
    """u[e, (k,) j, i, v], xyz[e, (k,) j, i, c], inv_jacobian[e, (k,) j, i];
    exact(x) -> u_exact[..., v]."""
    b = _lgl(None)
    N = len(nodes) - 1
    xa, wa = b.lgl_nodes_weights(2 * N)
    V = b.interpolation_matrix(np.asarray(nodes), xa)
    J = 1.0 / inv_jacobian
    if ndims == 2:
        def interp(f):
            return np.einsum("ai,bj,eji...->eba...", V, V, f, optimize=True)
        W = wa[:, None] * wa[None, :]
    else:
        def interp(f):
            return np.einsum("ai,bj,ck,ekji...->ecba...", V, V, V, f, optimize=True)
        W = wa[:, None, None] * wa[None, :, None] * wa[None, None, :]
    ua = interp(u)
    xa_ = interp(xyz)
    Ja = interp(J)
    diff = exact(xa_) - ua
    wJ = W[None] * Ja
    vol = wJ.sum()
    nv = u.shape[-1]
    l2 = np.sqrt((wJ[..., None] * diff * diff).reshape(-1, nv).sum(axis=0) / vol)
    linf = np.abs(diff).reshape(-1, u.shape[-1]).max(axis=0)
    return l2, linf


# ---- integrals (Trixi's integrate / entropy_timederivative) ----------------
# Quadrature on the solution nodes: w_i w_j (w_k) |J| per node, with
# J = 1 / inverse_jacobian on Cartesian meshes and the area element of the
# auxiliary variables (slot 12) for covariant equations
# (src/callbacks_step/analysis_covariant.jl:53-85).

def quadrature_weights(weights, ndims, inv_jacobian=None, aux=None):
    w = np.asarray(weights)
    if ndims == 2:
        W = w[None, :] * w[:, None]            # [j, i]
    else:
        W = w[:, None, None] * w[None, :, None] * w[None, None, :]
    if aux is not None:
        return W[None] * aux[..., 12]
    return W[None] * np.abs(1.0 / inv_jacobian)


def integrate(values, wJ, normalize=True):
    """sum wJ * values over the nodes (values [..., q] or [...])."""
    v = np.asarray(values)
    if v.ndim == wJ.ndim:
        s = (wJ * v).sum()
    else:
        s = (wJ[..., None] * v).reshape(-1, v.shape[-1]).sum(axis=0)
    return s / wJ.sum() if normalize else s


# Pointwise entropy, energy_total and cons2entropy of each equation system.

def energy_entropy(u, gamma):
    """entropy_math (compressible_euler_energy_with_gravity_{2d,3d}.jl); u[..., :nv]."""
    nd = u.shape[-1] - 3                      # velocity components
    e = u[..., nd + 1]
    ke = 0.5 * sum(u[..., 1 + d] ** 2 for d in range(nd)) / u[..., 0]
    p = (gamma - 1.0) * (e - ke)
    s = np.log(p) - gamma * np.log(u[..., 0])
    return -s * u[..., 0] / (gamma - 1.0)


def energy_cons2entropy(u, gamma):
    """cons2entropy (:539-557 in 2D, :581-601 in 3D); zero for phi."""
    nd = u.shape[-1] - 3
    rho = u[..., 0]
    v = [u[..., 1 + d] / rho for d in range(nd)]
    vsq = sum(x * x for x in v)
    p = (gamma - 1.0) * (u[..., nd + 1] - 0.5 * rho * vsq)
    s = np.log(p) - gamma * np.log(rho)
    rho_p = rho / p
    w = np.zeros_like(u)
    w[..., 0] = (gamma - s) / (gamma - 1.0) - 0.5 * rho_p * vsq
    for d in range(nd):
        w[..., 1 + d] = rho_p * v[d]
    w[..., nd + 1] = -rho_p
    return w


def pt_constants(c_p=1004.0, c_v=717.0):
    R = c_p - c_v
    gamma = c_p / c_v
    return dict(gamma=gamma, R=R, p_0=100000.0, K=100000.0 * (R / 100000.0) ** gamma)


def pt_entropy(u, k):
    """entropy_thermodynamic (compressible_euler_potential_temperature_gravity_2d.jl:381-387)."""
    p = k["K"] * u[..., 3] ** k["gamma"]
    s = np.log(p) - k["gamma"] * np.log(u[..., 0])
    return -s * u[..., 0] / (k["gamma"] - 1.0)


def pt_energy_total(u, k):
    """energy_total (:389-397), p = p_0 (R rho_theta / p_0)^gamma."""
    p = k["p_0"] * (k["R"] * u[..., 3] / k["p_0"]) ** k["gamma"]
    return p / (k["gamma"] - 1.0) + 0.5 * (u[..., 1] ** 2 + u[..., 2] ** 2) / u[..., 0]


def pt_cons2entropy(u, k):
    """cons2entropy (:371-379)."""
    w = np.zeros_like(u)
    w[..., 0] = np.log(k["K"] * (u[..., 3] / u[..., 0]) ** k["gamma"]) - k["gamma"]
    w[..., 3] = u[..., 0] / u[..., 3] * k["gamma"]
    return w


MOIST = dict(c_pd=1004.0, c_vd=717.0, c_pv=1885.0, c_vv=1424.0, c_pl=4186.0)
MOIST.update(R_d=MOIST["c_pd"] - MOIST["c_vd"], R_v=MOIST["c_pv"] - MOIST["c_vv"])
MOIST["L_00"] = 3147620.0  # CompressibleMoistEulerEquations2D constructor (:20-31)


def moist_condition(u, k=MOIST):
    """get_current_condition (compressible_moist_euler_2d.jl:383-402): p, T."""
    rho_qd = u[..., 0] - u[..., 4] - u[..., 5]
    rho_e = u[..., 3] - 0.5 * (u[..., 1] ** 2 + u[..., 2] ** 2) / u[..., 0]
    T = (rho_e - k["L_00"] * u[..., 4]) / (rho_qd * k["c_vd"] + u[..., 4] * k["c_vv"]
                                            + u[..., 5] * k["c_pl"])
    p = (rho_qd * k["R_d"] + u[..., 4] * k["R_v"]) * T
    return p, T


def moist_entropy(u, k=MOIST):
    """-entropy_thermodynamic (:733-757), without zero-density guards as there."""
    p, T = moist_condition(u, k)
    rho_qd, rho_qv, rho_ql = u[..., 0] - u[..., 4] - u[..., 5], u[..., 4], u[..., 5]
    with np.errstate(divide="ignore", invalid="ignore"):
        s_d = k["c_vd"] * np.log(T) - k["R_d"] * np.log(rho_qd * k["R_d"])
        s_v = k["c_vv"] * np.log(T) - k["R_v"] * np.log(rho_qv * k["R_v"])
        s_l = k["c_pl"] * np.log(T)
        return -(rho_qd * s_d + rho_qv * s_v + rho_ql * s_l)


def moist_cons2entropy(u, k=MOIST):
    """cons2entropy (:513-551) with its zero-density guards."""
    p, T = moist_condition(u, k)
    v1, v2 = u[..., 1] / u[..., 0], u[..., 2] / u[..., 0]
    rho_qd, rho_qv, rho_ql = u[..., 0] - u[..., 4] - u[..., 5], u[..., 4], u[..., 5]
    with np.errstate(divide="ignore", invalid="ignore"):
        s_d = np.where(rho_qd > 0, k["c_pd"] * np.log(T) - k["R_d"] * np.log(rho_qd * k["R_d"] * T), 0.0)
        s_v = np.where(rho_qv > 0, k["c_pv"] * np.log(T) - k["R_v"] * np.log(rho_qv * k["R_v"] * T), 0.0)
        s_l = np.where(rho_ql > 0, k["c_pl"] * np.log(T), 0.0)
    g_d = (k["c_pd"] - s_d) * T
    g_v = k["L_00"] + (k["c_pv"] - s_v) * T
    g_l = (k["c_pl"] - s_l) * T
    w = np.stack([g_d - 0.5 * (v1 ** 2 + v2 ** 2), v1, v2, -np.ones_like(T), g_v - g_d,
                  g_l - g_d], axis=-1)
    return w / T[..., None]


RAINY = dict(c_vd=717.0, c_vv=1424.0, c_l=4186.0, R_d=287.0, R_v=461.0, L_ref=2500000.0)


def rainy_cons2entropy(u, k=RAINY):
    """cons2entropy (compressible_rainy_euler_2d.jl:132-172); (rho_vapour,
    rho_cloud, T) from slots 7..9, or T from the energy when the air is dry
    (cons2nonlinearsystemsol :219-260)."""
    rho = u[..., 0] + u[..., 1] + u[..., 2]
    v1, v2 = u[..., 3] / rho, u[..., 4] / rho
    dry = (u[..., 1] == 0.0) & (u[..., 2] == 0.0)
    T_dry = (u[..., 5] - 0.5 * (v1 ** 2 + v2 ** 2) * rho) / (k["c_vd"] * rho)
    T = np.where(dry, T_dry, u[..., 8])
    rv = np.where(dry, 0.0, u[..., 6])
    rv = np.where((rv < 0) & (np.abs(rv) <= 1e-15), 0.0, rv)
    lT, iT = np.log(T), 1.0 / T
    vsq = 0.5 * (v1 ** 2 + v2 ** 2) * iT
    with np.errstate(divide="ignore", invalid="ignore"):
        rv_log = np.where(rv > 0, np.log(rv), 0.0)
    w_d = k["c_vd"] * lT - k["R_d"] * np.log(u[..., 0]) + vsq - k["c_vd"] - k["R_d"]
    w_v = k["c_vv"] * lT - k["R_v"] * rv_log + vsq - k["c_vv"] - k["R_v"] - k["L_ref"] * iT
    w_l = k["c_l"] * lT + vsq - k["c_l"]
    z = np.zeros_like(T)
    return np.stack([w_d, w_v + w_l, w_l, -v1 * iT, -v2 * iT, iT, z, z, z], axis=-1)


def cov_velocities(u, aux):
    vcon = np.stack([u[..., 1] / u[..., 0], u[..., 2] / u[..., 0]], axis=-1)
    vcov = np.stack([aux[..., 13] * vcon[..., 0] + aux[..., 14] * vcon[..., 1],
                     aux[..., 14] * vcon[..., 0] + aux[..., 15] * vcon[..., 1]], axis=-1)
    return vcon, vcov


def cov_entropy(u, aux, g):
    """entropy (covariant_shallow_water.jl:155-164): the total energy."""
    vcon, vcov = cov_velocities(u, aux)
    h = u[..., 0]
    return 0.5 * (h * (vcov * vcon).sum(-1) + g * h * h) + g * h * aux[..., 19]


def cov_cons2entropy(u, aux, g):
    """cons2entropy (:128-137)."""
    vcon, vcov = cov_velocities(u, aux)
    w0 = g * (u[..., 0] + aux[..., 19]) - 0.5 * (vcov * vcon).sum(-1)
    return np.stack([w0, vcov[..., 0], vcov[..., 1]], axis=-1)
