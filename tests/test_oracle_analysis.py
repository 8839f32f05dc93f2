"""The oracle's analysis restatements (oracle/analysis.py) checked on the CPU,
and the library's host-only LGL basis (tag_lgl_basis):

- tag_lgl_basis against the host mirror's LobattoLegendreBasis nodes/weights;
- cons2entropy is the gradient of entropy where the reference defines the two
  as a pair (energy equations 2D/3D: entropy_math; covariant shallow water:
  the total energy), by central differences;
- with the entropy-conservative covariant split form (flux_ec volume and
  surface flux, nonconservative flux_ec, no dissipation) the oracle's rhs
  conserves the total energy: the entropy time derivative
  sum wJ cons2entropy(u) . du vanishes to rounding."""
import ctypes

import numpy as np
import pytest


@pytest.fixture
def analysis(orc):
    import analysis as a  # oracle/analysis.py, on the path once the oracle is loaded
    return a


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("polydeg", [1, 2, 3, 5, 7, 10, 14])
def test_lgl_basis_matches_host_mirror(tg, polydeg):
    x, w = np.zeros(polydeg + 1), np.zeros(polydeg + 1)
    assert tg._lib.load().tag_lgl_basis(polydeg, _dp(x), _dp(w)) == 0
    b = tg.LobattoLegendreBasis(polydeg)
    assert np.abs(x - np.asarray(b.nodes)).max() <= 4e-16
    assert np.abs(w - np.asarray(b.weights)).max() <= 4e-16 * max(1.0, np.abs(w).max())
    assert abs(w.sum() - 2.0) <= 1e-14


def _grad(f, u, h=1e-6):
    g = np.zeros_like(u)
    for v in range(u.shape[-1]):
        du = np.zeros_like(u)
        du[..., v] = h * np.maximum(np.abs(u[..., v]), 1.0)
        g[..., v] = (f(u + du) - f(u - du)) / (2 * du[..., v])
    return g


@pytest.mark.parametrize("nd", [2, 3])
def test_energy_cons2entropy_is_entropy_gradient(analysis, nd):
    rng = np.random.default_rng(nd)
    gamma = 1004.0 / 717.0
    rho = rng.uniform(0.5, 1.5, 20)
    v = rng.uniform(-30, 30, (20, nd))
    p = rng.uniform(5e4, 1e5, 20)
    u = np.zeros((20, nd + 3))
    u[:, 0] = rho
    u[:, 1:nd + 1] = rho[:, None] * v
    u[:, nd + 1] = p / (gamma - 1) + 0.5 * rho * (v ** 2).sum(1)
    u[:, nd + 2] = 9.81 * rng.uniform(0, 1e4, 20)
    w = analysis.energy_cons2entropy(u, gamma)
    g = _grad(lambda x: analysis.energy_entropy(x, gamma), u)
    assert np.abs(w[:, :nd + 2] - g[:, :nd + 2]).max() <= 1e-5 * np.abs(w).max()
    assert np.all(w[:, nd + 2] == 0)


def _cov(tg, fluxes, k=3, polydeg=3):
    from test_oracle_cov_swe import setup
    eq, mesh, basis, aux, xyz, conn, icT, _, _ = setup(tg, "isolated_mountain", k, polydeg)
    u = np.ascontiguousarray(icT(xyz, 0.0, aux))
    rng = np.random.default_rng(1)
    u[..., 0] *= 1 + 1e-2 * rng.uniform(-1, 1, u.shape[:-1])
    u[..., 1:] += 1e-2 * np.abs(u[..., 1:]).max() * rng.uniform(-1, 1, u.shape[:-1] + (2,))
    return eq, basis, aux, xyz, conn, u


def test_covariant_cons2entropy_is_entropy_gradient(tg, analysis):
    eq, basis, aux, xyz, conn, u = _cov(tg, None)
    g = eq.gravity if hasattr(eq, "gravity") else 9.80616
    w = analysis.cov_cons2entropy(u, aux, g)
    gr = _grad(lambda x: analysis.cov_entropy(x, aux, g), u)
    assert np.abs(w - gr).max() <= 1e-5 * np.abs(w).max()


def test_covariant_ec_split_form_conserves_entropy(tg, orc, analysis):
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_ROTATION_RATE as OM)
    ec = dict(volume=1, vol_sym=1, vol_nc=1, surf_sym=1, surf_diss=0, surf_nc=1)
    eq, basis, aux, xyz, conn, u = _cov(tg, ec)
    ie, ifc, fl, _, _ = conn.arrays()
    c = orc.CovSWE(3, aux, xyz, ie, ifc, fl, G, OM, eq.split, ec)
    du = c.rhs(u)
    wJ = analysis.quadrature_weights(basis.weights, 2, aux=aux)
    wdu = (analysis.cov_cons2entropy(u, aux, G) * du).sum(-1)
    dsdt = analysis.integrate(wdu, wJ, normalize=False)
    scale = analysis.integrate(np.abs(wdu), wJ, normalize=False)
    assert abs(dsdt) <= 1e-11 * scale, dsdt / scale
    # with dissipation the same state loses entropy
    c2 = orc.CovSWE(3, aux, xyz, ie, ifc, fl, G, OM, eq.split, dict(ec, surf_diss=1))
    du2 = c2.rhs(u)
    wdu2 = (analysis.cov_cons2entropy(u, aux, G) * du2).sum(-1)
    assert analysis.integrate(wdu2, wJ, normalize=False) < -1e-6 * scale
