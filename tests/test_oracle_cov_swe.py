"""Pins the covariant shallow-water oracle, the host mirror's cubed-sphere mesh
and metric terms (26 auxiliary variables, Christoffel symbols by dual-number
differentiation or by the collocation derivative) and the test-case initial
conditions against the reference's golden vectors (CPU only).

test/test_2d_shallow_water_covariant.jl, each elixir from
examples/shallow_water/covariant/ on P4estMeshCubedSphere2D(5, EARTH_RADIUS;
polydeg 3, element_local_mapping = true) run to t = 1 day with CK2N54:
  * elixir_geostrophic_balance (:7-26): weak form, flux_lax_friedrichs,
    spherical global coordinates, CFL 0.4;
  * elixir_unsteady_solid_body_rotation_EC with the test's overrides (:66-88):
    split form, volume (flux_central, flux_nonconservative_ec), surface
    (flux_lax_friedrichs, flux_nonconservative_ec), bottom topography;
  * elixir_rossby_haurwitz (:28-40): split, (flux_ec, flux_nonconservative_ec),
    surface (flux_ec + LLF, flux_nonconservative_surface_simplified),
    collocation-derivative Christoffel symbols;
  * elixir_isolated_mountain (:42-54): as Rossby-Haurwitz, dual-number
    Christoffel symbols, bottom topography;
  * elixir_well_balanced (:90-101): l2 = linf = 0 at atol 1e-11, CFL 0.1;
  * elixir_barotropic_instability (:78-89): Galewsky et al.'s jet, as
    Rossby-Haurwitz but with dual-number Christoffel symbols; its height
    integral by composite Gauss-Legendre quadrature instead of QuadGK.
Time stepping: the elixirs pass SaveSolutionCallback(dt = (tspan[2] - tspan[1]) /
n_saves) with n_saves = 10, a PeriodicCallback that adds a tstop every tenth of
tspan; the step that would pass a tstop is shortened to land on it (as at
t_end).  With those ten stops every case reproduces its golden to 1e-11 relative
or better; stepping straight to t_end instead moves the time-dependent cases by
up to 6e-8.
Tolerance: Trixi's @test_trixi_include defaults (atol 500 eps, rtol sqrt(eps)),
and for the oracle also 1e-9 relative on every norm above 1e-9.
"""
import math

import numpy as np
import pytest

ATOL = 500 * np.finfo(np.float64).eps
RTOL = math.sqrt(np.finfo(np.float64).eps)
N_SAVES = 10  # the elixirs' SaveSolutionCallback(dt = tspan / n_saves)
ORACLE_RTOL = 1e-9

GOLDEN = {
    "geostrophic_balance": ([0.2782318946518096, 0.00021164119121947804, 8.588414721470694e-5],
                            [1.818810315677183, 0.0011402373824409423, 0.0010284231183849968]),
    "unsteady_solid_body_rotation": ([0.25500246412246835, 0.0002703652960705074,
                                      0.0001650991084937778],
                                     [2.11951898785469, 0.0013109661149978136,
                                      0.001328788247668855]),
    "rossby_haurwitz": ([265.9818260977567, 0.17644364627357362, 0.2535621726719579],
                        [574.6725801771354, 0.5155385127558593, 0.5497040481041348]),
    "isolated_mountain": ([13.18894432799001, 0.005698447961168719, 0.007624217062402512],
                          [116.645494528163, 0.052086295524203324, 0.07855675891709994]),
    "well_balanced": ([0.0, 0.0, 0.0], [0.0, 0.0, 0.0]),
    "barotropic_instability": ([21.08826693663232, 0.03006187671520436, 0.023421745045307123],
                               [122.9994523425994, 0.17997299389835533, 0.16659612583251238]),
}


def case(tg, name):
    """(equations, initial condition, oracle flux ids, CFL, metric terms,
    bottom topography) of one elixir."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_ROTATION_RATE as OM)
    split = cv.SplitCovariantShallowWaterEquations2D(G, OM, cv.GlobalCartesianCoordinates())
    ec = dict(volume=1, vol_sym=1, vol_nc=1, surf_sym=1, surf_diss=1, surf_nc=2)
    if name == "geostrophic_balance":
        eq = cv.CovariantShallowWaterEquations2D(G, OM, cv.GlobalSphericalCoordinates())
        return (eq, cv.initial_condition_geostrophic_balance, dict(volume=0, surf_sym=0, surf_diss=1),
                0.4, None, None)
    if name == "unsteady_solid_body_rotation":
        return (split, cv.initial_condition_unsteady_solid_body_rotation,
                dict(volume=1, vol_sym=0, vol_nc=1, surf_sym=0, surf_diss=1, surf_nc=1), 0.4, None,
                cv.bottom_topography_unsteady_solid_body_rotation)
    if name == "rossby_haurwitz":
        return (split, cv.initial_condition_rossby_haurwitz, ec, 0.4,
                cv.MetricTermsCovariantSphere(cv.ChristoffelSymbolsCollocationDerivative()), None)
    if name == "isolated_mountain":
        return (split, cv.initial_condition_isolated_mountain, ec, 0.4, None,
                cv.bottom_topography_isolated_mountain)
    if name == "barotropic_instability":
        return (split, cv.initial_condition_barotropic_instability, ec, 0.4, None, None)
    return (split, cv.initial_condition_well_balanced(), dict(ec, surf_nc=1), 0.1, None,
            cv.bottom_topography_isolated_mountain)


def setup(tg, name, k=5, polydeg=3):
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    eq, ic, fluxes, cfl, metric, topo = case(tg, name)
    mesh = cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=polydeg)
    basis = tg.LobattoLegendreBasis(polydeg)
    aux, xyz = cv.compute_aux_vars(mesh, basis, eq, metric, topo)
    conn = mesh.connectivity(basis)
    icT = cv.transform_initial_condition(ic, eq)
    return eq, mesh, basis, aux, xyz, conn, icT, fluxes, cfl


def check_golden(name, l2, linf, rtol=RTOL):
    g2, gi = GOLDEN[name]
    atol = 1e-11 if name == "well_balanced" else ATOL
    for v in range(3):
        assert abs(l2[v] - g2[v]) <= max(atol, rtol * max(abs(l2[v]), abs(g2[v]))), ("l2", v, l2[v], g2[v])
        assert abs(linf[v] - gi[v]) <= max(atol, rtol * max(abs(linf[v]), abs(gi[v]))), ("linf", v, linf[v], gi[v])


def save_stops(t_end, n_saves=N_SAVES):
    """The tstops of SaveSolutionCallback(dt = t_end / n_saves) from t = 0,
    ending with t_end."""
    return [t_end * k / n_saves for k in range(1, n_saves)] + [t_end]


@pytest.mark.parametrize("name", list(GOLDEN))
def test_oracle_covariant_golden(tg, orc, name):
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_ROTATION_RATE as OM)
    eq, mesh, basis, aux, xyz, conn, icT, fluxes, cfl = setup(tg, name)
    ie, ifc, fl, _, _ = conn.arrays()
    u = np.ascontiguousarray(icT(xyz, 0.0, aux))
    c = orc.CovSWE(3, aux, xyz, ie, ifc, fl, G, OM, eq.split, fluxes)
    t_end = 1.0 * cv.SECONDS_PER_DAY
    k, t = np.zeros_like(u), 0.0
    for stop in save_stops(t_end):
        t = c.ck_steps(u, k, t, cfl, 10 ** 7, 0.0, stop)
        assert t == stop
    l2, linf = cv.error_norms(u, icT(xyz, t, aux), aux, basis)
    check_golden(name, l2, linf)
    if name != "well_balanced":
        check_golden(name, l2, linf, ORACLE_RTOL)


def test_cubed_sphere_mesh_and_metric(tg):
    """Every edge matched once; nodes on the sphere; the contravariant basis is
    the dual of the covariant one; the area elements integrate to 4 pi a^2
    (to the mapping's interpolation error); Christoffel symbols by dual
    numbers and by the collocation derivative agree to the discretisation
    error."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    eq = cv.CovariantShallowWaterEquations2D(9.80616, 7.292e-5)
    for k, N in ((3, 3), (4, 5)):
        mesh = cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=N)
        basis = tg.LobattoLegendreBasis(N)
        conn = mesh.connectivity(basis)
        ie, ifc, fl, _, _ = conn.arrays()
        assert ie.shape[0] == 2 * mesh.nelements
        aux, xyz = cv.compute_aux_vars(mesh, basis, eq)
        assert np.allclose(np.sqrt((xyz ** 2).sum(-1)), EARTH_RADIUS, rtol=1e-14)
        A = aux[..., 0:6].reshape(aux.shape[:-1] + (2, 3)).swapaxes(-1, -2)
        Ac = aux[..., 6:12].reshape(aux.shape[:-1] + (3, 2)).swapaxes(-1, -2)
        assert np.allclose(np.einsum("...ik,...kj->...ij", Ac, A), np.eye(2), atol=1e-12)
        area = (basis.weights[None, :, None] * basis.weights[None, None, :] * aux[..., 12]).sum()
        assert abs(area / (4 * np.pi * EARTH_RADIUS ** 2) - 1) < 1e-3
        aux_c, _ = cv.compute_aux_vars(
            mesh, basis, eq, cv.MetricTermsCovariantSphere(cv.ChristoffelSymbolsCollocationDerivative()))
        scale = np.abs(aux[..., 20:26]).max()
        assert np.abs(aux_c[..., 20:26] - aux[..., 20:26]).max() < 0.05 * scale


def test_galewsky_height_is_in_gradient_wind_balance(tg):
    """The Galewsky height (reference_data.jl:427-474) solves
    dh/dlat = -(a/g) u (2 Omega sin + u tan / a) with h = 10158 m at the pole:
    checked by a sixth-order central difference of the quadrature, away from
    the perturbation (which lives near lon = 0)."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_RADIUS as A, EARTH_ROTATION_RATE as OM)
    eq = cv.SplitCovariantShallowWaterEquations2D(G, OM, cv.GlobalSphericalCoordinates())
    lat = np.linspace(0.3, 1.3, 41)
    lon = np.pi - 0.01

    def height(la):
        x = A * np.stack([np.cos(la) * np.cos(lon), np.cos(la) * np.sin(lon), np.sin(la)], -1)
        return cv.initial_condition_barotropic_instability(x, 0.0, eq)[..., 0]

    d = 1e-3
    c = np.array([-1, 9, -45, 0, 45, -9, 1]) / 60.0
    dh = sum(ck * height(lat + (k - 3) * d) for k, ck in enumerate(c)) / d
    u = cv.galewsky_velocity(lat)
    rhs = -(A / G) * u * (2 * OM * np.sin(lat) + u * np.tan(lat) / A)
    assert np.abs(dh - rhs).max() <= 1e-6 * np.abs(rhs).max()
    assert abs(height(np.array([np.pi / 2 - 1e-9]))[0] - 10158.0) < 1e-9
    assert np.all(u[(lat <= np.pi / 7) | (lat >= np.pi / 2 - np.pi / 7)] == 0)
