"""Known-answer checks of the oracle's output conversions
(oracle/solution_variables.py), before they serve as the checker of the
device's: the nodal derivative matrix is exact on polynomials of the
degree; for Williamson case 2 (solid-body zonal flow u = u0 cos(lat),
src/equations/reference_data.jl:145-164) the relative vorticity of
cons2prim_and_vorticity converges to 2 u0 sin(lat) / a with the mesh, and
contravariant2global / cons2prim return the initial condition's global
velocity and total height."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def sv(orc):
    import solution_variables
    return solution_variables


def zonal_flow(tg, k, N):
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_RADIUS, EARTH_ROTATION_RATE as OM)
    eq = cv.CovariantShallowWaterEquations2D(G, OM, cv.GlobalCartesianCoordinates())
    mesh = cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=N)
    basis = tg.LobattoLegendreBasis(N)
    aux, xyz = cv.compute_aux_vars(mesh, basis, eq)
    u = cv.transform_initial_condition(cv.initial_condition_geostrophic_balance, eq)(xyz, 0.0, aux)
    prim = cv.initial_condition_geostrophic_balance(xyz, 0.0, eq)
    lat = np.arcsin(xyz[..., 2] / np.linalg.norm(xyz, axis=-1)).reshape(-1)
    u0 = 2 * np.pi * EARTH_RADIUS / (12 * 86400.0)
    return u, aux, basis, prim, 2 * u0 * np.sin(lat) / EARTH_RADIUS


@pytest.mark.parametrize("N", [1, 3, 5, 7])
def test_derivative_matrix_exact_on_polynomials(tg, sv, N):
    x = np.asarray(tg.LobattoLegendreBasis(N).nodes)
    D = sv.derivative_matrix(x)
    for q in range(N + 1):
        d = q * x ** (q - 1) if q else np.zeros_like(x)
        assert np.abs(D @ x ** q - d).max() <= 1e-14 * max(1, N * N)


def test_vorticity_of_solid_body_rotation(tg, sv):
    errs = {}
    for k in (4, 6):
        u, aux, basis, prim, zeta = zonal_flow(tg, k, 7)
        rows = sv.covariant_rows(u, aux, basis.nodes, 3)
        errs[k] = np.abs(rows[5] - zeta).max() / np.abs(zeta).max()
        # H, the global velocity and b
        assert np.abs(rows[0] - prim[..., 0].ravel()).max() <= 1e-12 * np.abs(prim[..., 0]).max()
        vg = prim[..., 1:4].reshape(-1, 3).T
        assert np.abs(rows[1:4] - vg).max() <= 1e-14 * np.abs(vg).max()
        assert np.all(rows[4] == 0.0)
    assert errs[4] < 3e-6 and errs[6] < errs[4] / 10, errs


def test_conversions_consistent(tg, sv):
    u, aux, basis, prim, _ = zonal_flow(tg, 3, 4)
    r0, r1, r2 = (sv.covariant_rows(u, aux, basis.nodes, k) for k in range(3))
    assert np.array_equal(r0, u.reshape(-1, 3).T)
    assert np.array_equal(r1[0], r0[0] + aux[..., 19].ravel())
    assert np.allclose(r1[1:] * r0[0], r0[1:], rtol=1e-15, atol=0)
    vg = prim[..., 1:4].reshape(-1, 3).T
    assert np.abs(r2[1:] / r0[0] - vg).max() <= 1e-14 * np.abs(vg).max()
