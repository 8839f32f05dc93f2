"""Pins the 3D oracle, the host mirror's cubed-sphere shell geometry, the
baroclinic-instability initial state and the error analysis against the
reference's golden vector (CPU only).

test/test_3d_euler_energy.jl:7-29 runs
examples/euler/dry_air/global_circulation/elixir_energy_baroclinic_instability.jl
(P4estMeshCubedSphereTopography(8, 4, EARTH_RADIUS, 30000; polydeg = 5),
(flux_ranocha, flux_nonconservative_waruszewski_etal) / (FluxLMARS(340), flux_zero),
slip walls inside/outside, source_terms_coriolis) to t = 0.01 s with an
adaptive SSPRK43 at tol = 1e-15, and compares l2/linf with atol = 1e-8.
At that tolerance the time integration is exact to rounding, so ten
CarpenterKennedy2N54 steps of 1 ms stand in for it.
"""
import math

import numpy as np
import pytest

GOLDEN_L2 = [6.540827547514395e-7, 0.0001972937313811121, 0.00042458497371703434,
             0.00018720446122477726, 0.06698234918918748, 0.0408936452021324]
GOLDEN_LINF = [4.42523425103758e-6, 0.024276205576123866, 0.04570236938186356,
               0.022711920085996914, 0.9490993925137445, 0.3118668645620346]
ATOL = 1e-8
RTOL = math.sqrt(np.finfo(np.float64).eps)
# phi = -a^2 g / |x| ~ -6.2e7 never changes; its linf is the interpolation error
# of phi itself, reproducible only to a few ulp of |phi| (7.5e-9 each) across
# implementations of the cubed-sphere map, so it is checked to 1e-15 |phi|.
PHI_ULP_TOL = 1e-15 * 6.37122e6 ** 2 * 9.80616 / 6.37122e6


def isapprox(a, b):
    return abs(a - b) <= max(ATOL, RTOL * max(abs(a), abs(b)))


def shell_case(tg, trees=8, layers=4, polydeg=5):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, tg.EARTH_RADIUS, 30000.0,
                                             polydeg=polydeg)
    basis = tg.LobattoLegendreBasis(polydeg)
    xyz, Ja, invJ = mesh.geometry(basis)
    conn = mesh.connectivity(basis)
    return eq, mesh, basis, xyz, Ja, invJ, conn


def oracle_3d(orc, tg, polydeg, Ja, invJ, xyz, conn, omega=None):
    return orc.Euler3D(polydeg, Ja, invJ, xyz, *conn.arrays(), c_p=1004.0, c_v=717.0,
                       g=tg.EARTH_GRAVITATIONAL_ACCELERATION, c_lmars=340.0,
                       omega=tg.EARTH_ROTATION_RATE if omega is None else omega)


def check_golden(l2, linf):
    for v in range(6):
        assert isapprox(l2[v], GOLDEN_L2[v]), (v, l2[v], GOLDEN_L2[v])
        if v == 5:
            assert abs(linf[v] - GOLDEN_LINF[v]) <= 4 * PHI_ULP_TOL, (linf[v], GOLDEN_LINF[v])
        else:
            assert isapprox(linf[v], GOLDEN_LINF[v]), (v, linf[v], GOLDEN_LINF[v])


def test_oracle_baroclinic_instability_golden(tg, orc):
    import analysis
    eq, mesh, basis, xyz, Ja, invJ, conn = shell_case(tg)
    u = tg.initial_condition_baroclinic_instability(xyz, 0.0, eq)
    o = oracle_3d(orc, tg, 5, Ja, invJ, xyz, conn)
    t = o.ck_steps(u, np.zeros_like(u), 0.0, 1.0, 10, 0.001)
    assert abs(t - 0.01) < 1e-15
    l2, linf = analysis.error_norms(
        u, xyz, invJ, basis.nodes,
        lambda x: tg.initial_condition_baroclinic_instability(x, 0.0, eq), 3)
    check_golden(l2, linf)


def test_shell_mesh_connectivity_and_metric_identities(tg):
    eq, mesh, basis, xyz, Ja, invJ, conn = shell_case(tg, trees=3, layers=2, polydeg=3)
    E = mesh.nelements
    ie, ifc, io, be, bf = conn.arrays()
    assert E == 6 * 9 * 2
    assert len(be) == 2 * 6 * 9 and set(conn.bd_names) == {"inside", "outside"}
    assert len(io) == (6 * E - len(be)) // 2
    assert set(np.unique(io)) <= set(range(8)) and np.any(io != 0)  # panel edges are rotated
    assert np.all(invJ > 0)
    D = basis.derivative_matrix
    div = (np.einsum("ia,ekja...->ekji...", D, Ja[..., 0, :]) +
           np.einsum("ja,ekai...->ekji...", D, Ja[..., 1, :]) +
           np.einsum("ka,eaji...->ekji...", D, Ja[..., 2, :]))
    assert np.abs(div).max() <= 1e-13 * np.abs(Ja).max()


def test_shell_oracle_conserves_mass(tg, orc):
    """A smooth state on the shell: the total mass tendency vanishes, which
    holds only if every interface pairs the right face nodes."""
    eq, mesh, basis, xyz, Ja, invJ, conn = shell_case(tg, trees=3, layers=2, polydeg=3)
    u = tg.initial_condition_baroclinic_instability(xyz, 0.0, eq)
    u = perturb3d(u, eq, seed=4)
    du = oracle_3d(orc, tg, 3, Ja, invJ, xyz, conn).rhs(u)
    w = basis.weights
    W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    mass = np.sum(W / invJ * du[..., 0])
    assert abs(mass) <= 1e-13 * np.sum(W / invJ * np.abs(du[..., 0]))


def perturb3d(u, eq, seed, amplitude=1e-2, velocity=5.0):
    rng = np.random.Generator(np.random.Philox(seed))
    rho, v1, v2, v3, p, phi = eq.cons2prim(u)
    s = u.shape[:-1]
    return eq.prim2cons(rho * (1 + amplitude * rng.uniform(-1, 1, s)),
                        v1 + velocity * rng.uniform(-1, 1, s), v2 + velocity * rng.uniform(-1, 1, s),
                        v3 + velocity * rng.uniform(-1, 1, s),
                        p * (1 + amplitude * rng.uniform(-1, 1, s)), phi)


@pytest.mark.parametrize("vertical", ["galchen", "sleve"])
def test_shell_mesh_with_topography(tg, vertical):
    """P4estMeshCubedSphereTopography with an initial topography
    (src/meshes/p4est_cubed_sphere_topography.jl:596-620) and GalChen or
    Sleve(0.7, 0.8) vertical coordinates: the ground follows the topography,
    the top stays at inner_radius + thickness, interfaces still match node
    for node and the curl-form metric terms keep the discrete metric
    identities; zero topography gives the perfect sphere's nodes exactly."""
    from trixiatmo_gb300.meshes3d import GalChen, Sleve
    a, H = 6.371e6, 30000.0

    def mountain(lat, lon):
        return 2000.0 * np.exp(-((lat - 0.4) ** 2 + (lon - 0.3) ** 2) / 0.05)

    adapt = GalChen() if vertical == "galchen" else Sleve(0.7, 0.8)
    basis = tg.LobattoLegendreBasis(3)
    flat = tg.P4estMeshCubedSphereTopography(3, 2, a, H, polydeg=3)
    zero = tg.P4estMeshCubedSphereTopography(3, 2, a, H, polydeg=3,
                                             initial_topography=lambda lat, lon: 0.0 * lat,
                                             adapt_vertical_grid=adapt)
    x0, x1 = flat.geometry(basis)[0], zero.geometry(basis)[0]
    if vertical == "galchen":
        assert np.array_equal(x0, x1)
    else:  # eta H = (z_ref / H) H: the last bit of z_ref
        assert np.abs(x0 - x1).max() <= 1e-8
    mesh = tg.P4estMeshCubedSphereTopography(3, 2, a, H, polydeg=3, initial_topography=mountain,
                                             adapt_vertical_grid=adapt)
    xyz, Ja, invJ = mesh.geometry(basis)
    r = np.sqrt((xyz ** 2).sum(-1))
    top = r[:, -1][np.arange(mesh.nelements) % 2 == 1]   # layer 1, k = n - 1
    assert np.allclose(top, a + H, rtol=0, atol=1e-7)
    ground = r[:, 0][np.arange(mesh.nelements) % 2 == 0]  # layer 0, k = 0
    assert ground.max() - a > 1500.0 and ground.min() >= a - 1e-7
    # the reference's latitude: asin of the unit vector's z divided by the cube
    # point's radius 1 / max|unit_i|
    p = xyz[:, 0][np.arange(mesh.nelements) % 2 == 0]
    unit = p / np.sqrt((p ** 2).sum(-1))[..., None]
    lat_ref = np.arcsin(unit[..., 2] * np.abs(unit).max(-1))
    lon = np.arctan2(unit[..., 1], unit[..., 0])
    assert np.allclose(ground, a + mountain(lat_ref, lon), rtol=0, atol=1e-6)
    assert np.all(invJ > 0)
    conn = mesh.connectivity(basis)
    ie, ifc, io, be, bf = conn.arrays()
    assert len(be) == 2 * 6 * 9 and len(io) == (6 * mesh.nelements - len(be)) // 2
    D = basis.derivative_matrix
    div = (np.einsum("ia,ekja...->ekji...", D, Ja[..., 0, :]) +
           np.einsum("ja,ekai...->ekji...", D, Ja[..., 1, :]) +
           np.einsum("ka,eaji...->ekji...", D, Ja[..., 2, :]))
    assert np.abs(div).max() <= 1e-13 * np.abs(Ja).max()
