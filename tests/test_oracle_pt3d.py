"""The oracle's 3D potential-temperature equations with gravity
(oracle/orc_pt_3d.hpp), checked on the CPU.

The reference has no per-call golden for them (its 3D goldens run adaptive
SSPRK43 time steps), so the restatement is pinned through:
- the reference's own consistency checks (test/test_unit.jl:282-300, 346-362,
  410-424, 468-484): flux_tec / flux_ec / flux_etec / FluxLMARS of equal
  states equal the physical flux, at the states and normals used there;
- the 2D/3D relation the same tests check: with v3 = 0 and a normal without a
  z component the 3D two-point fluxes, nonconservative gravity terms and LMARS
  equal the 2D ones (components rho, rho_v1, rho_v2, rho_theta), and the 2D
  oracle is pinned to the reference's 2D gravity-wave golden;
- the DG discretisation on the cubed-sphere shell conserves total mass.
"""
import numpy as np
import pytest

NORMALS = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (0.5, -0.5, 0.2), (-1.2, 0.3, 1.4)]
RTOL = 1.4901161193847656e-08  # Julia's isapprox default, sqrt(eps)


@pytest.mark.parametrize("volume", [0, 1, 2])
def test_volume_fluxes_consistent(orc, volume):
    u = np.array([1.1, -0.5, 2.34, 2.4, 330.0, 1500.0])
    for n in NORMALS:
        f = orc.pt_pointwise(3, 0, u, u, n)
        fv = orc.pt_pointwise(3, 1, u, u, n, volume=volume)
        assert np.allclose(fv, f, rtol=RTOL, atol=0.0), (n, fv, f)


def test_lmars_consistent(orc):
    u = np.array([1.1, -0.5, 2.34, 2.4, 330.0, 1700.0])
    for n in NORMALS:
        f = orc.pt_pointwise(3, 0, u, u, n)
        fl = orc.pt_pointwise(3, 3, u, u, n, c=340.0)
        assert np.allclose(fl, f, rtol=RTOL, atol=1e-12 * np.abs(f).max()), (n, fl, f)


@pytest.mark.parametrize("kind,volume,nc", [(1, 0, 0), (1, 1, 0), (1, 2, 0), (2, 0, 0), (2, 0, 1),
                                            (2, 0, 2), (3, 0, 0)])
def test_3d_reduces_to_2d(orc, kind, volume, nc):
    rng = np.random.default_rng(kind * 10 + volume + nc)
    for _ in range(20):
        a2 = np.array([rng.uniform(0.5, 1.5), rng.uniform(-20, 20), rng.uniform(-20, 20),
                       rng.uniform(250, 350), rng.uniform(0, 1e5)])
        b2 = a2 * (1 + rng.uniform(-0.2, 0.2, 5))
        n2 = rng.uniform(-1, 1, 2)
        a3 = np.array([a2[0], a2[1], a2[2], 0.0, a2[3], a2[4]])
        b3 = np.array([b2[0], b2[1], b2[2], 0.0, b2[3], b2[4]])
        n3 = np.array([n2[0], n2[1], 0.0])
        f2 = orc.pt_pointwise(2, kind, a2, b2, n2, volume=volume, nc=nc)
        f3 = orc.pt_pointwise(3, kind, a3, b3, n3, volume=volume, nc=nc)
        scale = np.abs(f2).max()
        assert np.abs(f3[[0, 1, 2, 4]] - f2[[0, 1, 2, 3]]).max() <= 1e-14 * scale
        assert abs(f3[3]) <= 1e-14 * scale


def pt3d_shell(tg, orc, trees=3, layers=2, polydeg=3, volume=0, nc=0):
    from test_oracle_golden_3d import oracle_3d  # noqa: F401  (path set by the orc fixture)
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, tg.EARTH_RADIUS, 30000.0,
                                             polydeg=polydeg)
    basis = tg.LobattoLegendreBasis(polydeg)
    xyz, Ja, invJ = mesh.geometry(basis)
    conn = mesh.connectivity(basis)
    o = orc.PotTemp3D(polydeg, Ja, invJ, xyz, *conn.arrays(), c_p=1004.0, c_v=717.0,
                      g=tg.EARTH_GRAVITATIONAL_ACCELERATION, c_lmars=340.0,
                      omega=tg.EARTH_ROTATION_RATE, volume=volume, nc=nc)
    return eq, mesh, basis, xyz, Ja, invJ, conn, o


def perturb_pt3d(u, seed, amplitude=1e-2, velocity=5.0):
    rng = np.random.Generator(np.random.Philox(seed))
    v = u.copy()
    v[..., 0] *= 1 + amplitude * rng.uniform(-1, 1, v.shape[:-1])
    for k in (1, 2, 3):
        v[..., k] += velocity * v[..., 0] * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 4] *= 1 + amplitude * rng.uniform(-1, 1, v.shape[:-1])
    return v


@pytest.mark.parametrize("volume,nc", [(0, 2), (1, 0), (2, 1)])
def test_shell_conserves_mass(tg, orc, volume, nc):
    eq, mesh, basis, xyz, Ja, invJ, conn, o = pt3d_shell(tg, orc, volume=volume, nc=nc)
    u = perturb_pt3d(tg.initial_condition_baroclinic_instability(xyz, 0.0, eq), seed=4)
    du = o.rhs(u)
    w = basis.weights
    W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    mass = np.sum(W / invJ * du[..., 0])
    assert abs(mass) <= 1e-13 * np.sum(W / invJ * np.abs(du[..., 0]))
    assert np.all(du[..., 5] == 0)
