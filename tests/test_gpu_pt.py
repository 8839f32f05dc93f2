"""GPU parity of the potential-temperature path (flux_tec / flux_ec / flux_etec
with the nonconservative gravity terms, LMARS, slip walls) against the CPU
oracle, and the reference's inertia-gravity-wave golden with every stage on the
GPU (the library's integrator is CK2N54; the golden's SSPRK43 steps are driven
from the host, each rhs evaluated by the GPU)."""
import math

import numpy as np
import pytest

from test_oracle_pt import ATOL, GOLDEN_L2, GOLDEN_LINF, RTOL

pytestmark = pytest.mark.gpu
C_LMARS = math.sqrt(1004 / 717 * 287 * 250)


def make_pt(tg, nx=8, ny=6, polydeg=3, volume="tec", nc="waruszewski", normal_walls=False):
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity2D(c_p=1004, c_v=717,
                                                                         gravity=9.80616)
    vf = {"tec": tg.flux_tec, "ec": tg.flux_ec, "etec": tg.flux_etec}[volume]
    ncf = {"waruszewski": tg.flux_nonconservative_waruszewski_etal,
           "artiano": tg.flux_nonconservative_artiano_etal,
           "souza": tg.flux_nonconservative_souza_etal}[nc]
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(C_LMARS), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing((vf, ncf)))
    if normal_walls:
        mesh = tg.P4estMesh((2, 2), polydeg=1, coordinates_min=(0.0, 0.0),
                            coordinates_max=(300000.0, 10000.0), initial_refinement_level=2,
                            periodicity=(True, False))
    else:
        mesh = tg.StructuredMesh((nx, ny), (0.0, 0.0), (300000.0, 10000.0),
                                 periodicity=(True, False))
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.initial_condition_gravity_waves, solver,
                                           boundary_conditions=bcs)
    return eq, mesh, semi


def perturbed(u, seed):
    rng = np.random.Generator(np.random.Philox(seed))
    v = u.copy()
    v[..., 0] *= 1 + 1e-2 * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 1] += 5.0 * v[..., 0] * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 2] += 5.0 * v[..., 0] * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 3] *= 1 + 1e-2 * rng.uniform(-1, 1, v.shape[:-1])
    return v


@pytest.mark.parametrize("polydeg", [2, 3, 5])
@pytest.mark.parametrize("volume,nc", [("tec", "waruszewski"), ("ec", "waruszewski"),
                                       ("etec", "souza"), ("tec", "artiano")])
def test_pt_rhs_matches_oracle(tg, orc, gpu_lib, polydeg, volume, nc):
    eq, mesh, semi = make_pt(tg, polydeg=polydeg, volume=volume, nc=nc)
    u = perturbed(semi.compute_coefficients(), polydeg)
    du = semi.rhs(u)
    c = orc.PotTemp2D(polydeg, 8, 6, 0.0, 300000.0, 0.0, 10000.0, True, False,
                      volume={"tec": 0, "ec": 1, "etec": 2}[volume],
                      nc={"waruszewski": 0, "artiano": 1, "souza": 2}[nc], wall_kind=1,
                      c_lmars=C_LMARS)
    du_ref = c.rhs(u)
    assert np.abs(du - du_ref).max() <= 1e-12 * np.abs(du_ref).max()
    for v in range(4):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(du[..., v] - du_ref[..., v]).max() <= 1e-11 * s, v
    semi.close()


def test_pt_rhs_p4est_normal_walls(tg, orc, gpu_lib):
    eq, mesh, semi = make_pt(tg, normal_walls=True)
    u = perturbed(semi.compute_coefficients(), 9)
    du = semi.rhs(u)
    c = orc.PotTemp2D(3, 8, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, wall_kind=2,
                      c_lmars=C_LMARS)
    du_ref = c.rhs(u[mesh.inv])
    assert np.abs(du[mesh.inv] - du_ref).max() <= 1e-12 * np.abs(du_ref).max()
    semi.close()


def test_gpu_reproduces_pt_gravity_waves_golden(tg, orc, gpu_lib):
    """SSPRK43 at CFL 1 with every rhs evaluated on the GPU (the oracle's own
    max_dt and integrator drive it), to t = 1800 s."""
    eq, mesh, semi = make_pt(tg, nx=60, ny=8)
    c = orc.PotTemp2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, wall_kind=1,
                      c_lmars=C_LMARS)
    u = semi.compute_coefficients()
    t, t_end = 0.0, 1800.0
    while t < t_end:
        dt = min(c.max_dt(u), t_end - t)
        h = 0.5 * dt
        u0 = u.copy()
        tmp = u + h * semi.rhs(u, t)
        tmp = tmp + h * semi.rhs(tmp, t + h)
        tmp = (2.0 / 3.0) * u0 + (1.0 / 3.0) * (tmp + h * semi.rhs(tmp, t + dt))
        u = tmp + h * semi.rhs(tmp, t + h)
        t += dt
    l2, linf = c.errors_gravity_waves(u)
    for v in range(5):
        assert abs(l2[v] - GOLDEN_L2[v]) <= max(ATOL, RTOL * GOLDEN_L2[v])
        assert abs(linf[v] - GOLDEN_LINF[v]) <= max(ATOL, RTOL * GOLDEN_LINF[v])
    for v in range(4):
        assert abs(l2[v] / GOLDEN_L2[v] - 1) < 2e-3, v
    semi.close()
