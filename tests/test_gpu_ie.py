"""GPU parity of the internal-energy Euler equations with gravity
(elixir_internal_energy_inertia_gravity_waves: (flux_conservative_etec,
flux_nonconservative_etec) volume flux, (flux_conservative_es,
flux_nonconservative_es) surface flux with its per-side nonconservative part,
slip walls on a P4estMesh) against the CPU oracle, through the C ABI: rhs,
SSPRK43 steps, the elixir run to t = 1800 s, and the device entropy integral.

Tolerance as for the other 2D equations: ||a - a_oracle||_max <= 1e-12
||a_oracle||_max over the whole vector and every variable within 1e-11 of its
own max norm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LX, LZ = 300000.0, 10000.0


def make_ie(tg, trees=(8, 6), polydeg=3, level=0):
    eq = tg.CompressibleEulerInternalEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(polydeg, (tg.flux_conservative_es, tg.flux_nonconservative_es),
                      tg.VolumeIntegralFluxDifferencing((tg.flux_conservative_etec,
                                                         tg.flux_nonconservative_etec)))
    mesh = tg.P4estMesh(trees, polydeg=polydeg, coordinates_min=(0.0, 0.0),
                        coordinates_max=(LX, LZ), initial_refinement_level=level,
                        periodicity=(True, False))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_gravity_waves, solver,
        boundary_conditions={"y_neg": tg.boundary_condition_slip_wall,
                             "y_pos": tg.boundary_condition_slip_wall})
    return eq, mesh, semi


def perturbed(u, seed):
    rng = np.random.Generator(np.random.Philox(seed))
    v = u.copy()
    v[..., 0] *= 1 + 1e-2 * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 1] += 5.0 * v[..., 0] * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 2] += 5.0 * v[..., 0] * rng.uniform(-1, 1, v.shape[:-1])
    v[..., 3] *= 1 + 1e-2 * rng.uniform(-1, 1, v.shape[:-1])
    return v


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("polydeg", [2, 3, 4, 5, 7])
@pytest.mark.parametrize("trees,level", [((8, 6), 0), ((2, 2), 2)])
def test_ie_rhs_matches_oracle(tg, orc, gpu_lib, polydeg, trees, level):
    eq, mesh, semi = make_ie(tg, trees, polydeg, level)
    u = perturbed(semi.compute_coefficients(), polydeg)
    du = semi.rhs(u)
    nx, ny = trees[0] * 2 ** level, trees[1] * 2 ** level
    c = orc.InternalEnergy2D(polydeg, nx, ny, 0.0, LX, 0.0, LZ, True, False)
    du_ref = c.rhs(u[mesh.inv])
    dg = du[mesh.inv]
    assert rel(dg, du_ref) <= 1e-12, rel(dg, du_ref)
    for v in range(4):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(dg[..., v] - du_ref[..., v]).max() <= 1e-11 * s, v
    assert np.all(du[..., 4] == 0)
    semi.close()


def test_ie_ssprk43_steps_match_oracle(tg, orc, gpu_lib):
    eq, mesh, semi = make_ie(tg)
    u0 = perturbed(semi.compute_coefficients(), 11)
    semi.set_state(u0)
    c = orc.InternalEnergy2D(3, 8, 6, 0.0, LX, 0.0, LZ, True, False)
    assert abs(semi.max_dt() - c.max_dt(u0[mesh.inv])) <= 1e-13 * c.max_dt(u0[mesh.inv])
    t = semi.rk_steps(3, cfl=1.0, t=0.0, method="SSPRK43")
    uo = np.ascontiguousarray(u0[mesh.inv])
    t_ref = c.ssp_steps(uo, 0.0, 1.0, 3, 1)
    assert abs(t - t_ref) <= 1e-12 * t_ref
    ug = semi.get_state()[mesh.inv]
    assert rel(ug, uo) <= 1e-12
    assert rel(ug[..., :4] - u0[mesh.inv][..., :4], uo[..., :4] - u0[mesh.inv][..., :4]) <= 1e-9
    semi.close()


def test_ie_elixir_run_matches_oracle(tg, orc, gpu_lib):
    """The elixir (60 x 8 trees, N = 3, SSPRK43 at CFL 1) to t = 1800 s with
    every step on the GPU, against the oracle's run; the device entropy
    integral (the elixir's extra analysis integral) against the reference's
    `entropy` evaluated in NumPy."""
    from test_gpu_time_integrators import steps_to
    eq, mesh, semi = make_ie(tg, (60, 8))
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = steps_to(semi, 1.0, 1800.0, "SSPRK43")
    assert abs(t - 1800.0) < 1e-9
    ug = semi.get_state()
    c = orc.InternalEnergy2D(3, 60, 8, 0.0, LX, 0.0, LZ, True, False)
    uo = np.ascontiguousarray(u0[mesh.inv])
    assert c.ssp_steps(uo, 0.0, 1.0, 10 ** 7, 1, t_end=1800.0) == 1800.0
    assert rel(ug[mesh.inv], uo) <= 1e-11, rel(ug[mesh.inv], uo)
    w = np.asarray(semi.solver.basis.weights)
    invJ = np.asarray(semi.inverse_jacobian).reshape(ug.shape[:-1])
    wJ = (w[None, :] * w[:, None])[None] * np.abs(1.0 / invJ)
    p = (eq.gamma - 1) * ug[..., 3]
    S = -(np.log(p) - eq.gamma * np.log(ug[..., 0])) * ug[..., 0] / (eq.gamma - 1)
    ref = (wJ * S).sum() / wJ.sum()
    assert abs(semi.integrate("entropy") - ref) <= 1e-12 * (wJ * np.abs(S)).sum() / wJ.sum()
    semi.close()
