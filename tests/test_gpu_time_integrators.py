"""GPU time integrators SSPRK43 and SSPRK33 (tag_set_time_integrator +
tag_rk_steps: the stage update in Shu-Osher form fused into the element
kernels, one captured graph per step) against the oracle's step loops for
every element kernel (2D energy, moist, rainy with the Newton stage limiter,
potential temperature, 3D shell, covariant shallow water), and the reference's
SSPRK43 goldens reproduced with every step, stage and CFL reduction on the GPU.

Tolerances as in the per-equation GPU tests: the state within 1e-12 of its
max norm (whole vector), the change over the steps within 1e-10 of its own
max norm (FP64 reassociation and FMA contraction only)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHEMES = {"SSPRK43": 1, "SSPRK33": 2}


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def check_steps(ug, uo, u0, rtol=1e-12, rtol_change=1e-10):
    assert rel(ug, uo) <= rtol, rel(ug, uo)
    assert rel(ug - u0, uo - u0) <= rtol_change, rel(ug - u0, uo - u0)


def steps_to(semi, cfl, t_end, method):
    """StepsizeCallback(cfl) steps to t_end, the last one shortened to land on it."""
    return semi.solve((0.0, t_end), cfl=cfl, method=method)


@pytest.mark.parametrize("method", list(SCHEMES))
def test_energy2d_ssp_steps_match_oracle(tg, orc, gpu_lib, method):
    from test_gpu_euler2d import make_semi, oracle_case
    eq, semi = make_semi(tg, 16, 8, 3)
    u0 = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=5, amplitude=1e-3,
                                velocity=2.0)
    semi.set_state(u0)
    t = semi.rk_steps(5, cfl=1.0, t=0.0, method=method)
    o = oracle_case(orc, 16, 8, 3)
    uo = u0.copy()
    t_ref = o.ssp_steps(uo, 0.0, 1.0, 5, SCHEMES[method])
    assert abs(t - t_ref) <= 1e-13 * t_ref
    check_steps(semi.get_state(), uo, u0)
    # continuing, then switching back to CarpenterKennedy2N54 (graph rebuilt)
    t2 = semi.rk_steps(2, cfl=1.0, t=t, method=method)
    t2_ref = o.ssp_steps(uo, t_ref, 1.0, 2, SCHEMES[method])
    assert abs(t2 - t2_ref) <= 1e-12 * t2_ref
    t3 = semi.rk_steps(2, cfl=1.0, t=t2)
    t3_ref = o.ck_steps(uo, np.zeros_like(uo), t2_ref, 1.0, 2)
    assert abs(t3 - t3_ref) <= 1e-12 * t3_ref
    check_steps(semi.get_state(), uo, u0)
    assert semi.status() == 0
    semi.close()


def test_energy2d_golden_with_device_ssprk43(tg, orc, gpu_lib):
    """elixir_energy_inertia_gravity_waves (test/test_2d_euler_energy.jl:7-27):
    SSPRK43 at CFL 1 to t = 10 s entirely on the GPU; the state against the
    oracle's SSPRK43 run and the norms against the reference's golden."""
    from test_oracle_golden import GOLDEN_L2, GOLDEN_LINF, _isapprox, igw_case
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    cs = tg.speed_of_sound_isothermal(eq, 250.0)
    solver = tg.DGSEM(3, (tg.FluxLMARS(cs), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh((60, 8), (0.0, 0.0), (300000.0, 10000.0), periodicity=(True, False))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_gravity_waves, solver,
        boundary_conditions={"y_neg": tg.boundary_condition_slip_wall,
                             "y_pos": tg.boundary_condition_slip_wall})
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = steps_to(semi, 1.0, 10.0, "SSPRK43")
    assert abs(t - 10.0) < 1e-12
    ug = semi.get_state()
    c = igw_case(orc)
    uo = np.ascontiguousarray(u0.copy())
    c.ssprk43_run(uo, 0.0, 10.0, 1.0)
    # a near-rest state: the change over 10 s is rounding noise in some
    # components, so only the state is compared
    assert rel(ug, uo) <= 1e-12, rel(ug, uo)
    l2, linf = c.errors_gravity_waves(np.ascontiguousarray(ug))
    for v in range(5):
        assert _isapprox(l2[v], GOLDEN_L2[v]), (v, l2[v], GOLDEN_L2[v])
        assert _isapprox(linf[v], GOLDEN_LINF[v]), (v, linf[v], GOLDEN_LINF[v])
    semi.close()


def test_pt_golden_with_device_ssprk43(tg, orc, gpu_lib):
    """elixir_potential_temperature_inertia_gravity_waves
    (test/test_2d_potential_temperature.jl) to t = 1800 s with SSPRK43 at CFL 1
    entirely on the GPU."""
    from test_gpu_pt import C_LMARS, make_pt
    from test_oracle_pt import G_GOLDEN, check_gravity_waves_golden
    eq, mesh, semi = make_pt(tg, nx=60, ny=8, gravity=G_GOLDEN)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = steps_to(semi, 1.0, 1800.0, "SSPRK43")
    assert abs(t - 1800.0) < 1e-9
    c = orc.PotTemp2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, wall_kind=1,
                      g=G_GOLDEN, c_lmars=C_LMARS)
    ug = semi.get_state()
    l2, linf = c.errors_gravity_waves(np.ascontiguousarray(ug))
    check_gravity_waves_golden(l2, linf)
    uo = np.ascontiguousarray(u0.copy())
    c.ssprk43_run(uo, 0.0, 1800.0, 1.0)
    assert rel(ug, uo) <= 1e-11
    semi.close()


@pytest.mark.parametrize("method", list(SCHEMES))
def test_moist_ssp_steps_match_oracle(tg, orc, gpu_lib, method):
    """Moist bubble (flux_chandrashekar, LMARS, geopotential source) at CFL 0.2,
    the setting of elixir_gemein_nonhydrostatic_gravity_waves (SSPRK33)."""
    from test_gpu_moist import bubble_semi
    eq, mesh, semi = bubble_semi(tg, 3)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = semi.rk_steps(4, cfl=0.2, t=0.0, method=method)
    c = orc.Moist2D(3, 8, 6, 0.0, 20000.0, -5000.0, 15000.0, True, False, surface_kind=0,
                    source_kind=1, wall_kind=1)
    uo = u0.copy()
    t_ref = c.ssp_steps(uo, 0.0, 0.2, 4, SCHEMES[method])
    assert abs(t - t_ref) <= 1e-13 * t_ref
    # four CFL-0.2 steps change the state by ~1e-5 of its max norm, so
    # rounding at 1e-16 of the state is ~1e-11..1e-10 of the change
    check_steps(semi.get_state(), uo, u0, rtol_change=1e-9)
    semi.close()


def test_rainy_ssprk43_with_limiter_matches_oracle(tg, orc, gpu_lib):
    """SSPRK43 with the Newton stage limiter after every stage (the setting of
    elixir_hoeck_bubble)."""
    from test_gpu_rainy import make_rainy, moving, solved_state
    eq, semi = make_rainy(tg, 8, 4, 3)
    u0 = solved_state(orc, moving(semi.compute_coefficients(), seed=7, vel=3.0))
    semi.set_state(u0)
    t = semi.rk_steps(3, cfl=0.5, t=0.0, method="SSPRK43")
    uo = u0.copy()
    c = orc.Rainy2D(3, 8, 4, 0.0, 20000.0, 0.0, 10000.0, True, False)
    t_ref = c.ssp_steps(uo, 0.0, 0.5, 3, 1, 0.0, 0, 1e-9, 20)
    assert abs(t - t_ref) <= 1e-12 * t_ref
    assert rel(semi.get_state(), uo) <= 1e-12
    semi.close()


def test_shell3d_ssprk43_steps_match_oracle(tg, orc, gpu_lib):
    from test_gpu_euler3d import make_semi
    from test_oracle_golden_3d import oracle_3d
    eq, mesh, semi = make_semi(tg, 3, 2, 4)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = semi.rk_steps(3, cfl=1.0, t=0.0, method="SSPRK43")
    o = oracle_3d(orc, tg, 4, semi.contravariant_vectors, semi.inverse_jacobian,
                  semi.node_coordinates, mesh.connectivity(semi.solver.basis))
    uo = u0.copy()
    t_ref = o.ssp_steps(uo, 0.0, 1.0, 3, 1)
    assert abs(t - t_ref) <= 1e-12 * t_ref
    check_steps(semi.get_state(), uo, u0, rtol_change=1e-9)
    semi.close()


@pytest.mark.parametrize("method", list(SCHEMES))
def test_covariant_ssp_steps_match_oracle(tg, orc, gpu_lib, method):
    from test_gpu_cov_swe import make_semi, oracle_for
    eq, mesh, semi, fluxes, cfl = make_semi(tg, "isolated_mountain", k=4, polydeg=3)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = semi.rk_steps(4, cfl=cfl, t=0.0, method=method)
    uo = np.ascontiguousarray(u0).copy()
    t_ref = oracle_for(orc, semi, mesh, eq, fluxes).ssp_steps(uo, 0.0, cfl, 4, SCHEMES[method])
    assert abs(t - t_ref) <= 1e-12 * t_ref
    ug = semi.get_state()
    for v in range(3):
        assert np.abs(ug[..., v] - uo[..., v]).max() <= 1e-11 * np.abs(uo[..., v]).max()
    semi.close()


def test_unknown_integrator_rejected(tg, gpu_lib):
    from test_gpu_euler2d import make_semi
    eq, semi = make_semi(tg, 4, 2, 3)
    semi.set_state(semi.compute_coefficients())
    with pytest.raises(Exception):
        semi.rk_steps(1, method="RK4")
    assert semi._L.tag_set_time_integrator(semi._h, 7) != 0
    semi.close()
