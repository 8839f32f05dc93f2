"""GPU parity of the potential-temperature path (flux_tec / flux_ec / flux_etec
with the nonconservative gravity terms, LMARS, slip walls) against the CPU
oracle, and the reference's inertia-gravity-wave golden with every stage on the
GPU (the library's integrator is CK2N54; the golden's SSPRK43 steps are driven
from the host, each rhs evaluated by the GPU)."""
import math

import numpy as np
import pytest

from test_oracle_pt import G_GOLDEN, check_gravity_waves_golden

pytestmark = pytest.mark.gpu
C_LMARS = math.sqrt(1004 / 717 * 287 * 250)


def make_pt(tg, nx=8, ny=6, polydeg=3, volume="tec", nc="waruszewski", normal_walls=False,
            gravity=9.80616):
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity2D(c_p=1004, c_v=717,
                                                                         gravity=gravity)
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
    eq, mesh, semi = make_pt(tg, nx=60, ny=8, gravity=G_GOLDEN)
    c = orc.PotTemp2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, wall_kind=1,
                      g=G_GOLDEN, c_lmars=C_LMARS)
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
    check_gravity_waves_golden(l2, linf)
    semi.close()


def test_pt_ec_surface_rhs_matches_oracle(tg, orc, gpu_lib):
    """(flux_etec, Souza) volume flux with the entropy-conservative surface flux
    (flux_ec, flux_nonconservative_waruszewski_etal): the surface gravity term
    differs on the two sides of an interface; StructuredMesh and P4estMesh walls."""
    for normal_walls in (False, True):
        eq, mesh, semi = make_pt(tg, 8, 8, 3, "etec", "souza", normal_walls)
        semi.close()
        solver = tg.DGSEM(3, (tg.flux_ec, tg.flux_nonconservative_waruszewski_etal),
                          tg.VolumeIntegralFluxDifferencing((tg.flux_etec,
                                                             tg.flux_nonconservative_souza_etal)))
        bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
        semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.initial_condition_gravity_waves, solver,
                                               boundary_conditions=bcs)
        u = perturbed(semi.compute_coefficients(), 13)
        du = semi.rhs(u)
        c = orc.PotTemp2D(3, 8, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, volume=2, nc=2,
                          wall_kind=2 if normal_walls else 1, surface=1, snc=0)
        inv = mesh.inv if normal_walls else np.arange(u.shape[0])
        du_ref = c.rhs(u[inv])
        assert np.abs(du[inv] - du_ref).max() <= 1e-12 * np.abs(du_ref).max(), normal_walls
        for v in range(4):
            s = np.abs(du_ref[..., v]).max()
            assert np.abs(du[inv][..., v] - du_ref[..., v]).max() <= 1e-11 * s, (normal_walls, v)
        semi.close()


@pytest.mark.parametrize("name", ["default", "ec_surface"])
def test_gpu_reproduces_well_balanced_curvilinear_golden(tg, orc, gpu_lib, name):
    """elixir_potential_temperature_well_balanced_curvilinear
    (test/test_2d_potential_temperature.jl:100-144) on the curvilinear
    P4estMesh: the rhs against the oracle on the same arrays, then SSPRK43 at
    dt = 0.01 to t = 0.4 and the error norms, all on the GPU."""
    from test_oracle_pt import (WELL_BALANCED, check_well_balanced, well_balanced_arrays,
                                well_balanced_mesh)
    kw, g2, gi = WELL_BALANCED[name]
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity2D(c_p=1004, c_v=717,
                                                                         gravity=9.81)
    mesh = well_balanced_mesh(tg)
    vf = (tg.flux_etec, tg.flux_nonconservative_souza_etal) if name == "ec_surface" else \
        (tg.flux_tec, tg.flux_nonconservative_artiano_etal)
    sf = (tg.flux_ec, tg.flux_nonconservative_waruszewski_etal) if name == "ec_surface" else \
        (tg.FluxLMARS(340.0), tg.flux_zero)
    solver = tg.DGSEM(2, sf, tg.VolumeIntegralFluxDifferencing(vf))
    bcs = {k: tg.boundary_condition_slip_wall for k in ("x_neg", "x_pos", "y_neg", "y_pos")}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.initial_condition_adiabatic, solver,
                                           boundary_conditions=bcs)
    basis, xy, Ja, invJ, arrays = well_balanced_arrays(tg, mesh)
    c = orc.PotTemp2D(2, 0, 0, 0, 0, 0, 0, g=9.81, c_lmars=340.0, mesh=arrays, **kw)
    u = perturbed(semi.compute_coefficients(), 3)
    du, du_ref = semi.rhs(u), c.rhs(u)
    assert np.abs(du - du_ref).max() <= 1e-12 * np.abs(du_ref).max()
    semi.set_state(semi.compute_coefficients())
    t = semi.rk_steps(40, fixed_dt=0.01, t=0.0, method="SSPRK43")
    assert abs(t - 0.4) < 1e-12
    l2, linf = semi.calc_error_norms(0.4)
    check_well_balanced(l2, linf, g2, gi)
    semi.close()


def mountain_semi(tg, name, trees=(20, 12), polydeg=3):
    from test_oracle_pt import mountain_case
    eq, setup, mesh, basis, xy, invJ, arrays, bv, okw, solver = mountain_case(tg, name, trees,
                                                                            polydeg)
    bc = tg.BoundaryConditionDirichlet(setup)
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, setup, solver, source_terms=setup,
        boundary_conditions={"x_neg": bc, "x_pos": bc, "y_neg": tg.boundary_condition_slip_wall,
                             "y_pos": bc})
    return eq, setup, mesh, basis, xy, invJ, arrays, bv, okw, semi


@pytest.mark.parametrize("polydeg", [2, 3, 4])
@pytest.mark.parametrize("name", ["linear_hydrostatic", "schaer_mountain"])
def test_pt_mountain_rhs_matches_oracle(tg, orc, gpu_lib, name, polydeg):
    """Terrain-following P4estMesh, Dirichlet boundary states (left, right, top),
    slip wall at the ground, MountainWaveSetup's damping source, on a perturbed
    state (the damping acts in the absorbing layers)."""
    eq, setup, mesh, basis, xy, invJ, arrays, bv, okw, semi = mountain_semi(tg, name, (8, 6),
                                                                           polydeg)
    # the host mirror's Dirichlet states are the setup at the boundary face nodes
    dirichlet = arrays[-1] == 4
    assert np.abs(semi._H.boundary_values[dirichlet] - bv[dirichlet]).max() == 0.0
    u = perturbed(semi.compute_coefficients(), 30 + polydeg)
    du = semi.rhs(u)
    c = orc.PotTemp2D(polydeg, 0, 0, 0, 0, 0, 0, mesh=arrays, **okw)
    c.set_mountain(setup.params(), bv)
    du_ref = c.rhs(u)
    assert np.abs(du - du_ref).max() <= 1e-12 * np.abs(du_ref).max(), (
        np.abs(du - du_ref).max() / np.abs(du_ref).max())
    for v in range(4):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(du[..., v] - du_ref[..., v]).max() <= 1e-11 * s, v
    semi.close()


@pytest.mark.parametrize("name", ["linear_hydrostatic", "linear_nonhydrostatic",
                                  "schaer_mountain"])
def test_gpu_reproduces_mountain_wave_golden(tg, orc, gpu_lib, name):
    """test/test_2d_potential_temperature.jl:29-98 as the reference runs it:
    error-controlled SSPRK43 at OrdinaryDiffEq's default tolerances with every
    stage and the error estimate on the GPU (tag_rk_adaptive); norms by NumPy and
    on the device against the goldens; the step sequence (accepted and rejected
    steps, first dt) and the final state against the oracle's adaptive run."""
    import analysis
    from test_oracle_pt import MOUNTAIN_T_END, check_mountain
    eq, setup, mesh, basis, xy, invJ, arrays, bv, okw, semi = mountain_semi(tg, name)
    semi.set_state(semi.compute_coefficients())
    t, st = semi.solve_adaptive((0.0, MOUNTAIN_T_END))
    assert t == MOUNTAIN_T_END
    u = semi.get_state()
    l2, linf = analysis.error_norms(u, xy, invJ, basis.nodes, lambda x: setup(x, 0.0, eq), 2)
    check_mountain(name, l2, linf)
    l2d, linfd = semi.calc_error_norms(MOUNTAIN_T_END)
    check_mountain(name, l2d, linfd)
    c = orc.PotTemp2D(3, 0, 0, 0, 0, 0, 0, mesh=arrays, **okw)
    c.set_mountain(setup.params(), bv)
    uo = np.ascontiguousarray(semi.compute_coefficients())
    to, sto = c.ssprk43_adaptive(uo, 0.0, MOUNTAIN_T_END)
    assert (st["accepted"], st["rejected"]) == (sto["accepted"], sto["rejected"]), (st, sto)
    # the starting step divides a difference of two rhs evaluations by the
    # first trial step, which magnifies their rounding
    assert abs(st["dt_first"] / sto["dt_first"] - 1) <= 1e-9
    # the step sizes follow the error norms, whose small differences magnify
    # the rounding of the two implementations (the first dt agrees to 1e-11):
    # the final states agree to ~1e-10
    assert np.abs(u[..., :4] - uo[..., :4]).max() <= 1e-8 * np.abs(uo[..., :4]).max()
    semi.close()


def test_pt_time_dependent_dirichlet_states(tg, orc, gpu_lib):
    """set_boundary_time(t) re-evaluates BoundaryConditionDirichlet's function
    at the boundary nodes; the rhs then equals the oracle's with those states."""
    from test_oracle_pt import mountain_case
    eq, setup, mesh, basis, xy, invJ, arrays, bv, okw, solver = mountain_case(
        tg, "linear_hydrostatic", (6, 4), 3)

    def boundary_value(x, t, equations):
        s = setup(x, t, equations)
        s[..., 1] *= 1.0 + 0.01 * t  # a time-dependent inflow velocity
        return s

    bc = tg.BoundaryConditionDirichlet(boundary_value)
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, setup, solver, source_terms=setup,
        boundary_conditions={"x_neg": bc, "x_pos": bc, "y_neg": tg.boundary_condition_slip_wall,
                             "y_pos": bc})
    u = perturbed(semi.compute_coefficients(), 77)
    c = orc.PotTemp2D(3, 0, 0, 0, 0, 0, 0, mesh=arrays, **okw)
    for t in (0.0, 5.0):
        semi.set_boundary_time(t)
        bvt = bv.copy()
        bvt[..., 1] *= 1.0 + 0.01 * t
        c.set_mountain(setup.params(), bvt)
        du, du_ref = semi.rhs(u, t), c.rhs(u, t)
        assert np.abs(du - du_ref).max() <= 1e-12 * np.abs(du_ref).max(), t
    semi.close()


def test_adaptive_steps_argument_checks_and_stops(tg, orc, gpu_lib):
    """tag_rk_adaptive refuses what it does not define (a non-SSPRK43 scheme,
    decreasing stops, max_steps exhausted) with TAG_E_INVALID and leaves the
    state usable; with stops it lands on each of them (as the reference's
    SaveSolutionCallback tstops) and on t_end, close to the oracle's run."""
    import ctypes
    eq, mesh, semi = make_pt(tg, 8, 6, 3)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    L, h = semi._L, semi._h
    t = ctypes.c_double(0.0)
    st = tg._lib.AdaptiveStats()
    dp = ctypes.POINTER(ctypes.c_double)
    _lib = tg._lib
    assert L.tag_set_time_integrator(h, _lib.TAG_RK_CK2N54) == 0
    assert L.tag_rk_adaptive(h, ctypes.byref(t), 10.0, 1e-6, 1e-3, None, 0, 100,
                             ctypes.byref(st)) == _lib.TAG_E_INVALID
    assert L.tag_set_time_integrator(h, _lib.TAG_RK_SSPRK43) == 0
    bad = np.array([5.0, 2.0])
    assert L.tag_rk_adaptive(h, ctypes.byref(t), 10.0, 1e-6, 1e-3, bad.ctypes.data_as(dp), 2,
                             100, ctypes.byref(st)) == _lib.TAG_E_INVALID
    assert L.tag_rk_adaptive(h, ctypes.byref(t), 1000.0, 1e-6, 1e-3, None, 0, 2,
                             ctypes.byref(st)) == _lib.TAG_E_INVALID
    assert st.accepted + st.rejected == 2 and 0.0 < t.value < 1000.0
    # a fresh run with stops every 7 s to 60 s, against the oracle's
    semi.set_state(u0)
    tf, s = semi.solve_adaptive((0.0, 60.0), save_dt=7.0)
    assert tf == 60.0
    c = orc.PotTemp2D(3, 8, 6, 0.0, 300000.0, 0.0, 10000.0, periodic_x=True, periodic_y=False,
                      volume=0, nc=0, g=9.80616, c_lmars=C_LMARS)
    uo = np.ascontiguousarray(u0).copy()
    to, so = c.ssprk43_adaptive(uo, 0.0, 60.0, stops=np.arange(7.0, 60.0, 7.0))
    # a step that ends just short of a stop adds a short one, decided by the
    # error norm's last bits: the counts agree to a step or two
    assert to == 60.0 and abs(s["accepted"] - so["accepted"]) <= 2, (s, so)
    u = semi.get_state()
    assert np.abs(u[..., :4] - uo[..., :4]).max() <= 1e-7 * np.abs(uo[..., :4]).max()
    semi.close()
