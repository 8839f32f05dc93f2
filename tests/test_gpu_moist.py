"""GPU parity of the moist-Euler path (flux_chandrashekar / weak form, FluxLMARS /
flux_lax_friedrichs / flux_chandrashekar surface fluxes, pressure-Riemann slip
walls, geopotential, phase-change and manufactured sources) against the CPU
oracle, and the reference's three moist goldens reproduced with every stage on
the GPU.  All calls go through the C ABI."""
import numpy as np
import pytest

from test_oracle_moist import CASES, check_golden

pytestmark = pytest.mark.gpu

RTOL = 1e-12
CP = dict(c_pd=1004, c_vd=717, c_pv=1885, c_vv=1424)


def max_norm_rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def moist_state(eq, u, seed, vel=15.0):
    """Seeded moisture and velocities on top of a dry state, keeping T."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = u.copy()
    rho = u[..., 0]
    _, T = eq.get_current_condition(u)
    qv = rng.uniform(1e-3, 1.5e-2, rho.shape)
    ql = rng.uniform(0.0, 2e-3, rho.shape)
    v = vel * rng.uniform(-1, 1, rho.shape + (2,))
    qd = 1.0 - qv - ql
    out[..., 1] = rho * v[..., 0]
    out[..., 2] = rho * v[..., 1]
    out[..., 3] = (rho * (qd * eq.c_vd + qv * eq.c_vv + ql * eq.c_pl) * T + rho * qv * eq.L_00 +
                   0.5 * rho * (v ** 2).sum(-1))
    out[..., 4] = rho * qv
    out[..., 5] = rho * ql
    return out


def bubble_semi(tg, polydeg, nx=8, ny=6, surface="lmars", p4est=False, source=None):
    eq = tg.CompressibleMoistEulerEquations2D(**CP, gravity=9.80616)
    sf = {"lmars": tg.FluxLMARS(360.0), "llf": tg.flux_lax_friedrichs,
          "ec": tg.flux_chandrashekar}[surface]
    solver = tg.DGSEM(polydeg, sf, tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
    if p4est:
        mesh = tg.P4estMesh((2, 2), polydeg=1, coordinates_min=(0.0, -5000.0),
                            coordinates_max=(20000.0, 15000.0), initial_refinement_level=2,
                            periodicity=(True, False))
    else:
        mesh = tg.StructuredMesh((nx, ny), (0.0, -5000.0), (20000.0, 15000.0),
                                 periodicity=(True, False))
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.initial_condition_gemein_bubble, solver,
                                           boundary_conditions=bcs,
                                           source_terms=source or tg.source_terms_geopotential)
    return eq, mesh, semi


@pytest.mark.parametrize("polydeg", [2, 3, 4, 5])
@pytest.mark.parametrize("surface,source", [("lmars", "geopotential"), ("llf", "moist_bubble"),
                                            ("ec", "moist_bubble")])
def test_moist_rhs_matches_oracle(tg, orc, gpu_lib, polydeg, surface, source):
    src = {"geopotential": tg.source_terms_geopotential,
           "moist_bubble": tg.source_terms_moist_bubble}[source]
    eq, mesh, semi = bubble_semi(tg, polydeg, surface=surface, source=src)
    u = moist_state(eq, semi.compute_coefficients(), seed=polydeg)
    du = semi.rhs(u)
    c = orc.Moist2D(polydeg, 8, 6, 0.0, 20000.0, -5000.0, 15000.0, True, False,
                    surface_kind={"lmars": 0, "llf": 1, "ec": 2}[surface],
                    source_kind={"geopotential": 1, "moist_bubble": 2}[source], wall_kind=1)
    du_ref = c.rhs(u)
    assert max_norm_rel(du, du_ref) <= RTOL, max_norm_rel(du, du_ref)
    for v in range(6):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(du[..., v] - du_ref[..., v]).max() <= 1e-11 * s, v
    semi.close()


def test_moist_rhs_p4est_walls_and_order(tg, orc, gpu_lib):
    """P4estMesh element order and outward-normal slip walls."""
    eq, mesh, semi = bubble_semi(tg, 3, p4est=True)
    u = moist_state(eq, semi.compute_coefficients(), seed=11)
    du = semi.rhs(u)
    c = orc.Moist2D(3, 8, 8, 0.0, 20000.0, -5000.0, 15000.0, True, False, surface_kind=0,
                    source_kind=1, wall_kind=2)
    du_ref = c.rhs(u[mesh.inv])
    assert max_norm_rel(du[mesh.inv], du_ref) <= RTOL
    semi.close()


def test_moist_weak_form_and_manufactured_sources(tg, orc, gpu_lib):
    for kind, src, ic, sf, weak in (
            (3, tg.source_terms_convergence_test_dry, tg.initial_condition_convergence_test_dry,
             tg.flux_lax_friedrichs, True),
            (4, tg.source_terms_convergence_test_moist,
             tg.initial_condition_convergence_test_moist, tg.flux_chandrashekar, False)):
        g = 0.0 if kind == 3 else 9.80616
        eq = tg.CompressibleMoistEulerEquations2D(**CP, gravity=g)
        vi = (tg.VolumeIntegralWeakForm() if weak
              else tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
        mesh = tg.StructuredMesh((6, 5), (0.0, 0.0), (2.0, 2.0), periodicity=(True, True))
        semi = tg.SemidiscretizationHyperbolic(mesh, eq, ic, tg.DGSEM(3, sf, vi), source_terms=src)
        u = semi.compute_coefficients()
        rng = np.random.default_rng(kind)
        u = u * (1.0 + 1e-3 * rng.standard_normal(u.shape))
        c = orc.Moist2D(3, 6, 5, 0.0, 2.0, 0.0, 2.0, True, True, weak_form=weak,
                        surface_kind=1 if kind == 3 else 2, source_kind=kind, gravity=g,
                        ic_kind=kind - 2)
        c0 = orc.Moist2D(3, 6, 5, 0.0, 2.0, 0.0, 2.0, True, True, weak_form=weak,
                         surface_kind=1 if kind == 3 else 2, source_kind=0, gravity=g)
        for t in (0.0, 0.3):
            du = semi.rhs(u, t)
            du_ref = c.rhs(u, t)
            scale = np.abs(c0.rhs(u, t)).max()
            assert np.abs(du - du_ref).max() <= RTOL * scale, (kind, t)
        semi.close()


def _gpu_golden_run(tg, semi, cfl, t_end):
    semi.set_state(semi.compute_coefficients())
    t = 0.0
    while t < t_end - 1e-15:
        dt = cfl * semi.max_dt()
        if t + dt >= t_end:
            t = semi.rk_steps(1, fixed_dt=t_end - t, t=t)
        else:
            t = semi.rk_steps(1, cfl=cfl, t=t)
    assert abs(t - t_end) < 1e-13
    return semi.get_state(), t


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_reproduces_moist_golden(tg, orc, gpu_lib, name):
    kw, cfl, golden = CASES[name]
    g = kw.get("gravity", 9.80616)
    eq = tg.CompressibleMoistEulerEquations2D(**CP, gravity=g)
    if name == "dry_bubble":
        mesh = tg.P4estMesh((2, 2), polydeg=1, coordinates_min=(0.0, -5000.0),
                            coordinates_max=(20000.0, 15000.0), initial_refinement_level=5,
                            periodicity=(True, False))
        solver = tg.DGSEM(4, tg.FluxLMARS(360.0),
                          tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
        semi = tg.SemidiscretizationHyperbolic(
            mesh, eq, tg.initial_condition_gemein_bubble, solver,
            boundary_conditions={"y_neg": tg.boundary_condition_slip_wall,
                                 "y_pos": tg.boundary_condition_slip_wall},
            source_terms=tg.source_terms_geopotential)
    elif name == "moist_source":
        mesh = tg.StructuredMesh((10, 8), (0.0, 0.0), (2.0, 2.0), periodicity=(True, True))
        solver = tg.DGSEM(3, tg.flux_chandrashekar,
                          tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
        semi = tg.SemidiscretizationHyperbolic(
            mesh, eq, tg.initial_condition_convergence_test_moist, solver,
            source_terms=tg.source_terms_convergence_test_moist)
    else:
        mesh = tg.StructuredMesh((10, 8), (0.0, 0.0), (2.0, 2.0), periodicity=(True, True))
        solver = tg.DGSEM(3, tg.flux_lax_friedrichs)
        semi = tg.SemidiscretizationHyperbolic(
            mesh, eq, tg.initial_condition_convergence_test_dry, solver,
            source_terms=tg.source_terms_convergence_test_dry)
    u, t = _gpu_golden_run(tg, semi, cfl, 0.1)
    if name == "dry_bubble":
        u = u[mesh.inv]
    c = orc.Moist2D(**kw)
    l2, linf = c.errors(u, t)
    rtol = 5e-8 if name == "dry_bubble" else 1.4901161193847656e-8
    check_golden(l2, linf, golden, rtol)
    # the same norms computed on the device (tag_analyze_errors)
    l2d, linfd = semi.calc_error_norms(t)
    check_golden(l2d, linfd, golden, rtol)
    semi.close()


def gravity_wave_semi(tg, polydeg=3, cells=(10, 8)):
    from test_oracle_moist import gravity_wave_faces
    eq = tg.CompressibleMoistEulerEquations2D(**CP, gravity=9.80616)
    mesh = tg.StructuredMesh(cells, periodicity=(True, False), faces=gravity_wave_faces())
    solver = tg.DGSEM(polydeg, tg.FluxLMARS(360.0),
                      tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_nonhydrostatic_gravity_wave, solver,
        boundary_conditions={"y_neg": tg.boundary_condition_slip_wall,
                             "y_pos": tg.boundary_condition_slip_wall},
        source_terms=tg.source_terms_nonhydrostatic_gravity_wave)
    return eq, mesh, semi


@pytest.mark.parametrize("polydeg", [2, 3, 4, 5])
def test_moist_rhs_curved_mesh_with_sponge(tg, orc, gpu_lib, polydeg):
    """The witch-of-Agnesi StructuredMesh (transfinite mapping, curved bottom
    slip wall) with geopotential + phase change + Rayleigh sponge sources, on a
    moist state with random velocities (the sponge acts above 9 km)."""
    from test_oracle_moist import gravity_wave_mesh
    eq, mesh, semi = gravity_wave_semi(tg, polydeg, (8, 6))
    *_, arrays = gravity_wave_mesh(tg, (8, 6), polydeg)
    u = moist_state(eq, semi.compute_coefficients(), seed=40 + polydeg)
    du = semi.rhs(u)
    c = orc.Moist2D(polydeg, 0, 0, 0, 0, 0, 0, surface_kind=0, source_kind=5, c_lmars=360.0,
                    gravity=9.80616, ic_kind=3, mesh=arrays)
    du_ref = c.rhs(u)
    assert max_norm_rel(du, du_ref) <= RTOL, max_norm_rel(du, du_ref)
    for v in range(6):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(du[..., v] - du_ref[..., v]).max() <= 1e-11 * s, v
    semi.close()


def test_gpu_reproduces_nonhydrostatic_gravity_waves_golden(tg, orc, gpu_lib):
    """test/test_2d_moist_euler.jl:59-84 with every SSPRK33 stage on the GPU
    (CFL 0.2, t = 0.1); error norms by the oracle and on the device."""
    from test_oracle_moist import NONHYDROSTATIC_GRAVITY_WAVES, gravity_wave_mesh
    eq, mesh, semi = gravity_wave_semi(tg)
    *_, arrays = gravity_wave_mesh(tg)
    semi.set_state(semi.compute_coefficients())
    t, t_end = 0.0, 0.1
    while t < t_end - 1e-15:
        dt = 0.2 * semi.max_dt()
        if t + dt >= t_end:
            t = semi.rk_steps(1, fixed_dt=t_end - t, t=t, method="SSPRK33")
        else:
            t = semi.rk_steps(1, cfl=0.2, t=t, method="SSPRK33")
    assert abs(t - t_end) < 1e-13
    u = semi.get_state()
    c = orc.Moist2D(3, 0, 0, 0, 0, 0, 0, surface_kind=0, source_kind=5, c_lmars=360.0,
                    gravity=9.80616, ic_kind=3, mesh=arrays)
    l2, linf = c.errors(u, t)
    check_golden(l2, linf, NONHYDROSTATIC_GRAVITY_WAVES)
    l2d, linfd = semi.calc_error_norms(t)
    check_golden(l2d, linfd, NONHYDROSTATIC_GRAVITY_WAVES)
    uo = np.ascontiguousarray(semi.compute_coefficients())
    assert c.ssp_steps(uo, 0.0, 0.2, 10 ** 6, 2, t_end=0.1) == 0.1
    assert max_norm_rel(u, uo) <= 1e-13
    semi.close()


def test_gpu_reproduces_moist_bubble_golden(tg, orc, gpu_lib):
    """test/test_2d_moist_euler.jl:32-57 (Bryan & Fritsch moist bubble on the
    saturated AtmosphereLayers background, 16x8 StructuredMesh, N = 3, slip
    walls all round) with every CK2N54 stage on the GPU; norms by NumPy and on
    the device; the state against the oracle's run."""
    import analysis
    from test_oracle_moist import check_moist_bubble, moist_bubble_ic, moist_bubble_mesh
    eq = tg.CompressibleMoistEulerEquations2D(**CP, gravity=9.80616)
    ic = moist_bubble_ic(tg, eq)
    mesh, basis, xy, Ja, invJ, arrays = moist_bubble_mesh(tg)
    solver = tg.DGSEM(3, tg.FluxLMARS(360.0),
                      tg.VolumeIntegralFluxDifferencing(tg.flux_chandrashekar))
    wall = tg.boundary_condition_slip_wall
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, ic, solver, source_terms=tg.source_terms_moist_bubble,
        boundary_conditions={"x_neg": wall, "x_pos": wall, "y_neg": wall, "y_pos": wall})
    u, t = _gpu_golden_run(tg, semi, 0.2, 0.1)
    l2, linf = analysis.error_norms(u, xy, invJ, basis.nodes, lambda x: ic(x, 0.0, eq), 2)
    check_moist_bubble(l2, linf)
    l2d, linfd = semi.calc_error_norms(t)
    check_moist_bubble(l2d, linfd)
    c = orc.Moist2D(3, 0, 0, 0, 0, 0, 0, surface_kind=0, source_kind=2, c_lmars=360.0,
                    gravity=9.80616, mesh=arrays)
    uo = np.ascontiguousarray(ic(xy, 0.0, eq))
    c.ck_steps(uo, np.zeros_like(uo), 0.0, 0.2, 100000, 0.0, 0.1)
    assert max_norm_rel(u, uo) <= 1e-13
    semi.close()
