"""GPU parity of the 3D potential-temperature equations with gravity on the
cubed-sphere shell (flux_tec / flux_ec / flux_etec with the Waruszewski,
Artiano or Souza gravity term, (FluxLMARS(340), flux_zero), slip walls,
Coriolis) against the CPU oracle, through the C ABI: rhs, CK2N54 and SSPRK43
steps, and the device analysis integrals.

Tolerance as for the 3D energy equations: ||a - a_oracle||_max <= 1e-12
||a_oracle||_max over the whole vector and every variable within 1e-11 of its
own max norm on seeded far-from-balance states."""
import numpy as np
import pytest

from test_oracle_pt3d import perturb_pt3d

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL_VAR = 1e-11
VOLUME = {"tec": 0, "ec": 1, "etec": 2, "kennedy_gruber": 3}
NC = {"waruszewski": 0, "artiano": 1, "souza": 2}


def make_pt3d(tg, trees, layers, polydeg, volume="tec", nc="souza"):
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, tg.EARTH_RADIUS, 30000.0,
                                             polydeg=polydeg)
    vf = {"tec": tg.flux_tec, "ec": tg.flux_ec, "etec": tg.flux_etec,
          "kennedy_gruber": tg.flux_kennedy_gruber}[volume]
    ncf = {"waruszewski": tg.flux_nonconservative_waruszewski_etal,
           "artiano": tg.flux_nonconservative_artiano_etal,
           "souza": tg.flux_nonconservative_souza_etal}[nc]
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing((vf, ncf)))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_baroclinic_instability, solver,
        source_terms=tg.source_terms_coriolis,
        boundary_conditions={"inside": tg.boundary_condition_slip_wall,
                             "outside": tg.boundary_condition_slip_wall})
    return eq, mesh, semi


def oracle_pt3d(orc, tg, semi, mesh, volume, nc):
    return orc.PotTemp3D(semi.solver.polydeg, semi.contravariant_vectors, semi.inverse_jacobian,
                         semi.node_coordinates, *mesh.connectivity(semi.solver.basis).arrays(),
                         c_p=1004.0, c_v=717.0, g=tg.EARTH_GRAVITATIONAL_ACCELERATION,
                         c_lmars=340.0, omega=tg.EARTH_ROTATION_RATE, volume=VOLUME[volume],
                         nc=NC[nc])


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("polydeg", [2, 3, 4, 5, 7])
@pytest.mark.parametrize("volume,nc", [("tec", "souza"), ("ec", "waruszewski"),
                                       ("etec", "artiano"), ("tec", "waruszewski"),
                                       ("kennedy_gruber", "souza"),
                                       ("kennedy_gruber", "waruszewski")])
def test_pt3d_rhs_matches_oracle(tg, orc, gpu_lib, polydeg, volume, nc):
    eq, mesh, semi = make_pt3d(tg, 3, 2, polydeg, volume, nc)
    u = perturb_pt3d(semi.compute_coefficients(), seed=polydeg)
    du = semi.rhs(u)
    du_ref = oracle_pt3d(orc, tg, semi, mesh, volume, nc).rhs(u)
    assert rel(du, du_ref) <= RTOL, rel(du, du_ref)
    for v in range(5):
        s = np.abs(du_ref[..., v]).max()
        assert np.abs(du[..., v] - du_ref[..., v]).max() <= RTOL_VAR * s, v
    assert np.all(du[..., 5] == 0)
    semi.close()


@pytest.mark.parametrize("method", ["CarpenterKennedy2N54", "SSPRK43"])
def test_pt3d_steps_match_oracle(tg, orc, gpu_lib, method):
    eq, mesh, semi = make_pt3d(tg, 3, 2, 4, "tec", "souza")
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    o = oracle_pt3d(orc, tg, semi, mesh, "tec", "souza")
    assert abs(semi.max_dt() - o.max_dt(u0)) <= 1e-13 * o.max_dt(u0)
    t = semi.rk_steps(3, cfl=1.0, t=0.0, method=method)
    uo = u0.copy()
    if method == "SSPRK43":
        t_ref = o.ssp_steps(uo, 0.0, 1.0, 3, 1)
    else:
        t_ref = o.ck_steps(uo, np.zeros_like(uo), 0.0, 1.0, 3)
    assert abs(t - t_ref) <= 1e-12 * t_ref
    ug = semi.get_state()
    assert rel(ug, uo) <= RTOL
    # the change of the active variables; the passive geopotential (|phi| up to
    # 6e7 here) stays exact on the GPU, while the oracle's SSP combination
    # 2/3 u0 + 1/3 u rounds it by ~1e-8
    assert rel(ug[..., :5] - u0[..., :5], uo[..., :5] - u0[..., :5]) <= 1e-9
    assert np.array_equal(ug[..., 5], u0[..., 5])
    assert semi.status() == 0
    semi.close()


def test_pt3d_analysis_integrals(tg, orc, gpu_lib):
    """Device entropy, total energy and entropy time derivative against the
    reference's formulas (entropy :571-578, energy_total :593-603, cons2entropy
    :560-569) evaluated in NumPy on the same state."""
    eq, mesh, semi = make_pt3d(tg, 3, 2, 3, "ec", "waruszewski")
    u = np.ascontiguousarray(perturb_pt3d(semi.compute_coefficients(), seed=7))
    semi.set_state(u)
    w = np.asarray(semi.solver.basis.weights)
    invJ = np.asarray(semi.inverse_jacobian).reshape(u.shape[:-1])
    wJ = (w[:, None, None] * w[None, :, None] * w[None, None, :])[None] * np.abs(1.0 / invJ)
    g, K, R, p0 = eq.gamma, eq.K, eq.R, eq.p_0
    p = K * u[..., 4] ** g
    S = -(np.log(p) - g * np.log(u[..., 0])) * u[..., 0] / (g - 1)
    E = p0 * (R * u[..., 4] / p0) ** g / (g - 1) + 0.5 * (u[..., 1:4] ** 2).sum(-1) / u[..., 0]
    du = semi.rhs(u)
    wdu = (np.log(K * (u[..., 4] / u[..., 0]) ** g) - g) * du[..., 0] + \
        u[..., 0] / u[..., 4] * g * du[..., 4]
    vol = wJ.sum()
    for got, f, tol in ((semi.integrate("entropy"), S, 1e-12),
                        (semi.integrate("energy_total"), E, 1e-12),
                        (semi.entropy_timederivative(), wdu, 1e-10)):
        ref = (wJ * f).sum() / vol
        assert abs(got - ref) <= tol * (wJ * np.abs(f)).sum() / vol, (got, ref)
    semi.close()


@pytest.mark.parametrize("name,volume,nc", [("souza", "tec", "souza"),
                                            ("waruszewski", "ec", "waruszewski"),
                                            ("artiano", "etec", "artiano")])
def test_gpu_reproduces_baroclinic_instability_goldens(tg, orc, gpu_lib, name, volume, nc):
    """test/test_3d_potential_temperature.jl:100-177 as the reference runs them:
    error-controlled SSPRK43 (abstol = reltol = 1e-6, stops every 100 s) with
    every stage and the error estimate on the GPU (tag_rk_adaptive).  The
    stops every 100 s make the step count sensitive to the last bits of the
    error norms: a step that ends just short of a stop adds one short step, so
    the GPU's step count is within a few of the oracle's (equal for two of the
    three cases) and its final state within 1e-6 of the oracle's; norms against the goldens within the bounds
    of tests/test_oracle_pt3d.py."""
    import analysis
    from test_oracle_pt3d import BAROCLINIC_T_END, baroclinic_stops, check_baroclinic
    eq, mesh, semi = make_pt3d(tg, 2, 2, 5, volume, nc)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t, st = semi.solve_adaptive((0.0, BAROCLINIC_T_END), abstol=1e-6, reltol=1e-6, save_dt=100.0)
    assert t == BAROCLINIC_T_END
    u = semi.get_state()
    basis = semi.solver.basis
    ic = lambda x: tg.initial_condition_baroclinic_instability(x, 0.0, eq)  # noqa: E731
    l2, linf = analysis.error_norms(u, semi.node_coordinates, semi.inverse_jacobian, basis.nodes,
                                    ic, 3)
    check_baroclinic(name, l2, linf)
    o = oracle_pt3d(orc, tg, semi, mesh, volume, nc)
    uo = np.ascontiguousarray(u0).copy()
    to, sto = o.ssprk43_adaptive(uo, 0.0, BAROCLINIC_T_END, abstol=1e-6, reltol=1e-6,
                                 stops=baroclinic_stops())
    assert abs(st["accepted"] - sto["accepted"]) <= 5 and st["rejected"] == sto["rejected"], (
        st, sto)
    assert rel(u[..., :5], uo[..., :5]) <= 1e-6
    semi.close()


@pytest.mark.parametrize("case", ["galchen", "sleve"])
def test_gpu_reproduces_vortex_shedding_goldens(tg, orc, gpu_lib, case):
    """test/test_3d_potential_temperature.jl:244-296 (small-Earth vortex
    shedding over a Gaussian mountain, GalChen or Sleve vertical coordinates)
    with error-controlled SSPRK43 on the GPU: goldens at the test's own rtol
    1e-9, step sequence and final state against the oracle's run."""
    import analysis
    from test_oracle_pt3d import VORTEX_T_END, check_vortex, vortex_mesh
    eq = tg.CompressibleEulerPotentialTemperatureEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = vortex_mesh(tg, case)
    solver = tg.DGSEM(5, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing((tg.flux_tec,
                                                         tg.flux_nonconservative_souza_etal)))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_vortex_shedding, solver,
        source_terms=tg.source_terms_coriolis_small_earth,
        boundary_conditions={"inside": tg.boundary_condition_slip_wall,
                             "outside": tg.boundary_condition_slip_wall})
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t, st = semi.solve_adaptive((0.0, VORTEX_T_END), abstol=1e-6, reltol=1e-6)
    assert t == VORTEX_T_END
    u = semi.get_state()
    ic = lambda x: tg.initial_condition_vortex_shedding(x, 0.0, eq)  # noqa: E731
    l2, linf = analysis.error_norms(u, semi.node_coordinates, semi.inverse_jacobian,
                                    semi.solver.basis.nodes, ic, 3)
    check_vortex(case, l2, linf)
    o = orc.PotTemp3D(5, semi.contravariant_vectors, semi.inverse_jacobian, semi.node_coordinates,
                      *mesh.connectivity(semi.solver.basis).arrays(), c_p=1004.0, c_v=717.0,
                      g=tg.EARTH_GRAVITATIONAL_ACCELERATION, c_lmars=340.0,
                      omega=tg.SMALL_EARTH_ROTATION_RATE, volume=0, nc=2)
    uo = np.ascontiguousarray(u0).copy()
    to, sto = o.ssprk43_adaptive(uo, 0.0, VORTEX_T_END, abstol=1e-6, reltol=1e-6)
    assert (st["accepted"], st["rejected"]) == (sto["accepted"], sto["rejected"]), (st, sto)
    assert rel(u[..., :5], uo[..., :5]) <= 1e-8  # step sizes from rounding-sensitive norms
    semi.close()


def test_combined_fluxes_run_as_their_tuples(tg, orc, gpu_lib):
    """The reference's "combined fluxes" testset
    (test/test_3d_potential_temperature.jl:179-208): the baroclinic instability
    on trees_per_cube_face = (2, 2) for 100 s with (flux_kennedy_gruber,
    flux_nonconservative_souza_etal) / (FluxLMARS(340), flux_zero), and the
    same with the fused flux_kennedy_gruber_souza_etal / flux_lmars_combined.
    The fused spellings run the same kernels (same bits); the run matches the
    oracle's step for step (error-controlled SSPRK43, abstol = reltol = 1e-6 as
    the elixir; no stop before the end)."""
    eq, mesh, semi = make_pt3d(tg, 2, 2, 5, "kennedy_gruber", "souza")
    fused = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_baroclinic_instability,
        tg.DGSEM(5, tg.flux_lmars_combined,
                 tg.VolumeIntegralFluxDifferencing(tg.flux_kennedy_gruber_souza_etal)),
        source_terms=tg.source_terms_coriolis,
        boundary_conditions={"inside": tg.boundary_condition_slip_wall,
                             "outside": tg.boundary_condition_slip_wall})
    u0 = semi.compute_coefficients()
    runs = []
    for s_ in (semi, fused):
        s_.set_state(u0)
        t, st = s_.solve_adaptive((0.0, 100.0), abstol=1e-6, reltol=1e-6)
        assert t == 100.0
        runs.append((s_.get_state(), st))
    assert np.array_equal(runs[0][0], runs[1][0]) and runs[0][1] == runs[1][1]
    o = oracle_pt3d(orc, tg, semi, mesh, "kennedy_gruber", "souza")
    uo = np.ascontiguousarray(u0).copy()
    to, sto = o.ssprk43_adaptive(uo, 0.0, 100.0, abstol=1e-6, reltol=1e-6)
    assert to == 100.0 and abs(runs[0][1]["accepted"] - sto["accepted"]) <= 1, (runs[0][1], sto)
    assert rel(runs[0][0][..., :5], uo[..., :5]) <= 1e-8, rel(runs[0][0][..., :5], uo[..., :5])
    semi.close()
    fused.close()
