"""Device analysis (tag_analyze_integral, tag_analysis_nodes,
tag_analyze_errors) against the oracle's NumPy restatement (oracle/analysis.py)
for every equation system; reference goldens reproduced with the error norms
computed on the GPU; ensemble members analysed in one call equal to the
members analysed alone (bitwise); repeated calls bitwise equal.

Tolerances: integrals within 1e-12 of the sum of the absolute integrands
(summation order only); the entropy time derivative within 1e-10 of
sum wJ |w . du| (its terms cancel); error norms within 1e-12 relative plus
1e-14 of the variable's largest magnitude (the difference u_exact - u of
values of size |u| rounds at that level, so a near-zero error is noise)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def analysis(orc):
    import analysis as a
    return a


def _weights(analysis, semi):
    w = np.asarray(semi.solver.basis.weights)
    if getattr(semi, "aux_node_vars", None) is not None:
        return analysis.quadrature_weights(w, 2, aux=np.asarray(semi.aux_node_vars))
    nd = semi.ndims
    invJ = np.asarray(semi.inverse_jacobian).reshape((semi.nelements,) + (semi.n,) * nd)
    return analysis.quadrature_weights(w, nd, inv_jacobian=invJ)


def _norms_close(a, b, u):
    mag = np.abs(np.asarray(u)).reshape(-1, np.shape(u)[-1]).max(axis=0)
    return np.all(np.abs(np.asarray(a) - np.asarray(b)) <= 1e-12 * np.asarray(b) + 1e-14 * mag)


def _close(a, b, scale, rtol=1e-12):
    return np.all(np.abs(np.asarray(a) - np.asarray(b)) <= rtol * np.asarray(scale))


def _cases(tg, orc, analysis, name):
    """(semi, state, entropy(u), energy_total(u), cons2entropy(u)) of one system."""
    if name == "energy2d":
        from test_gpu_euler2d import make_semi
        eq, semi = make_semi(tg, 16, 8, 3)
        u = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=3, amplitude=1e-2,
                                   velocity=5.0)
        g = 1004.0 / 717.0
        return semi, u, (lambda x: analysis.energy_entropy(x, g)), (lambda x: x[..., 3]), \
            (lambda x: analysis.energy_cons2entropy(x, g))
    if name == "energy3d":
        from test_gpu_euler3d import make_semi
        from test_oracle_golden_3d import perturb3d
        eq, mesh, semi = make_semi(tg, 3, 2, 4)
        u = perturb3d(semi.compute_coefficients(), eq, seed=2)
        g = 1004.0 / 717.0
        return semi, u, (lambda x: analysis.energy_entropy(x, g)), (lambda x: x[..., 4]), \
            (lambda x: analysis.energy_cons2entropy(x, g))
    if name == "pt":
        from test_gpu_pt import make_pt, perturbed
        eq, mesh, semi = make_pt(tg)
        u = perturbed(semi.compute_coefficients(), 4)
        k = analysis.pt_constants()
        return semi, u, (lambda x: analysis.pt_entropy(x, k)), \
            (lambda x: analysis.pt_energy_total(x, k)), (lambda x: analysis.pt_cons2entropy(x, k))
    if name == "moist":
        from test_gpu_moist import bubble_semi, moist_state
        eq, mesh, semi = bubble_semi(tg, 3)
        u = moist_state(eq, semi.compute_coefficients(), seed=5)
        return semi, u, analysis.moist_entropy, (lambda x: x[..., 3]), analysis.moist_cons2entropy
    if name == "rainy":
        from test_gpu_rainy import make_rainy, moving, solved_state
        eq, semi = make_rainy(tg, 8, 4, 3)
        u = solved_state(orc, moving(semi.compute_coefficients(), seed=7, vel=3.0))
        return semi, u, None, None, analysis.rainy_cons2entropy
    from test_gpu_cov_swe import make_semi, perturbed
    eq, mesh, semi, fluxes, cfl = make_semi(tg, "isolated_mountain", k=3, polydeg=4)
    u = perturbed(semi.compute_coefficients(), seed=6)
    aux = np.asarray(semi.aux_node_vars)
    G = eq.gravity
    return semi, u, (lambda x: analysis.cov_entropy(x, aux, G)), None, \
        (lambda x: analysis.cov_cons2entropy(x, aux, G))


NAMES = ["energy2d", "energy3d", "pt", "moist", "rainy", "covariant"]


@pytest.mark.parametrize("name", NAMES)
def test_integrals_match_oracle(tg, orc, analysis, gpu_lib, name):
    semi, u, S, E, W = _cases(tg, orc, analysis, name)
    u = np.ascontiguousarray(u)
    semi.set_state(u)
    wJ = _weights(analysis, semi)
    vol = wJ.sum()
    for normalize in (True, False):
        d = 1.0 / vol if normalize else 1.0
        st = semi.integrate("cons2cons", normalize=normalize)
        ref = analysis.integrate(u, wJ, normalize=False) * d
        scale = analysis.integrate(np.abs(u), wJ, normalize=False) * d
        assert _close(st, ref, scale), (st, ref)
    if S is not None:
        s = semi.integrate("entropy")
        assert _close(s, analysis.integrate(S(u), wJ), analysis.integrate(np.abs(S(u)), wJ))
    else:
        with pytest.raises(Exception):
            semi.integrate("entropy")
    if E is not None:
        e = semi.integrate("energy_total")
        assert _close(e, analysis.integrate(E(u), wJ), analysis.integrate(np.abs(E(u)), wJ))
    t = 0.3
    du = semi.rhs(u, t) if name != "covariant" else semi.rhs(u)
    wdu = (W(u) * du).sum(-1)
    dsdt = semi.entropy_timederivative(t)
    assert _close(dsdt, analysis.integrate(wdu, wJ), analysis.integrate(np.abs(wdu), wJ),
                  rtol=1e-10), (dsdt, analysis.integrate(wdu, wJ))
    # the same bits on a repeated call
    assert semi.entropy_timederivative(t) == dsdt
    assert np.array_equal(semi.integrate("cons2cons"), semi.integrate("cons2cons"))
    semi.close()


def test_error_norms_reproduce_energy_golden(tg, orc, analysis, gpu_lib):
    """elixir_energy_inertia_gravity_waves (test/test_2d_euler_energy.jl:7-27):
    SSPRK43 to t = 10 s and the l2 / linf norms all on the GPU."""
    from test_gpu_time_integrators import steps_to
    from test_oracle_golden import GOLDEN_L2, GOLDEN_LINF, _isapprox
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
    semi.set_state(semi.compute_coefficients())
    steps_to(semi, 1.0, 10.0, "SSPRK43")
    l2, linf = semi.calc_error_norms(10.0)
    for v in range(5):
        assert _isapprox(l2[v], GOLDEN_L2[v]), (v, l2[v], GOLDEN_L2[v])
        assert _isapprox(linf[v], GOLDEN_LINF[v]), (v, linf[v], GOLDEN_LINF[v])
    # against the oracle's NumPy analysis of the same state
    u = semi.get_state()
    invJ = np.asarray(semi.inverse_jacobian).reshape(u.shape[:-1])
    l2o, linfo = analysis.error_norms(
        u, np.asarray(semi.node_coordinates).reshape(u.shape[:-1] + (2,)), invJ,
        np.asarray(semi.solver.basis.nodes),
        lambda x: tg.initial_condition_gravity_waves(x, 10.0, eq), 2)
    assert _norms_close(l2, l2o, u), (l2, l2o)
    assert _norms_close(linf, linfo, u), (linf, linfo)
    m, x = semi.analysis_nodes()
    assert m == 7 and x.shape == (480, 7, 7, 2)
    xh = semi.analysis_coordinates_host()
    assert np.abs(x - xh).max() <= 1e-14 * np.abs(xh).max()
    semi.close()


def test_error_norms_3d_match_oracle(tg, orc, analysis, gpu_lib):
    from test_gpu_euler3d import make_semi
    from test_oracle_golden_3d import perturb3d
    eq, mesh, semi = make_semi(tg, 3, 2, 3)
    u = np.ascontiguousarray(perturb3d(semi.compute_coefficients(), eq, seed=9))
    semi.set_state(u)
    l2, linf = semi.calc_error_norms(0.0)
    xyz = np.asarray(semi.node_coordinates).reshape(u.shape[:-1] + (3,))
    invJ = np.asarray(semi.inverse_jacobian).reshape(u.shape[:-1])
    l2o, linfo = analysis.error_norms(
        u, xyz, invJ, np.asarray(semi.solver.basis.nodes),
        lambda x: tg.initial_condition_baroclinic_instability(x, 0.0, eq), 3)
    assert _norms_close(l2, l2o, u), (l2, l2o)
    assert _norms_close(linf, linfo, u), (linf, linfo)
    m, x = semi.analysis_nodes()  # device interpolation of the coordinates
    xh = semi.analysis_coordinates_host()
    assert m == 7 and np.abs(x - xh).max() <= 1e-14 * np.abs(xh).max()
    semi.close()


@pytest.mark.parametrize("name", ["well_balanced", "isolated_mountain"])
def test_covariant_golden_with_device_error_norms(tg, gpu_lib, name):
    """One day of the covariant elixir and its l2 / linf norms, all on the GPU."""
    from test_gpu_cov_swe import make_semi
    from test_oracle_cov_swe import N_SAVES, RTOL, check_golden
    cv = tg.covariant
    eq, mesh, semi, fluxes, cfl = make_semi(tg, name)
    semi.set_state(semi.compute_coefficients())
    t_end = cv.SECONDS_PER_DAY
    semi.solve((0.0, t_end), cfl=cfl, save_dt=t_end / N_SAVES)
    l2, linf = semi.calc_error_norms(t_end)
    check_golden(name, l2, linf, RTOL)
    ug = semi.get_state()
    l2h, linfh = cv.error_norms(ug, semi.compute_coefficients(t_end), semi.aux_node_vars,
                                semi.solver.basis)
    assert _norms_close(l2, l2h, ug), (l2, l2h)
    assert _norms_close(linf, linfh, ug), (linf, linfh)
    semi.close()


def test_covariant_ec_entropy_conserved_at_scale(tg, analysis, gpu_lib):
    """Entropy-conservative split form (flux_ec + nonconservative flux_ec,
    no dissipation) on 6 x 16^2 elements of degree 3: the device entropy time
    derivative vanishes to rounding; with LLF dissipation it is negative."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    from test_gpu_cov_swe import perturbed
    eq = cv.SplitCovariantShallowWaterEquations2D(9.80616, 7.292e-5)
    mesh = cv.P4estMeshCubedSphere2D(16, EARTH_RADIUS, polydeg=3)
    vol = tg.VolumeIntegralFluxDifferencing((cv.flux_ec, cv.flux_nonconservative_ec))
    ic = cv.transform_initial_condition(cv.initial_condition_isolated_mountain, eq)
    out = []
    for sf in ((cv.flux_ec, cv.flux_nonconservative_ec),
               (cv.FluxPlusDissipation(cv.flux_ec, cv.DissipationLocalLaxFriedrichs()),
                cv.flux_nonconservative_ec)):
        semi = tg.SemidiscretizationHyperbolic(
            mesh, eq, ic, tg.DGSEM(3, sf, vol), source_terms=cv.source_terms_geometric_coriolis,
            auxiliary_field=cv.bottom_topography_isolated_mountain)
        u = np.ascontiguousarray(perturbed(semi.compute_coefficients(), seed=11))
        semi.set_state(u)
        du = semi.rhs(u)
        aux = np.asarray(semi.aux_node_vars)
        wdu = (analysis.cov_cons2entropy(u, aux, eq.gravity) * du).sum(-1)
        scale = analysis.integrate(np.abs(wdu), _weights(analysis, semi))
        out.append((semi.entropy_timederivative(), scale))
        semi.close()
    (ec, s0), (diss, s1) = out
    assert abs(ec) <= 1e-11 * s0, ec / s0
    assert diss < -1e-6 * s1


def test_ensemble_members_analysed_as_alone(tg, gpu_lib):
    from test_gpu_euler2d import LX, LZ
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(3, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    meshes = [tg.StructuredMesh((nx, 4), (0.0, 0.0), (LX, LZ), periodicity=(True, False))
              for nx in (8, 6, 10)]
    ics = [tg.WarmBubble(), tg.WarmBubble(), tg.WarmBubble()]
    ens = tg.SemidiscretizationEnsemble(meshes, eq, ics, solver, boundary_conditions=bcs)
    u = ens.compute_coefficients()
    u = u * (1 + 1e-3 * np.random.default_rng(0).standard_normal(u.shape))
    ens.set_state(u)
    st, s, dsdt = ens.integrate("cons2cons"), ens.integrate("entropy"), ens.entropy_timederivative()
    l2, linf = ens.calc_error_norms(0.0)
    for m, mesh in enumerate(meshes):
        alone = tg.SemidiscretizationHyperbolic(mesh, eq, ics[m], solver, boundary_conditions=bcs)
        alone.set_state(np.ascontiguousarray(u[ens.member_slice(m)]))
        assert np.array_equal(alone.integrate("cons2cons"), st[m])
        assert alone.integrate("entropy") == s[m]
        assert alone.entropy_timederivative() == dsdt[m]
        a2, ai = alone.calc_error_norms(0.0)
        assert np.array_equal(a2, l2[m]) and np.array_equal(ai, linf[m])
        alone.close()
    ens.close()
