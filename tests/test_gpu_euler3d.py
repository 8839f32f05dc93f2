"""GPU parity of the 3D dry-Euler path (energy + gravity + Coriolis on the
cubed-sphere shell) against the CPU oracle, through the C ABI.

Tolerance as for 2D: ||a - a_oracle||_max <= 1e-12 ||a_oracle||_max over the
whole vector; on seeded far-from-balance states every variable also within
1e-11 of its own max norm.
"""
import numpy as np
import pytest

from test_oracle_golden_3d import check_golden, oracle_3d, perturb3d, shell_case

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL_VAR = 1e-11


def max_norm_rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def per_var(a, b):
    out = 0.0
    for v in range(b.shape[-1]):
        s = np.abs(b[..., v]).max()
        d = np.abs(a[..., v] - b[..., v]).max()
        out = max(out, d / s if s > 0 else (0.0 if d == 0 else np.inf))
    return out


def make_semi(tg, trees, layers, polydeg, coriolis=True, topography=None, adapt=None):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, tg.EARTH_RADIUS, 30000.0,
                                             polydeg=polydeg, initial_topography=topography,
                                             adapt_vertical_grid=adapt)
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, tg.initial_condition_baroclinic_instability, solver,
        source_terms=tg.source_terms_coriolis if coriolis else None,
        boundary_conditions={"inside": tg.boundary_condition_slip_wall,
                             "outside": tg.boundary_condition_slip_wall})
    return eq, mesh, semi


@pytest.mark.parametrize("polydeg", [2, 3, 4, 5, 7])
def test_rhs3d_matches_oracle_seeded(tg, orc, gpu_lib, polydeg):
    eq, mesh, semi = make_semi(tg, 2, 2, polydeg)
    u = perturb3d(semi.compute_coefficients(), eq, seed=300 + polydeg)
    du = semi.rhs(u)
    o = oracle_3d(orc, tg, polydeg, semi.contravariant_vectors, semi.inverse_jacobian,
                  semi.node_coordinates, mesh.connectivity(solver_basis(semi)))
    du_ref = o.rhs(u)
    assert max_norm_rel(du, du_ref) <= RTOL, max_norm_rel(du, du_ref)
    assert per_var(du, du_ref) <= RTOL_VAR, per_var(du, du_ref)
    assert semi.status() == 0
    semi.close()


def solver_basis(semi):
    return semi.solver.basis


def test_rhs3d_independent_of_elements_per_block(tg, gpu_lib):
    eq, mesh, semi = make_semi(tg, 2, 2, 4)
    u = perturb3d(semi.compute_coefficients(), eq, seed=9)
    outs = []
    for epb in (1, 2, 3):
        semi.set_elements_per_block(epb)
        outs.append(semi.rhs(u))
        outs.append(semi.rhs(u))
    for epb in (1, 2):  # half-width CTAs: each warp takes two groups of lines
        semi.set_tile(epb, 2)
        outs.append(semi.rhs(u))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    semi.close()


def test_rk3d_steps_match_oracle(tg, orc, gpu_lib):
    eq, mesh, semi = make_semi(tg, 3, 2, 4)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    dt = semi.max_dt()
    o = oracle_3d(orc, tg, 4, semi.contravariant_vectors, semi.inverse_jacobian,
                  semi.node_coordinates, mesh.connectivity(solver_basis(semi)))
    assert abs(dt - o.max_dt(u0)) <= 1e-13 * dt
    t = semi.rk_steps(3, cfl=1.0, t=0.0)
    uo = u0.copy()
    t_ref = o.ck_steps(uo, np.zeros_like(uo), 0.0, 1.0, 3)
    assert abs(t - t_ref) <= 1e-12 * t_ref
    ug = semi.get_state()
    assert max_norm_rel(ug, uo) <= RTOL
    assert max_norm_rel(ug - u0, uo - u0) <= 1e-9
    assert semi.status() == 0
    semi.close()


def test_gpu_reproduces_reference_golden_3d(tg, orc, gpu_lib):
    """The reference's elixir_energy_baroclinic_instability golden
    (test/test_3d_euler_energy.jl:7-29), time-stepped entirely on the GPU
    (ten CK2N54 steps of 1 ms, one CUDA-graph replay each)."""
    import analysis
    eq, mesh, semi = make_semi(tg, 8, 4, 5)
    u = semi.compute_coefficients()
    semi.set_state(u)
    t = semi.rk_steps(10, fixed_dt=0.001, t=0.0)
    assert abs(t - 0.01) < 1e-15
    ug = semi.get_state()
    l2, linf = analysis.error_norms(
        ug, semi.node_coordinates, semi.inverse_jacobian, solver_basis(semi).nodes,
        lambda x: tg.initial_condition_baroclinic_instability(x, 0.0, eq), 3)
    check_golden(l2, linf)
    # and with the error norms computed on the device (tag_analyze_errors)
    l2d, linfd = semi.calc_error_norms(0.0)
    check_golden(l2d, linfd)
    semi.close()


@pytest.mark.parametrize("vertical", ["galchen", "sleve"])
def test_rhs3d_with_topography_matches_oracle(tg, orc, gpu_lib, vertical):
    """A shell whose ground carries a 2 km Gaussian mountain (GalChen or
    Sleve(0.7, 0.8) vertical coordinates): curved, non-radial element faces
    and slip walls on the terrain."""
    from trixiatmo_gb300.meshes3d import GalChen, Sleve

    def mountain(lat, lon):
        return 2000.0 * np.exp(-((lat - 0.4) ** 2 + (lon - 0.3) ** 2) / 0.05)

    adapt = GalChen() if vertical == "galchen" else Sleve(0.7, 0.8)
    eq, mesh, semi = make_semi(tg, 3, 2, 4, topography=mountain, adapt=adapt)
    u = perturb3d(semi.compute_coefficients(), eq, seed=321)
    du = semi.rhs(u)
    o = oracle_3d(orc, tg, 4, semi.contravariant_vectors, semi.inverse_jacobian,
                  semi.node_coordinates, mesh.connectivity(solver_basis(semi)))
    du_ref = o.rhs(u)
    assert max_norm_rel(du, du_ref) <= RTOL, max_norm_rel(du, du_ref)
    assert per_var(du, du_ref) <= RTOL_VAR, per_var(du, du_ref)
    assert semi.status() == 0
    semi.close()


def test_set_state_from_pinned_memory_matches_pageable(tg, gpu_lib):
    """A state in pinned (mapped) host memory is read by one kernel that stores
    it on the device and reduces the CFL speeds in the same pass; the result
    equals the copy-engine path from pageable memory bit for bit: the state,
    max_dt and the steps that follow."""
    torch = pytest.importorskip("torch")
    eq, mesh, semi = make_semi(tg, 2, 2, 4)
    u = perturb3d(semi.compute_coefficients(), eq, seed=21)
    pinned = torch.empty(u.shape, dtype=torch.float64, pin_memory=True).numpy()
    pinned[...] = u
    out = []
    for src in (np.ascontiguousarray(u), pinned):
        semi.set_state(src)
        back = semi.get_state()
        dt = semi.max_dt()
        t = semi.rk_steps(2, cfl=0.8, t=0.0)
        out.append((back, dt, t, semi.get_state()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][0], u)
    assert out[0][1] == out[1][1] and out[0][2] == out[1][2]
    assert np.array_equal(out[0][3], out[1][3])
    semi.close()


def test_state_sink_holds_each_steps_result(tg, gpu_lib):
    """With a state sink registered, the last stage of every step stores the
    new state into the pinned buffer from inside its kernel: after rk_steps it
    equals get_state bit for bit, for one step and for several; the steps
    themselves are unchanged; error-controlled stepping does not write it, nor
    do steps after it is cleared; a pageable array is refused."""
    torch = pytest.importorskip("torch")
    eq, mesh, semi = make_semi(tg, 2, 2, 4)
    u = perturb3d(semi.compute_coefficients(), eq, seed=5)
    ref = []
    semi.set_state(u)
    for nsteps in (1, 3):
        semi.rk_steps(nsteps, cfl=0.8, t=0.0)
        ref.append(semi.get_state())
    sink = torch.empty(u.shape, dtype=torch.float64, pin_memory=True).numpy()
    sink[...] = np.nan
    semi.set_state_sink(sink)
    semi.set_state(u)
    for k, nsteps in enumerate((1, 3)):
        semi.rk_steps(nsteps, cfl=0.8, t=0.0)
        assert np.array_equal(sink, semi.get_state())
        assert np.array_equal(sink, ref[k])
    # error-controlled stepping (whose rejected steps are discarded) leaves it alone
    sink[...] = 0.0
    semi.set_state(u)
    semi.solve_adaptive((0.0, 2.0), abstol=1e-6, reltol=1e-6)
    assert not sink.any()
    semi.set_state_sink(None)
    semi.rk_steps(1, cfl=0.8, t=0.0)
    assert not sink.any()
    with pytest.raises(tg._lib.TagError, match="pinned"):
        semi.set_state_sink(np.zeros_like(u))
    semi.close()
