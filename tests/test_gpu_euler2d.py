"""GPU parity of the 2D dry-Euler (energy + gravity) path against the CPU oracle.

Tolerance: ||a - a_oracle||_max <= 1e-12 ||a_oracle||_max over the whole
vector (FP64 reassociation and FMA contraction only).  On the seeded,
far-from-balance states every variable must in addition be within 1e-11 of its
own max norm; on states at rest some components of du are pure rounding noise
(e.g. rho_v1 of a bubble at rest, ~1e-13 on both sides), where a per-variable
ratio has no meaning.  Every call goes through the C ABI (libtrixiatmo_gpu.so).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12      # whole-vector max norm
RTOL_VAR = 1e-11  # per variable
LX, LZ = 20000.0, 10000.0


def make_semi(tg, nx, ny, polydeg=3, c=340.0, periodic=(True, False), bc=True):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(c), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh((nx, ny), (0.0, 0.0), (LX, LZ), periodicity=periodic)
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall,
           "x_neg": tg.boundary_condition_slip_wall, "x_pos": tg.boundary_condition_slip_wall}
    return eq, tg.SemidiscretizationHyperbolic(mesh, eq, tg.WarmBubble(), solver,
                                               boundary_conditions=bcs)


def oracle_case(orc, nx, ny, polydeg=3, c=340.0, periodic=(True, False)):
    return orc.Euler2D(polydeg, nx, ny, 0.0, LX, 0.0, LZ, periodic[0], periodic[1], 1004.0, 717.0,
                       9.81, c)


def max_norm_rel(a, b):
    """||a - b||_max / ||b||_max over the whole array."""
    return np.abs(a - b).max() / np.abs(b).max()


def close(a, b):
    return max_norm_rel(a, b) <= RTOL


def close_per_variable(a, b):
    return max_norm_rel(a, b) <= RTOL and rel_err(a, b) <= RTOL_VAR


def rel_err(a, b):
    """max over variables of max|a_v - b_v| / max|b_v| (variables with b = 0
    must match to an absolute 1e-300)."""
    out = 0.0
    for v in range(b.shape[-1]):
        scale = np.abs(b[..., v]).max()
        d = np.abs(a[..., v] - b[..., v]).max()
        out = max(out, d / scale if scale > 0 else (0.0 if d < 1e-300 else math.inf))
    return out


@pytest.mark.parametrize("polydeg", [1, 2, 3, 4, 5, 7])
def test_rhs_matches_oracle_seeded(tg, orc, gpu_lib, polydeg):
    eq, semi = make_semi(tg, 8, 4, polydeg)
    u = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=100 + polydeg)
    du = semi.rhs(u)
    du_ref = oracle_case(orc, 8, 4, polydeg).rhs(u)
    assert close_per_variable(du, du_ref), (max_norm_rel(du, du_ref), rel_err(du, du_ref))
    assert semi.status() == 0
    semi.close()


def test_rhs_matches_oracle_bubble(tg, orc, gpu_lib):
    """Unperturbed warm bubble at cfg0 resolution (64x32, N = 3), at rest.

    Away from the bubble du is the residual of a near-hydrostatic balance:
    O(1e-7) left over from flux terms of size |p| |Ja| |Dsplit| |invJ| ~ 5e3, so
    any two FP64 evaluation orders differ there by ~1e-10 absolute.  The
    tolerance is therefore taken relative to that term magnitude."""
    eq, semi = make_semi(tg, 64, 32, 3)
    u = semi.compute_coefficients()
    du = semi.rhs(u)
    du_ref = oracle_case(orc, 64, 32, 3).rhs(u)
    _, _, _, p, _ = eq.cons2prim(u)
    term = (np.abs(p).max() * np.abs(semi.contravariant_vectors).max() *
            np.abs(semi.solver.basis.derivative_split).max() *
            np.abs(semi.inverse_jacobian).max())
    assert np.abs(du - du_ref).max() <= RTOL * term, (np.abs(du - du_ref).max(), term)
    # the buoyancy signal itself (rho_v2 inside the bubble) agrees far better
    big = np.abs(du_ref[..., 2]) > 1e-3 * np.abs(du_ref[..., 2]).max()
    assert np.abs(du[..., 2] - du_ref[..., 2])[big].max() <= 1e-8 * np.abs(du_ref[..., 2]).max()
    semi.close()


def test_rhs_walls_all_sides(tg, orc, gpu_lib):
    eq, semi = make_semi(tg, 6, 5, 3, periodic=(False, False))
    u = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=3)
    # the StructuredMesh slip wall of the reference mirrors v2 on every wall
    du = semi.rhs(u)
    du_ref = oracle_case(orc, 6, 5, 3, periodic=(False, False)).rhs(u)
    assert close_per_variable(du, du_ref), (max_norm_rel(du, du_ref), rel_err(du, du_ref))
    semi.close()


def test_rhs_independent_of_elements_per_block_and_deterministic(tg, gpu_lib):
    eq, semi = make_semi(tg, 16, 8, 3)
    u = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=11)
    outs = []
    for epb in (1, 2, 3, 4, 8, 16):
        semi.set_elements_per_block(epb)
        outs.append(semi.rhs(u))
        outs.append(semi.rhs(u))
    # the autotuner's other dimension: two work items per thread and phase
    for epb in (4, 8, 16):
        semi.set_tile(epb, 2)
        assert semi.cta_threads() < semi_threads_full(semi, epb)
        outs.append(semi.rhs(u))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    semi.close()


def semi_threads_full(semi, epb):
    semi.set_tile(epb, 1)
    full = semi.cta_threads()
    semi.set_tile(epb, 2)
    return full


def test_max_dt_matches_oracle(tg, orc, gpu_lib):
    eq, semi = make_semi(tg, 16, 8, 3)
    u = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=5)
    semi.set_state(u)
    dt = semi.max_dt()
    dt_ref = oracle_case(orc, 16, 8, 3).max_dt(u)
    assert abs(dt - dt_ref) <= 1e-13 * dt_ref
    semi.close()


@pytest.mark.parametrize("epb", [0, 1, 4])
def test_rk_steps_match_oracle(tg, orc, gpu_lib, epb):
    """CarpenterKennedy2N54 steps with dt = cfl * max_dt (StepsizeCallback)."""
    eq, semi = make_semi(tg, 16, 8, 3)
    if epb:
        semi.set_elements_per_block(epb)
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    t = semi.rk_steps(5, cfl=1.0, t=0.0)
    ug = semi.get_state()
    o = oracle_case(orc, 16, 8, 3)
    uo = u0.copy()
    k = np.zeros_like(uo)
    t_ref = o.ck_steps(uo, k, 0.0, 1.0, 5)
    assert abs(t - t_ref) <= 1e-13 * t_ref
    assert max_norm_rel(ug - u0, uo - u0) <= 1e-10
    assert close(ug, uo)
    # continuing keeps the 2N register and the CFL reduction consistent
    t2 = semi.rk_steps(3, cfl=1.0, t=t)
    t2_ref = o.ck_steps(uo, k, t_ref, 1.0, 3)
    assert abs(t2 - t2_ref) <= 1e-12 * t2_ref
    assert close(semi.get_state(), uo)
    assert semi.status() == 0
    semi.close()


def test_rk_fixed_dt_matches_oracle(tg, orc, gpu_lib):
    eq, semi = make_semi(tg, 8, 4, 3)
    u0 = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=21, amplitude=1e-3,
                                velocity=1.0)
    semi.set_state(u0)
    t = semi.rk_steps(4, fixed_dt=0.05, t=1.0)
    o = oracle_case(orc, 8, 4, 3)
    uo = u0.copy()
    t_ref = o.ck_steps(uo, np.zeros_like(uo), 1.0, 1.0, 4, 0.05)
    assert abs(t - t_ref) < 1e-14
    assert close(semi.get_state(), uo)
    semi.close()


def test_gpu_rhs_reproduces_reference_golden(tg, orc, gpu_lib):
    """The reference's elixir_energy_inertia_gravity_waves golden
    (test/test_2d_euler_energy.jl:7-27) with every rhs evaluated on the GPU
    (SSPRK43 stages combined on the host) and the oracle's error analysis."""
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
    u = semi.compute_coefficients()
    t, t_end = 0.0, 10.0
    while t < t_end:
        semi.set_state(u)
        dt = semi.max_dt()
        dt = min(dt, t_end - t)
        h = 0.5 * dt
        u0 = u.copy()
        u1 = u + h * semi.rhs(u, t)
        u2 = u1 + h * semi.rhs(u1, t + h)
        u3 = (2.0 / 3.0) * u0 + (1.0 / 3.0) * (u2 + h * semi.rhs(u2, t + dt))
        u = u3 + h * semi.rhs(u3, t + h)
        t += dt
    from test_oracle_golden import GOLDEN_L2, GOLDEN_LINF, _isapprox, igw_case
    l2, linf = igw_case(orc).errors_gravity_waves(np.ascontiguousarray(u))
    for v in range(5):
        assert _isapprox(l2[v], GOLDEN_L2[v]), (v, l2[v], GOLDEN_L2[v])
        assert _isapprox(linf[v], GOLDEN_LINF[v]), (v, linf[v], GOLDEN_LINF[v])
    semi.close()


def test_status_flags_bad_state_injected_on_host(tg, gpu_lib):
    """Failure detection without a GPU fault: a negative density planted in the
    host state sets the status bits; the context stays usable."""
    eq, semi = make_semi(tg, 8, 4, 3)
    u = semi.compute_coefficients()
    bad = u.copy()
    bad[3, 1, 1, 0] = -1.0
    semi.rhs(bad)
    st = semi.status(clear=True)
    assert st & tg._lib.TAG_S_NEG_DENSITY
    semi.rhs(u)
    assert semi.status() == 0
    semi.close()


def test_ensemble_members_match_independent_oracle_runs(tg, orc, gpu_lib):
    """Members of uneven bubble amplitude advance with their own dt and match
    independent oracle runs of each member."""
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(3, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh((8, 4), (0.0, 0.0), (LX, LZ), periodicity=(True, False))
    params = [(9000.0, 2500.0, 1.0), (10500.0, 1500.0, 3.0), (10000.0, 2000.0, 2.0)]
    ics = [tg.WarmBubble(xc=a, zc=b, dtheta=c, v1=5.0 * k) for k, (a, b, c) in enumerate(params)]
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    ens = tg.SemidiscretizationEnsemble([mesh] * 3, eq, ics, solver, boundary_conditions=bcs)
    u0 = ens.compute_coefficients()
    ens.set_state(u0)
    dts = ens.max_dt_members()
    t = ens.rk_steps(4, cfl=1.0, t=np.zeros(3))
    ug = ens.get_state()
    for m in range(3):
        sl = ens.member_slice(m)
        o = oracle_case(orc, 8, 4, 3)
        uo = np.ascontiguousarray(u0[sl])
        assert abs(dts[m] - o.max_dt(uo)) <= 1e-13 * dts[m]
        t_ref = o.ck_steps(uo, np.zeros_like(uo), 0.0, 1.0, 4)
        assert abs(t[m] - t_ref) <= 1e-12 * t_ref
        assert close(ug[sl], uo)
    # members really have different time steps
    assert len(set(np.round(t, 12))) == 3
    ens.close()


def test_state_sink_2d_ensemble_and_rainy(tg, gpu_lib):
    """A 2D ensemble's state sink: after rk_steps it holds every member's new
    state, bit for bit what get_state copies; for the rainy equations the
    stage limiter after the last stage stores the limited state."""
    torch = pytest.importorskip("torch")
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(3, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    meshes = [tg.StructuredMesh((nx, 4), (0.0, 0.0), (LX, LZ), periodicity=(True, False))
              for nx in (6, 8, 4)]
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    ens = tg.SemidiscretizationEnsemble(meshes, eq, [tg.WarmBubble()] * 3, solver,
                                        boundary_conditions=bcs)
    u = ens.compute_coefficients()
    ens.set_state(u)
    ens.rk_steps(2, cfl=1.0, t=np.zeros(3))
    ref = ens.get_state()
    sink = torch.empty(u.shape, dtype=torch.float64, pin_memory=True).numpy()
    sink[...] = np.nan
    ens.set_state_sink(sink)
    ens.set_state(u)
    ens.rk_steps(2, cfl=1.0, t=np.zeros(3))
    assert np.array_equal(sink, ref) and np.array_equal(sink, ens.get_state())
    ens.set_state_sink(None)
    ens.close()
    from test_gpu_rainy import make_rainy
    _, rainy = make_rainy(tg, 8, 4, 3)
    u = rainy.compute_coefficients()
    rainy.set_state(u)
    rainy.rk_steps(2, cfl=0.5, t=0.0)
    ref = rainy.get_state()
    sink = torch.empty(u.shape, dtype=torch.float64, pin_memory=True).numpy()
    sink[...] = np.nan
    rainy.set_state_sink(sink)
    rainy.set_state(u)
    rainy.rk_steps(2, cfl=0.5, t=0.0)
    assert np.array_equal(sink, ref) and np.array_equal(sink, rainy.get_state())
    rainy.close()
