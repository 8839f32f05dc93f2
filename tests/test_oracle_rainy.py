"""Pins the rainy-Euler oracle against the reference's own golden vector
(CPU only): test/test_2d_rainy_euler.jl:7-40 runs
examples/euler/precipitation/tests/convergence_test.jl (StructuredMesh 6x6 on
[0,2]^2, polydeg 3, VolumeIntegralWeakForm, flux_lax_friedrichs, manufactured
source, CarpenterKennedy2N54 at CFL 1 with the Newton stage limiter of
tolerance 1e-8) to t = 2 and compares l2/linf with Julia's default rtol."""
import math

import numpy as np

GOLDEN_L2 = [2.39895785368954e-6, 3.892427386570826e-5, 1.5186141589998252e-5,
             0.007532307120716242, 0.02085654062623111, 51.988569260688045,
             1.7470730680079724e-8, 3.892376665583286e-5, 0.0002156633044466944]
GOLDEN_LINF = [1.675032502916618e-5, 0.0002740479581908595, 8.691475272920579e-5,
               0.023414703432404593, 0.06248365429859781, 385.10196906188503,
               6.003313225070965e-8, 0.000274026861750043, 0.0007433951467703537]
RTOL = math.sqrt(np.finfo(np.float64).eps)


def test_oracle_rainy_convergence_golden(orc):
    c = orc.Rainy2D(3, 6, 6, 0.0, 2.0, 0.0, 2.0, True, True, weak_form=True, source_kind=1)
    u = c.initial_condition_convergence(0.0)
    t = c.ck_steps(u, np.zeros_like(u), 0.0, 1.0, 100000, 0.0, 0, 1e-8, 20, 2.0)
    assert abs(t - 2.0) < 1e-14
    l2, linf = c.errors_convergence(u, t)
    for v in range(9):
        assert abs(l2[v] - GOLDEN_L2[v]) <= RTOL * GOLDEN_L2[v], (v, l2[v], GOLDEN_L2[v])
        assert abs(linf[v] - GOLDEN_LINF[v]) <= RTOL * GOLDEN_LINF[v], (v, linf[v], GOLDEN_LINF[v])


def test_rainy_ec_flux_consistency(orc):
    """flux_ec_rain(u, u, n) == flux(u, n) (test/test_unit.jl:526-544 checks
    the same identity, marking the energy component as not required)."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        rd = rng.uniform(0.5, 1.2)
        rv = rng.uniform(1e-3, 2e-2)
        rc = rng.uniform(0, 1e-3)
        rr = rng.uniform(1e-6, 1e-3)
        T = rng.uniform(250, 300)
        v = rng.uniform(-20, 20, 2)
        rho = rd + rv + rc + rr
        E = (717 * rd + 1424 * rv + 4186 * (rc + rr)) * T + rv * 2.5e6 + 0.5 * rho * (v @ v)
        u = np.array([rd, rv + rc, rr, rho * v[0], rho * v[1], E, rv, rc, T])
        n = rng.uniform(-1, 1, 2)
        fe, f = orc.rainy_flux_ec(u, u, n), orc.rainy_flux(u, n)
        assert np.allclose(fe[:5], f[:5], rtol=1e-12, atol=1e-12 * np.abs(f).max())


def test_rainy_newton_recovers_saturation_state(orc):
    """Newton from a perturbed guess returns the equilibrium partition."""
    c = orc.Rainy2D(1, 1, 1, 0.0, 1.0, 0.0, 1.0, True, True)
    rng = np.random.default_rng(5)
    u = np.zeros((1, 2, 2, 9))
    for q in np.ndindex(1, 2, 2):
        T = rng.uniform(260, 295)
        rd = rng.uniform(0.8, 1.2)
        rm = rng.uniform(5e-3, 2e-2)
        rr = rng.uniform(0, 1e-3)
        u[q][:3] = (rd, rm, rr)
        u[q][5] = (717 * rd + 1424 * rm + 4186 * rr) * T + rm * 2.5e6
        u[q][6:] = (0.5 * rm, 0.5 * rm, T + 5.0)
    tot, iters, nfail = c.newton(u, mode=1, tol=1e-12, maxit=30)
    assert nfail == 0 and iters.max() < 30
    e_s = np.vectorize(orc.lib().orc_rainy_saturation_vapour_pressure)(u[..., 8])
    rv_sat = np.minimum(e_s / (461.0 * u[..., 8]), u[..., 1])
    assert np.allclose(u[..., 6], rv_sat, rtol=1e-10)
    assert np.allclose(u[..., 6] + u[..., 7], u[..., 1], rtol=1e-12)
