"""Pins the CPU oracle against the reference's own golden vectors (CPU only).

The reference test test/test_2d_euler_energy.jl:7-27 runs
examples/euler/dry_air/buoyancy/elixir_energy_inertia_gravity_waves.jl to
t = 10 s (StructuredMesh 60x8, polydeg 3, flux_ranocha + waruszewski volume
flux, (FluxLMARS(c_s), flux_zero) surface flux, slip walls in z, SSPRK43 with
adaptive = false and CFL 1.0) and compares end-of-run l2/linf errors with
atol = 5e-11 and Julia's default rtol = sqrt(eps).
"""
import math

import numpy as np
import pytest

GOLDEN_L2 = [2.3800999105272615e-7, 6.190703408721927e-6, 3.3821288686132935e-5,
             0.04382810097184301, 9.251160452856857e-12]
GOLDEN_LINF = [1.2362858294867607e-6, 6.0616987290984525e-5, 0.00033470830315131473,
               0.27272386016556993, 4.3655745685100555e-11]
ATOL = 5e-11
RTOL = math.sqrt(np.finfo(np.float64).eps)


def _isapprox(a, b):
    # Julia isapprox: |a - b| <= max(atol, rtol * max(|a|, |b|))
    return abs(a - b) <= max(ATOL, RTOL * max(abs(a), abs(b)))


def igw_case(orc):
    cp, cv = 1004.0, 717.0
    cs = math.sqrt(cp / cv * (cp - cv) * 250.0)
    return orc.Euler2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, cp, cv, 9.81, cs)


def test_oracle_inertia_gravity_waves_golden(orc):
    c = igw_case(orc)
    u = c.initial_condition(0)
    steps = c.ssprk43_run(u, 0.0, 10.0, 1.0)
    assert steps > 0
    l2, linf = c.errors_gravity_waves(u)
    for v in range(5):
        assert _isapprox(l2[v], GOLDEN_L2[v]), (v, l2[v], GOLDEN_L2[v])
        assert _isapprox(linf[v], GOLDEN_LINF[v]), (v, linf[v], GOLDEN_LINF[v])
    # the physical components agree far better than the test tolerance
    rel = np.abs(l2[:4] - GOLDEN_L2[:4]) / np.asarray(GOLDEN_L2[:4])
    assert rel.max() < 1e-7


def test_oracle_well_posed_hydrostatic_rest(orc):
    """A hydrostatic state at rest with the well-balanced nonconservative term:
    the oracle's rhs is small compared with the individual flux terms."""
    c = orc.Euler2D(3, 8, 4, 0.0, 20000.0, 0.0, 10000.0, True, False, 1004.0, 717.0, 9.81, 340.0)
    u = c.initial_condition(1, (10000.0, 2000.0, 2000.0, 0.0, 0.0))  # no bubble
    du = c.rhs(u)
    assert np.all(np.isfinite(du))
    # momentum tendency relative to the gravity term rho*g
    assert np.abs(du[..., 2]).max() < 1e-3 * np.abs(u[..., 0] * 9.81).max()


@pytest.mark.parametrize("polydeg", [1, 2, 3, 4, 5, 7])
def test_oracle_basis_exactness(orc, tg, polydeg):
    """LGL quadrature integrates degree 2N-1 exactly; D differentiates degree N
    exactly; host mirror and oracle agree bitwise."""
    b = tg.LobattoLegendreBasis(polydeg)
    x, w = b.nodes, b.weights
    for k in range(2 * polydeg):
        exact = (1 - (-1) ** (k + 1)) / (k + 1)
        assert abs(np.dot(w, x ** k) - exact) < 1e-14
    for k in range(polydeg + 1):
        assert np.abs(b.derivative_matrix @ x ** k - k * x ** max(k - 1, 0) * (k > 0)).max() < 1e-12
    o = orc.Euler2D(polydeg, 2, 2, 0.0, 1.0, 0.0, 1.0, True, True)
    xo, wo, Do, Dso = o.basis()
    assert np.array_equal(xo, x) and np.array_equal(wo, w)
    assert np.allclose(Do, b.derivative_matrix, rtol=0, atol=1e-13)
    assert np.allclose(Dso, b.derivative_split, rtol=0, atol=1e-13)
    # diagonal of the split operator vanishes (Dsplit[i,i] = 0 up to rounding)
    assert np.abs(np.diag(b.derivative_split)).max() < 1e-12
