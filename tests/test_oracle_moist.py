"""Pins the moist-Euler oracle against the reference's golden vectors (CPU only).

test/test_2d_moist_euler.jl:
  * "elixir_gemein_bubble dry" (:7-30): examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl,
    CompressibleMoistEulerEquations2D without moisture, flux_chandrashekar /
    FluxLMARS(360), source_terms_geopotential, pressure-Riemann slip walls,
    P4estMesh of 2x2 trees refined 5 times (64x64 affine elements over
    [0, 20 km] x [-5 km, 15 km]), polydeg 4, CK2N54 at CFL 0.2 to t = 0.1;
  * "elixir_gemein_source_terms moist" (:152-177): examples/euler/moist_air/tests/
    elixir_gemein_source_terms.jl with polydeg 3 and 10x8 cells, flux_chandrashekar
    as volume and surface flux, the moist convergence source (phase change);
  * "elixir_gemein_source_terms dry" (:126-150): examples/euler/dry_air/tests/
    elixir_gemein_source_terms.jl, weak form, flux_lax_friedrichs, gravity 0.
Tolerances are Trixi's @test_trixi_include defaults (atol 500 eps, rtol sqrt(eps)).
The P4estMesh of the first test is affine, so the StructuredMesh of the same
64x64 elements with outward-normal wall semantics has the same nodes, metric
terms and boundary fluxes; the error norms do not depend on element order.
Only the last bits of the node coordinates differ (P4est interpolates each
quadrant's nodes from its tree's corners); the energy linf, an O(0.1)
difference of O(2e5) energies, magnifies that to 1.7e-8 relative, so that case
is checked at rtol 5e-8.
"""
import math

import numpy as np
import pytest

ATOL = 500 * np.finfo(np.float64).eps
RTOL = math.sqrt(np.finfo(np.float64).eps)

DRY_BUBBLE = ([9.104437114458848e-7, 1.8210536975490044e-5, 0.0004707887343135412,
               0.0063400898518523935, 0.0, 0.0],
              [1.0258941581242631e-5, 0.00020520634691933992, 0.006392782691233334,
               0.07637640493339859, 0.0, 0.0])
MOIST_SOURCE = ([0.0001480393714768623, 0.11945481031503036, 0.07460345535073129,
                 5.9430508465000385, 4.471792794168725e-9, 7.10320253652373e-10],
                [0.0007084175808387272, 0.504796333566, 0.3697160820183014,
                 27.843165651072923, 2.1168438904322837e-8, 3.691699932047233e-9])
DRY_SOURCE = ([1.3992076791281227e-5, 1.4486417486907815e-5, 2.609465609739115e-5,
               6.323484379066432e-5, 0.0, 0.0],
              [7.549984224430872e-5, 0.00010065352517929504, 0.00015964938767742964,
               0.0005425860570698049, 0.0, 0.0])

# (constructor arguments, CFL, golden)
CASES = {
    "dry_bubble": (dict(polydeg=4, nx=64, ny=64, x0=0.0, x1=20000.0, y0=-5000.0, y1=15000.0,
                        periodic_x=True, periodic_y=False, surface_kind=0, source_kind=1,
                        wall_kind=2, c_lmars=360.0, ic_kind=0), 0.2, DRY_BUBBLE),
    "moist_source": (dict(polydeg=3, nx=10, ny=8, x0=0.0, x1=2.0, y0=0.0, y1=2.0,
                          periodic_x=True, periodic_y=True, surface_kind=2, source_kind=4,
                          ic_kind=2), 1.0, MOIST_SOURCE),
    "dry_source": (dict(polydeg=3, nx=10, ny=8, x0=0.0, x1=2.0, y0=0.0, y1=2.0,
                        periodic_x=True, periodic_y=True, weak_form=True, surface_kind=1,
                        source_kind=3, gravity=0.0, ic_kind=1), 1.0, DRY_SOURCE),
}


def close(a, b, rtol=RTOL):
    return abs(a - b) <= max(ATOL, rtol * max(abs(a), abs(b)))


def check_golden(l2, linf, golden, rtol=RTOL):
    for v in range(6):
        assert close(l2[v], golden[0][v], rtol), ("l2", v, l2[v], golden[0][v])
        assert close(linf[v], golden[1][v], rtol), ("linf", v, linf[v], golden[1][v])


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_moist_golden(orc, name):
    kw, cfl, golden = CASES[name]
    c = orc.Moist2D(**kw)
    u = c.initial_condition()
    t = c.ck_steps(u, np.zeros_like(u), 0.0, cfl, 100000, 0.0, 0.1)
    assert abs(t - 0.1) < 1e-15
    l2, linf = c.errors(u, t)
    check_golden(l2, linf, golden, 5e-8 if name == "dry_bubble" else RTOL)


def test_chandrashekar_consistency(orc):
    """flux_chandrashekar(u, u, n) == flux(u, n) (test/test_unit.jl checks the
    same consistency for the moist fluxes)."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        rho = rng.uniform(0.5, 1.3)
        qv, ql = rng.uniform(0, 0.02), rng.uniform(0, 0.002)
        v = rng.uniform(-30, 30, 2)
        T = rng.uniform(250, 300)
        mu = (1 - qv - ql) * 717.0 + qv * 1424.0 + ql * 4186.0
        E = rho * (mu * T + qv * 3147620.0) + 0.5 * rho * (v ** 2).sum()
        u = np.array([rho, rho * v[0], rho * v[1], E, rho * qv, rho * ql])
        n = rng.normal(size=2)
        f = orc.moist_flux(u, n)
        fe = orc.moist_flux_chandrashekar(u, u, n)
        assert np.allclose(fe, f, rtol=1e-12, atol=1e-12 * np.abs(f).max())
