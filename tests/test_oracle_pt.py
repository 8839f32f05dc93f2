"""Pins the potential-temperature oracle against the reference's golden
vector (CPU only): test/test_2d_potential_temperature.jl:7-27 runs
examples/euler/dry_air/buoyancy/elixir_potential_temperature_inertia_gravity_waves.jl
(StructuredMesh 60x8 over 300 km x 10 km, polydeg 3, (flux_tec,
flux_nonconservative_waruszewski_etal) / (FluxLMARS(sqrt(gamma R 250)), flux_zero),
slip walls in z, SSPRK43 at CFL 1 without adaptivity) to t = 1800 s and compares
with atol 1e-5.  The oracle's l2/linf agree with the golden to 3e-4 .. 1.1e-3
relative (far inside that test's tolerance); the Stolarsky mean is checked
against its definition in extended precision."""
import math

import numpy as np
import pytest

GOLDEN_L2 = [5.360162314066379e-7, 0.00013097436752903342, 7.172813096420895e-5,
             3.560199562542724e-5, 9.251160452856857e-12]
GOLDEN_LINF = [3.7348732354614e-6, 0.0005402594042358544, 0.00023237719913361634,
               0.00015331821185782246, 4.3655745685100555e-11]
ATOL = 1e-5
RTOL = math.sqrt(np.finfo(np.float64).eps)


def test_oracle_pt_gravity_waves_golden(orc):
    c = orc.PotTemp2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False, volume=0, nc=0,
                      wall_kind=1, c_lmars=math.sqrt(1004 / 717 * 287 * 250))
    u = c.initial_condition_gravity_waves()
    c.ssprk43_run(u, 0.0, 1800.0, 1.0)
    l2, linf = c.errors_gravity_waves(u)
    for v in range(5):
        assert abs(l2[v] - GOLDEN_L2[v]) <= max(ATOL, RTOL * GOLDEN_L2[v])
        assert abs(linf[v] - GOLDEN_LINF[v]) <= max(ATOL, RTOL * GOLDEN_LINF[v])
    # far tighter than the test's atol: the physical variables within 2e-3
    for v in range(4):
        assert abs(l2[v] / GOLDEN_L2[v] - 1) < 2e-3, v
        assert abs(linf[v] / GOLDEN_LINF[v] - 1) < 2e-3, v


def test_stolarsky_mean_against_definition(orc):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    g = mp.mpf(1004) / 717
    for x, y in [(1.0, 1.0), (1.0, 1.0001), (1.0, 1.05), (1.0, 1.099), (1.0, 1.3), (0.5, 2.0)]:
        got = orc.stolarsky(x, y, 1004 / 717)
        if x == y:
            assert got == x
            continue
        ex = (g - 1) / g * (mp.mpf(y) ** g - mp.mpf(x) ** g) / (mp.mpf(y) ** (g - 1) - mp.mpf(x) ** (g - 1))
        assert abs(got - float(ex)) <= 2e-15 * float(ex), (x, y)
