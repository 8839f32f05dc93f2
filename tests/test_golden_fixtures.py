"""The golden vectors the oracle and GPU tests check against are the
reference's own: every constant below equals the l2 / linf arrays of the
named testset in tests/golden/reference_goldens.json, which
tests/golden/extract_goldens.py extracted from the reference's test/*.jl
(CPU only)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = json.load(open(os.path.join(HERE, "golden", "reference_goldens.json")))


def _cases():
    import test_oracle_cov_swe as cov
    import test_oracle_golden as e2
    import test_oracle_golden_3d as e3
    import test_oracle_moist as moist
    import test_oracle_pt as pt
    import test_oracle_rainy as rainy
    c = "test/test_2d_shallow_water_covariant.jl:"
    return {
        "test/test_2d_euler_energy.jl:7 elixir_energy_inertia_gravity_waves":
            (e2.GOLDEN_L2, e2.GOLDEN_LINF),
        "test/test_3d_euler_energy.jl:7 elixir_energy_baroclinic_instability":
            (e3.GOLDEN_L2, e3.GOLDEN_LINF),
        "test/test_2d_rainy_euler.jl:7 convergence_test": (rainy.GOLDEN_L2, rainy.GOLDEN_LINF),
        "test/test_2d_rainy_euler.jl:42 elixir_hoeck_bubble moist": rainy.HOECK_MOIST,
        "test/test_2d_moist_euler.jl:7 elixir_gemein_bubble dry": moist.DRY_BUBBLE,
        "test/test_2d_moist_euler.jl:32 elixir_gemein_bubble moist": moist.MOIST_BUBBLE,
        "test/test_2d_moist_euler.jl:59 elixir_gemein_nonhydrostatic_gravity_waves":
            moist.NONHYDROSTATIC_GRAVITY_WAVES,
        "test/test_2d_moist_euler.jl:86 elixir_gemein_source_terms dry": moist.DRY_SOURCE,
        "test/test_2d_moist_euler.jl:113 elixir_gemein_source_terms moist": moist.MOIST_SOURCE,
        c + "7 elixir_geostrophic_balance": cov.GOLDEN["geostrophic_balance"],
        c + "28 elixir_rossby_haurwitz": cov.GOLDEN["rossby_haurwitz"],
        c + "42 elixir_isolated_mountain": cov.GOLDEN["isolated_mountain"],
        c + "55 elixir_unsteady_solid_body_rotation_EC": cov.GOLDEN["unsteady_solid_body_rotation"],
        c + "78 elixir_barotropic_instability": cov.GOLDEN["barotropic_instability"],
        c + "91 elixir_well_balanced": cov.GOLDEN["well_balanced"],
        "test/test_2d_potential_temperature.jl:7 elixir_potential_temperature_inertia_gravity_waves":
            (pt.GOLDEN_L2, pt.GOLDEN_LINF),
        "test/test_2d_potential_temperature.jl:29 elixir_potential_temperature_linear_hydrostatic":
            pt.MOUNTAIN["linear_hydrostatic"]["golden"],
        "test/test_2d_potential_temperature.jl:53 elixir_potential_temperature_linear_nonhydrostatic":
            pt.MOUNTAIN["linear_nonhydrostatic"]["golden"],
        "test/test_2d_potential_temperature.jl:76 elixir_potential_temperature_schaer_mountain":
            pt.MOUNTAIN["schaer_mountain"]["golden"],
        "test/test_2d_potential_temperature.jl:100 elixir_potential_temperature_well_balanced_curvilinear":
            pt.WELL_BALANCED["default"][1:],
        "test/test_2d_potential_temperature.jl:122 elixir_potential_temperature_well_balanced_curvilinear":
            pt.WELL_BALANCED["ec_surface"][1:],
    }


def test_every_golden_constant_is_the_reference_vector():
    cases = _cases()
    assert len(cases) == 21
    for key, (l2, linf) in cases.items():
        assert key in FIXTURES, key
        ref = FIXTURES[key]
        assert np.array_equal(np.asarray(l2, dtype=float), np.asarray(ref["l2"])), key
        assert np.array_equal(np.asarray(linf, dtype=float), np.asarray(ref["linf"])), key
