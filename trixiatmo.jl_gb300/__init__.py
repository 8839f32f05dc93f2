"""trixiatmo_gb300 — GB300-native (sm_103a, FP64) DGSEM `rhs!` for TrixiAtmo.jl.

The hot path is libtrixiatmo_gpu.so (CUDA kernels behind the C ABI in
include/trixiatmo_gpu.h).  This package is the host-side mirror of the
reference's Julia API for that path, used by the tests and the benchmark.
The directory name is not a Python identifier; load it with
``load_package()`` from ``__graft_entry__`` (or importlib) under the name
``trixiatmo_gb300``.
"""
from . import _lib, covariant, learned_guess, output, trixi_connectivity
from .basis import LobattoLegendreBasis
from .equations import (CompressibleEulerEnergyEquationsWithGravity2D,
                        CompressibleEulerEnergyEquationsWithGravity3D,
                        CompressibleRainyEulerEquations2D, VolumeIntegralWeakForm,
                        boundary_condition_simple_slip_wall, flux_ec_rain, flux_lax_friedrichs,
                        source_terms_convergence_test_rainy, source_terms_rainy, FluxLMARS,
                        VolumeIntegralFluxDifferencing, boundary_condition_periodic,
                        boundary_condition_slip_wall, flux_nonconservative_waruszewski_etal,
                        flux_ranocha, flux_zero, speed_of_sound_isothermal,
                        CompressibleMoistEulerEquations2D, flux_chandrashekar,
                        source_terms_geopotential, source_terms_moist_bubble,
                        source_terms_convergence_test_dry, source_terms_convergence_test_moist,
                        source_terms_nonhydrostatic_gravity_wave, flux_LMARS,
                        source_terms_no_phase_change,
                        CompressibleEulerPotentialTemperatureEquationsWithGravity2D,
                        CompressibleEulerPotentialTemperatureEquationsWithGravity3D,
                        CompressibleEulerInternalEnergyEquationsWithGravity2D,
                        flux_conservative_etec, flux_nonconservative_etec,
                        flux_conservative_es, flux_nonconservative_es, flux_ec,
                        flux_tec, flux_etec, flux_kennedy_gruber,
                        flux_kennedy_gruber_souza_etal, flux_lmars_combined,
                        flux_nonconservative_artiano_etal,
                        flux_nonconservative_souza_etal)
from .initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION, EARTH_RADIUS,
                                 EARTH_ROTATION_RATE, SMALL_EARTH_RADIUS,
                                 SMALL_EARTH_ROTATION_RATE, SMALL_EARTH_SCALING,
                                 initial_condition_vortex_shedding,
                                 AtmosphereLayersRainyBubble, initial_condition_bubble_rainy,
                                 IsothermalShell, MoistBubbleRainy,
                                 WarmBubble, initial_condition_convergence_test_rainy,
                                 initial_condition_baroclinic_instability,
                                 initial_condition_gravity_waves, seeded_perturbation,
                                 initial_condition_adiabatic,
                                 initial_condition_gemein_bubble,
                                 initial_condition_convergence_test_dry,
                                 initial_condition_convergence_test_moist,
                                 initial_condition_nonhydrostatic_gravity_wave,
                                 AtmosphereLayers, initial_condition_moist_bubble)
from .meshes import (P4estMesh, SchaerMountain, SchärMountain, StructuredMesh, WitchOfAgnesi,
                     terrain_following_faces)
from .equations import BoundaryConditionDirichlet
from .initial_conditions import MountainWaveSetup
from .meshes3d import GalChen, P4estMeshCubedSphereTopography, Sleve
from .output import (convert_variables, cons2cons, cons2prim, cons2prim_and_vorticity,
                     contravariant2global, save_solution_file, varnames)
from .semidiscretization import (DGSEM, SemidiscretizationCovariant,
                                 SemidiscretizationCovariantEnsemble, SemidiscretizationEnsemble,
                                 SemidiscretizationHyperbolic, fp64_peak, source_terms_coriolis,
                                 source_terms_coriolis_small_earth)

__all__ = [
    "LobattoLegendreBasis", "CompressibleEulerEnergyEquationsWithGravity2D", "FluxLMARS",
    "VolumeIntegralFluxDifferencing", "boundary_condition_periodic",
    "boundary_condition_slip_wall", "flux_nonconservative_waruszewski_etal", "flux_ranocha",
    "flux_zero", "speed_of_sound_isothermal", "WarmBubble", "initial_condition_gravity_waves",
    "seeded_perturbation", "StructuredMesh", "DGSEM", "SemidiscretizationHyperbolic",
    "SemidiscretizationEnsemble", "CompressibleEulerEnergyEquationsWithGravity3D",
    "EARTH_GRAVITATIONAL_ACCELERATION", "EARTH_RADIUS", "EARTH_ROTATION_RATE", "IsothermalShell",
    "initial_condition_baroclinic_instability", "P4estMeshCubedSphereTopography",
    "source_terms_coriolis", "source_terms_coriolis_small_earth", "SMALL_EARTH_RADIUS",
    "SMALL_EARTH_ROTATION_RATE", "SMALL_EARTH_SCALING", "initial_condition_vortex_shedding",
    "AtmosphereLayersRainyBubble", "initial_condition_bubble_rainy",
    "fp64_peak", "CompressibleRainyEulerEquations2D",
    "VolumeIntegralWeakForm", "boundary_condition_simple_slip_wall", "flux_ec_rain",
    "flux_lax_friedrichs", "source_terms_convergence_test_rainy", "source_terms_rainy",
    "MoistBubbleRainy", "initial_condition_convergence_test_rainy", "learned_guess",
    "CompressibleMoistEulerEquations2D", "flux_chandrashekar", "source_terms_geopotential",
    "source_terms_moist_bubble", "source_terms_convergence_test_dry",
    "source_terms_convergence_test_moist", "initial_condition_gemein_bubble",
    "initial_condition_convergence_test_dry", "initial_condition_convergence_test_moist",
    "P4estMesh", "covariant", "SemidiscretizationCovariant", "initial_condition_adiabatic",
    "SemidiscretizationCovariantEnsemble", "source_terms_nonhydrostatic_gravity_wave",
    "initial_condition_nonhydrostatic_gravity_wave", "AtmosphereLayers",
    "initial_condition_moist_bubble", "flux_LMARS", "source_terms_no_phase_change",
    "SchaerMountain", "SchärMountain", "WitchOfAgnesi", "terrain_following_faces",
    "BoundaryConditionDirichlet", "MountainWaveSetup", "GalChen", "Sleve",
    "CompressibleEulerPotentialTemperatureEquationsWithGravity2D",
    "CompressibleEulerPotentialTemperatureEquationsWithGravity3D",
    "CompressibleEulerInternalEnergyEquationsWithGravity2D", "flux_conservative_etec",
    "flux_nonconservative_etec", "flux_conservative_es", "flux_nonconservative_es",
    "flux_ec", "flux_tec",
    "flux_etec", "flux_nonconservative_artiano_etal", "flux_nonconservative_souza_etal",
    "flux_kennedy_gruber", "flux_kennedy_gruber_souza_etal", "flux_lmars_combined",
    "trixi_connectivity", "output", "save_solution_file", "convert_variables", "varnames",
    "cons2cons", "cons2prim", "contravariant2global", "cons2prim_and_vorticity",
]
