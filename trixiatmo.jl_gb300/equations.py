"""Equation, flux and boundary-condition descriptors of the host mirror.

They carry the parameters and identifiers the C ABI needs; all arithmetic on
the solution happens in the CUDA kernels.  Names follow TrixiAtmo/Trixi:
`CompressibleEulerEnergyEquationsWithGravity2D`
(src/equations/compressible_euler_energy_with_gravity_2d.jl:40-60),
`flux_ranocha` (:366), `flux_nonconservative_waruszewski_etal` (:186),
`FluxLMARS` (:397), `flux_zero`, `boundary_condition_slip_wall` (:77, :102).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib


class CompressibleEulerEnergyEquationsWithGravity2D:
    """State (rho, rho_v1, rho_v2, rho_e, phi); rho_e total energy w/o potential."""

    nvariables = 5
    ndims = 2
    eq_id = _lib.TAG_EQ_EULER_ENERGY_2D

    def __init__(self, *, c_p, c_v, gravity):
        self.c_p = float(c_p)
        self.c_v = float(c_v)
        self.g = float(gravity)
        self.R = self.c_p - self.c_v
        self.gamma = self.c_p / self.c_v
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)
        self.p_0 = 100000.0

    # host-side conversions used to build initial states (compute_coefficients!)
    def prim2cons(self, rho, v1, v2, p, phi):
        rv1, rv2 = rho * v1, rho * v2
        return np.stack([rho * np.ones_like(p), rv1 * np.ones_like(p), rv2 * np.ones_like(p),
                         p * self.inv_gamma_minus_one + 0.5 * (rv1 * v1 + rv2 * v2),
                         phi * np.ones_like(p)], axis=-1)

    def cons2prim(self, u):
        rho = u[..., 0]
        v1 = u[..., 1] / rho
        v2 = u[..., 2] / rho
        p = (self.gamma - 1.0) * (u[..., 3] - 0.5 * (u[..., 1] * v1 + u[..., 2] * v2))
        return rho, v1, v2, p, u[..., 4]


class CompressibleEulerPotentialTemperatureEquationsWithGravity2D:
    """State (rho, rho_v1, rho_v2, rho_theta, phi), p = K rho_theta^gamma
    (src/equations/compressible_euler_potential_temperature_gravity_2d.jl:5-33)."""

    nvariables = 5
    ndims = 2
    eq_id = _lib.TAG_EQ_POTENTIAL_TEMPERATURE_2D

    def __init__(self, *, c_p, c_v, gravity):
        self.c_p = float(c_p)
        self.c_v = float(c_v)
        self.g = float(gravity)
        self.p_0 = 100000.0
        self.R = self.c_p - self.c_v
        self.gamma = self.c_p / self.c_v
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)
        self.K = self.p_0 * (self.R / self.p_0) ** self.gamma

    def prim2cons(self, rho, v1, v2, p, phi):
        one = np.ones_like(p)
        rho_theta = (p / self.p_0) ** (1 / self.gamma) * self.p_0 / self.R
        return np.stack([rho * one, rho * v1 * one, rho * v2 * one, rho_theta * one, phi * one],
                        axis=-1)

    def cons2prim(self, u):
        rho = u[..., 0]
        return rho, u[..., 1] / rho, u[..., 2] / rho, self.K * u[..., 3] ** self.gamma, u[..., 4]


class CompressibleEulerPotentialTemperatureEquationsWithGravity3D:
    """State (rho, rho_v1, rho_v2, rho_v3, rho_theta, phi), p = K rho_theta^gamma
    (src/equations/compressible_euler_potential_temperature_gravity_3d.jl:42-66)."""

    nvariables = 6
    ndims = 3
    eq_id = _lib.TAG_EQ_POTENTIAL_TEMPERATURE_3D

    def __init__(self, *, c_p, c_v, gravity):
        self.c_p = float(c_p)
        self.c_v = float(c_v)
        self.g = float(gravity)
        self.p_0 = 100000.0
        self.R = self.c_p - self.c_v
        self.gamma = self.c_p / self.c_v
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)
        self.K = self.p_0 * (self.R / self.p_0) ** self.gamma

    def prim2cons(self, rho, v1, v2, v3, p, phi):
        """:535-543: rho_theta = (p / K)^(1 / gamma)."""
        one = np.ones_like(p)
        rho_theta = (p / self.K) ** (1 / self.gamma)
        return np.stack([rho * one, rho * v1 * one, rho * v2 * one, rho * v3 * one,
                         rho_theta * one, phi * one], axis=-1)

    def cons2prim(self, u):
        rho = u[..., 0]
        return (rho, u[..., 1] / rho, u[..., 2] / rho, u[..., 3] / rho,
                self.K * u[..., 4] ** self.gamma, u[..., 5])


class CompressibleEulerInternalEnergyEquationsWithGravity2D:
    """State (rho, rho_v1, rho_v2, rho_e_internal, phi), p = (gamma - 1) rho_e_internal
    (src/equations/compressible_euler_internal_energy_with_gravity_2d.jl:42-62)."""

    nvariables = 5
    ndims = 2
    eq_id = _lib.TAG_EQ_INTERNAL_ENERGY_2D

    def __init__(self, *, c_p, c_v, gravity):
        self.c_p = float(c_p)
        self.c_v = float(c_v)
        self.g = float(gravity)
        self.p_0 = 100000.0
        self.R = self.c_p - self.c_v
        self.gamma = self.c_p / self.c_v
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)

    def prim2cons(self, rho, v1, v2, p, phi):
        """:248-255."""
        one = np.ones_like(p)
        return np.stack([rho * one, rho * v1 * one, rho * v2 * one,
                         p * self.inv_gamma_minus_one * one, phi * one], axis=-1)

    def cons2prim(self, u):
        rho = u[..., 0]
        return rho, u[..., 1] / rho, u[..., 2] / rho, (self.gamma - 1.0) * u[..., 3], u[..., 4]


class CompressibleEulerEnergyEquationsWithGravity3D:
    """State (rho, rho_v1, rho_v2, rho_v3, rho_e, phi)
    (src/equations/compressible_euler_energy_with_gravity_3d.jl:45-65)."""

    nvariables = 6
    ndims = 3
    eq_id = _lib.TAG_EQ_EULER_ENERGY_3D

    def __init__(self, *, c_p, c_v, gravity):
        self.c_p = float(c_p)
        self.c_v = float(c_v)
        self.g = float(gravity)
        self.R = self.c_p - self.c_v
        self.gamma = self.c_p / self.c_v
        self.inv_gamma_minus_one = 1.0 / (self.gamma - 1.0)
        self.p_0 = 100000.0

    def prim2cons(self, rho, v1, v2, v3, p, phi):
        one = np.ones_like(p)
        return np.stack([rho * one, rho * v1 * one, rho * v2 * one, rho * v3 * one,
                         p * self.inv_gamma_minus_one + 0.5 * rho * (v1 * v1 + v2 * v2 + v3 * v3),
                         phi * one], axis=-1)

    def cons2prim(self, u):
        rho = u[..., 0]
        v1, v2, v3 = u[..., 1] / rho, u[..., 2] / rho, u[..., 3] / rho
        p = (self.gamma - 1.0) * (u[..., 4] - 0.5 * (u[..., 1] * v1 + u[..., 2] * v2 +
                                                     u[..., 3] * v3))
        return rho, v1, v2, v3, p, u[..., 5]


class CompressibleRainyEulerEquations2D:
    """State (rho_dry, rho_moist, rho_rain, rho_v1, rho_v2, energy, rho_vapour,
    rho_cloud, temperature) (src/equations/compressible_rainy_euler_2d.jl:49-110);
    slots 7-9 solve the saturation system (Newton stage limiter)."""

    nvariables = 9
    ndims = 2
    eq_id = _lib.TAG_EQ_RAINY_2D
    c_l, c_pd, c_vd, c_pv, c_vv = 4186.0, 1004.0, 717.0, 1885.0, 1424.0
    R_d, R_v = 287.0, 461.0
    ref_saturation_pressure, ref_temperature = 610.7, 273.15
    ref_latent_heat_vap_temp, ref_pressure = 2500000.0, 100000.0
    gravity = 9.80616

    def saturation_vapour_pressure(self, T):
        """:397-419 (Clausius-Clapeyron)."""
        e = self.ref_saturation_pressure * (T / self.ref_temperature) ** (
            (self.c_pv - self.c_l) / self.R_v)
        return e * np.exp(((self.ref_latent_heat_vap_temp - (self.c_pv - self.c_l) *
                            self.ref_temperature) / self.R_v) *
                          (1.0 / self.ref_temperature - 1.0 / T))


class CompressibleMoistEulerEquations2D:
    """State (rho, rho_v1, rho_v2, rho_E, rho_qv, rho_ql)
    (src/equations/compressible_moist_euler_2d.jl:5-32); gravity enters
    through source_terms_geopotential."""

    nvariables = 6
    ndims = 2
    eq_id = _lib.TAG_EQ_MOIST_EULER_2D

    def __init__(self, *, c_pd, c_vd, c_pv, c_vv, gravity):
        self.c_pd, self.c_vd = float(c_pd), float(c_vd)
        self.c_pv, self.c_vv = float(c_pv), float(c_vv)
        self.g = float(gravity)
        self.p_0 = 100000.0
        self.R_d = self.c_pd - self.c_vd
        self.R_v = self.c_pv - self.c_vv
        self.c_pl = 4186.0
        self.gamma = self.c_pd / self.c_vd
        self.kappa = 1.0 - 1.0 / self.gamma
        self.L_00 = 3147620.0

    def get_current_condition(self, u):
        """(p, T) of states u[..., 6] (:383-402)."""
        rho_qd = u[..., 0] - u[..., 4] - u[..., 5]
        rho_e = u[..., 3] - 0.5 * (u[..., 1] ** 2 + u[..., 2] ** 2) / u[..., 0]
        T = (rho_e - self.L_00 * u[..., 4]) / (rho_qd * self.c_vd + u[..., 4] * self.c_vv +
                                                u[..., 5] * self.c_pl)
        return (rho_qd * self.R_d + u[..., 4] * self.R_v) * T, T


class _NamedFlux:
    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return self.name


flux_ranocha = _NamedFlux("flux_ranocha")
flux_nonconservative_waruszewski_etal = _NamedFlux("flux_nonconservative_waruszewski_etal")
flux_zero = _NamedFlux("flux_zero")
flux_ec_rain = _NamedFlux("flux_ec_rain")
flux_lax_friedrichs = _NamedFlux("flux_lax_friedrichs")
# the rainy equations' own LMARS (src/equations/compressible_rainy_euler_2d.jl:817-861,
# speed of sound 360)
flux_LMARS = _NamedFlux("flux_LMARS")
flux_chandrashekar = _NamedFlux("flux_chandrashekar")
# entropy / total-energy conservative fluxes; flux_ec is shared with the
# covariant shallow-water equations (the reference dispatches one name on the
# equation type)
flux_ec = _NamedFlux("flux_ec")
flux_tec = _NamedFlux("flux_tec")
# CompressibleEulerInternalEnergyEquationsWithGravity2D (:110-246)
flux_conservative_etec = _NamedFlux("flux_conservative_etec")
flux_nonconservative_etec = _NamedFlux("flux_nonconservative_etec")
flux_conservative_es = _NamedFlux("flux_conservative_es")
flux_nonconservative_es = _NamedFlux("flux_nonconservative_es")
flux_etec = _NamedFlux("flux_etec")
flux_nonconservative_artiano_etal = _NamedFlux("flux_nonconservative_artiano_etal")
flux_nonconservative_souza_etal = _NamedFlux("flux_nonconservative_souza_etal")
# CompressibleEulerPotentialTemperatureEquationsWithGravity3D
# (src/equations/compressible_euler_potential_temperature_gravity_3d.jl):
# flux_kennedy_gruber (:333-359); the fused flux_kennedy_gruber_souza_etal
# (:377-414), which equals (flux_kennedy_gruber, flux_nonconservative_souza_etal);
# the fused surface flux flux_lmars_combined (:258-293), which equals
# (FluxLMARS(340), flux_zero), and its slip wall (:299-320), the one of the tuple
flux_kennedy_gruber = _NamedFlux("flux_kennedy_gruber")
flux_kennedy_gruber_souza_etal = _NamedFlux("flux_kennedy_gruber_souza_etal")
flux_lmars_combined = _NamedFlux("flux_lmars_combined")


class FluxLMARS:
    """Low Mach number approximate Riemann solver with a fixed speed of sound."""

    def __init__(self, speed_of_sound):
        self.speed_of_sound = float(speed_of_sound)

    def __repr__(self):
        return f"FluxLMARS({self.speed_of_sound})"


class VolumeIntegralFluxDifferencing:
    def __init__(self, volume_flux):
        self.volume_flux = volume_flux


class VolumeIntegralWeakForm:
    """The weak-form volume integral (Trixi's default of `DGSEM`)."""


class _BC:
    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return self.name


boundary_condition_slip_wall = _BC("boundary_condition_slip_wall")


class BoundaryConditionDirichlet:
    """Trixi's BoundaryConditionDirichlet(boundary_value_function): the
    surface flux (plus half the nonconservative surface flux) of the inner
    state and boundary_value_function(x, t, equations) at the boundary node.
    The boundary states are evaluated on the host at the boundary nodes when
    the semidiscretization is built (at t = 0) and uploaded to the device;
    SemidiscretizationHyperbolic.set_boundary_time(t) re-evaluates them for
    time-dependent data."""

    def __init__(self, boundary_value_function):
        self.boundary_value_function = boundary_value_function

    def __repr__(self):
        return f"BoundaryConditionDirichlet({self.boundary_value_function})"
boundary_condition_periodic = _BC("boundary_condition_periodic")
boundary_condition_simple_slip_wall = _BC("boundary_condition_simple_slip_wall")


class _Source:
    def __init__(self, name, kind):
        self.name = name
        self.kind = kind

    def __repr__(self):
        return self.name


source_terms_rainy = _Source("source_terms_rainy", _lib.TAG_SRC_RAINY)
source_terms_convergence_test_rainy = _Source("source_terms_convergence_test_rainy",
                                              _lib.TAG_SRC_RAINY_CONVERGENCE)
# rainy equations, gravity only (compressible_rainy_euler_2d.jl:580-593)
source_terms_no_phase_change = _Source("source_terms_no_phase_change",
                                       _lib.TAG_SRC_RAINY_NO_PHASE_CHANGE)
# moist equations, src/equations/compressible_moist_euler_2d.jl:320-340, :376-380,
# :203-241, :275-317
source_terms_geopotential = _Source("source_terms_geopotential", _lib.TAG_SRC_GEOPOTENTIAL)
source_terms_moist_bubble = _Source("source_terms_moist_bubble", _lib.TAG_SRC_MOIST_BUBBLE)
source_terms_convergence_test_dry = _Source("source_terms_convergence_test_dry",
                                            _lib.TAG_SRC_MOIST_CONVERGENCE_DRY)
source_terms_convergence_test_moist = _Source("source_terms_convergence_test_moist",
                                              _lib.TAG_SRC_MOIST_CONVERGENCE)
# source_terms_geopotential + source_terms_phase_change +
# source_terms_nonhydrostatic_rayleigh_sponge (:346-373), the sum the
# nonhydrostatic gravity-wave elixir defines
# (examples/euler/dry_air/buoyancy/elixir_gemein_nonhydrostatic_gravity_waves.jl:50-56)
source_terms_nonhydrostatic_gravity_wave = _Source("source_terms_nonhydrostatic_gravity_wave",
                                                   _lib.TAG_SRC_MOIST_GRAVITY_WAVE)


def speed_of_sound_isothermal(equations, T0):
    return math.sqrt(equations.gamma * equations.R * T0)
