"""Host-side initial conditions (the reference's `initial_condition_*` functions,
evaluated at the node coordinates like Trixi's `compute_coefficients!`).

Each takes x[..., 2] (node coordinates), t and the equations, and returns the
conservative state u[..., nv].
"""
from __future__ import annotations

import numpy as np


def initial_condition_gravity_waves(x, t, equations):
    """src/equations/initial_condition_compressible_euler_2d.jl:11-35."""
    g, c_p, c_v = equations.g, equations.c_p, equations.c_v
    x_c, a, H = 100_000.0, 5_000.0, 10_000.0
    R = c_p - c_v
    T0 = 250.0
    delta = g / (R * T0)
    DeltaT = 0.001
    Tb = DeltaT * np.sin(np.pi * x[..., 1] / H) * np.exp(-(x[..., 0] - x_c) ** 2 / a ** 2)
    ps = 100_000.0
    rhos = ps / (T0 * R)
    rho_b = rhos * (-Tb / T0)
    p = ps * np.exp(-delta * x[..., 1])
    rho = rhos * np.exp(-delta * x[..., 1]) + rho_b * np.exp(-0.5 * delta * x[..., 1])
    return equations.prim2cons(rho, 20.0, 0.0, p, g * x[..., 1])


class WarmBubble:
    """Dry warm bubble (Wicker & Skamarock 1998) of
    examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl:20-51 for the
    energy-with-gravity equations: neutral background theta_ref = 300 K and a
    cos^2 potential-temperature bubble of amplitude `dtheta` and radius `rc`
    centred at (xc, zc); horizontal wind `v1`."""

    def __init__(self, xc=10_000.0, zc=2_000.0, rc=2_000.0, dtheta=2.0, v1=0.0, theta_ref=300.0):
        self.xc, self.zc, self.rc, self.dtheta, self.v1 = xc, zc, rc, dtheta, v1
        self.theta_ref = theta_ref

    def __call__(self, x, t, equations):
        eq = equations
        kappa = eq.R / eq.c_p
        r = np.sqrt((x[..., 0] - self.xc) ** 2 + (x[..., 1] - self.zc) ** 2)
        dth = np.where(r <= self.rc, self.dtheta * np.cos(0.5 * np.pi * r / self.rc) ** 2, 0.0)
        theta = self.theta_ref + dth
        p = eq.p_0 * (1.0 - kappa * eq.g * x[..., 1] / (eq.R * self.theta_ref)) ** (eq.c_p / eq.R)
        rho = p / ((p / eq.p_0) ** kappa * eq.R * theta)
        T = p / (eq.R * rho)
        rho_e = rho * eq.c_v * T + 0.5 * rho * self.v1 ** 2
        z = np.zeros_like(rho)
        return np.stack([rho, rho * self.v1 + z, z, rho_e, eq.g * x[..., 1]], axis=-1)


def seeded_perturbation(u, equations, seed, amplitude=1e-2, velocity=5.0):
    """Seeded (Philox) non-hydrostatic perturbation of a state: relative density
    and energy noise of `amplitude` and velocities of up to `velocity` m/s.
    Used for parity tests on states far from balance."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = u.copy()
    rho = u[..., 0] * (1.0 + amplitude * rng.uniform(-1, 1, u.shape[:-1]))
    v1 = velocity * rng.uniform(-1, 1, u.shape[:-1])
    v2 = velocity * rng.uniform(-1, 1, u.shape[:-1])
    _, _, _, p, phi = equations.cons2prim(u)
    p = p * (1.0 + amplitude * rng.uniform(-1, 1, u.shape[:-1]))
    return equations.prim2cons(rho, v1, v2, p, phi)
