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


def initial_condition_adiabatic(x, t, equations):
    """src/equations/initial_condition_compressible_euler_2d.jl:44-67: an
    adiabatic atmosphere at rest (potential temperature 300 K) in hydrostatic
    balance."""
    g, c_p, c_v = equations.g, equations.c_p, equations.c_v
    p0 = 100_000.0
    R = c_p - c_v
    theta = 300.0
    exner = 1.0 - g / (c_p * theta) * x[..., 1]
    p = p0 * exner ** (c_p / R)
    T = theta * exner
    rho = p / (R * T)
    return equations.prim2cons(rho, 0.0, 0.0, p, g * x[..., 1])


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


# ---- 3D spherical-shell states ------------------------------------------------
EARTH_RADIUS = 6.37122e6                  # src/equations/reference_data.jl:11
EARTH_GRAVITATIONAL_ACCELERATION = 9.80616  # :19
EARTH_ROTATION_RATE = 7.292e-5            # :27
SECONDS_PER_DAY = 8.64e4                  # :35


def cartesian_to_sphere(x):
    """(lon in [0, 2pi), lat, r) of Cartesian points (src/auxiliary/auxiliary.jl:25-34)."""
    r = np.linalg.norm(x, axis=-1)
    lam = np.arctan2(x[..., 1], x[..., 0])
    lam = np.where(lam < 0, lam + 2 * np.pi, lam)
    return lam, np.arcsin(x[..., 2] / r), r


def _baroclinic_basic_state(lon, lat, z):
    """Balanced zonal state (rho, u, p) of Ullrich et al. (2013), as in
    src/equations/initial_condition_compressible_euler_3d.jl:4-66."""
    a = EARTH_RADIUS
    b = 2.0
    g = EARTH_GRAVITATIONAL_ACCELERATION
    k = 3.0
    p0 = 1.0e5
    Rg = 287.0
    TE, TP = 310.0, 240.0
    lapse = 0.005
    omega = EARTH_ROTATION_RATE
    r = z + a
    T0 = 0.5 * (TE + TP)
    A = 1.0 / lapse
    B = (T0 - TP) / (T0 * TP)
    C = 0.5 * (k + 2) * (TE - TP) / (TE * TP)
    H = Rg * T0 / g
    sz = z / (b * H)
    t1 = np.exp(lapse / T0 * z)
    t2 = np.exp(-sz ** 2)
    tau1 = A * lapse / T0 * t1 + B * (1 - 2 * sz ** 2) * t2
    tau2 = C * (1 - 2 * sz ** 2) * t2
    inttau1 = A * (t1 - 1) + B * z * t2
    inttau2 = C * z * t2
    t3 = r / a * np.cos(lat)
    t4 = t3 ** k - k / (k + 2) * t3 ** (k + 2)
    T = 1.0 / ((r / a) ** 2 * (tau1 - tau2 * t4))
    big_u = g / a * k * T * inttau2 * (t3 ** (k - 1) - t3 ** (k + 1))
    t5 = a * np.cos(lat)
    u = -omega * t5 + np.sqrt(omega ** 2 * t5 ** 2 + t5 * big_u)
    p = p0 * np.exp(-g / Rg * (inttau1 - inttau2 * t4))
    rho = p / (Rg * T)
    return rho, u, p


def _baroclinic_perturbation(lon, lat, z):
    """Stream-function perturbation (u', v'), :68-108."""
    d0 = 1.0 / 6.0
    vp = 1.0
    plon, plat = np.pi / 9, 2 * np.pi / 9
    pertz = 15000.0
    gc = np.arccos(np.clip(np.sin(plat) * np.sin(lat) +
                           np.cos(plat) * np.cos(lat) * np.cos(lon - plon), -1, 1))
    active = (z <= pertz) & (gc <= d0)
    taper = 1 - 3 * z ** 2 / pertz ** 2 + 2 * z ** 3 / pertz ** 3
    s = np.sin(0.5 * np.pi * gc / d0)
    c = np.cos(0.5 * np.pi * gc / d0)
    with np.errstate(divide="ignore", invalid="ignore"):
        factor = 16 / (3 * np.sqrt(3)) * vp * taper * c ** 3 * s
        up = -factor * (-np.sin(plat) * np.cos(lat) +
                        np.cos(plat) * np.sin(lat) * np.cos(lon - plon)) / np.sin(gc)
        vpp = factor * np.cos(plat) * np.sin(lon - plon) / np.sin(gc)
    return np.where(active, up, 0.0), np.where(active, vpp, 0.0)


def initial_condition_baroclinic_instability(x, t, equations):
    """:110-160 — balanced zonal flow plus a localized stream-function bump;
    phi = -a^2 g / |x|."""
    lon, lat, r = cartesian_to_sphere(x)
    z = np.maximum(r - EARTH_RADIUS, 0.0)
    rho, u, p = _baroclinic_basic_state(lon, lat, z)
    up, vp = _baroclinic_perturbation(lon, lat, z)
    u = u + up
    v = vp
    v1 = -np.sin(lon) * u - np.sin(lat) * np.cos(lon) * v
    v2 = np.cos(lon) * u - np.sin(lat) * np.sin(lon) * v
    v3 = np.cos(lat) * v
    phi = -EARTH_RADIUS ** 2 * EARTH_GRAVITATIONAL_ACCELERATION / r
    return equations.prim2cons(rho, v1, v2, v3, p, phi)


class IsothermalShell:
    """Isothermal atmosphere at rest in hydrostatic balance on the shell (the
    pattern of initial_condition_isothermal, :171-196, with temperature T),
    phi = g (a - a^2 / r), plus seeded Gaussian density perturbations of
    relative amplitude `amplitude` and horizontal width `width` centred at
    `ncenters` points drawn uniformly on the sphere (Philox stream `seed`)."""

    def __init__(self, T=250.0, amplitude=1e-3, width=500e3, ncenters=16, seed=1,
                 radius=EARTH_RADIUS, gravity=EARTH_GRAVITATIONAL_ACCELERATION):
        self.T, self.amplitude, self.width = T, amplitude, width
        self.radius, self.g = radius, gravity
        rng = np.random.Generator(np.random.Philox(seed))
        zc = rng.uniform(-1, 1, ncenters)
        lc = rng.uniform(0, 2 * np.pi, ncenters)
        s = np.sqrt(1 - zc ** 2)
        self.centers = np.stack([s * np.cos(lc), s * np.sin(lc), zc], axis=-1)

    def __call__(self, x, t, equations):
        a, g = self.radius, self.g
        r = np.linalg.norm(x, axis=-1)
        rr = np.maximum(r - a, 0.0) + a
        p = equations.p_0 * np.exp(g * (a * a / rr - a) / (equations.R * self.T))
        rho = p / (equations.R * self.T)
        unit = x / r[..., None]
        bump = np.zeros_like(r)
        for c in self.centers:
            ang = np.arccos(np.clip(unit @ c, -1.0, 1.0))
            bump += np.exp(-(a * ang / self.width) ** 2)
        rho = rho * (1.0 + self.amplitude * bump)
        phi = g * (a - a * a / rr)
        z = np.zeros_like(r)
        return equations.prim2cons(rho, z, z, z, p, phi)


# ---- 2D rainy states ---------------------------------------------------------
def initial_condition_convergence_test_rainy(x, t, equations):
    """examples/euler/precipitation/tests/convergence_test.jl:8-40 (manufactured
    solution, travelling along x + y)."""
    eq = equations
    rho = 2.0 + 0.1 * np.sin(np.pi * (x[..., 0] + x[..., 1] - t))
    T = rho + 250.0
    rv = eq.saturation_vapour_pressure(T) / (eq.R_v * T)
    rc = rho / eq.c_l * 3000.0
    rr = rho / eq.c_l * 1000.0
    rm = rv + rc
    rd = rho - rm - rr
    e = (eq.c_vd * rd + eq.c_vv * rv + eq.c_l * (rc + rr)) * T + rv * eq.ref_latent_heat_vap_temp + rho
    return np.stack([rd, rm, rr, rho, rho, e, rv, rc, T], axis=-1)


class MoistBubbleRainy:
    """Seeded moist state for the learned-Newton-guess benchmark (20 km x 10 km):
    a dry-adiabatic-ish background (surface 288 K, lapse 6.5 K/km, hydrostatic
    pressure), per-node relative humidity U[rh_min, rh_max], a saturated bubble
    (RH = 1) of radius `radius` at (xc, zc), cloud and rain mixing ratios
    U[0, qmax] of the dry density, and zero velocity.  Slots 7-9 hold the
    constructed (vapour, cloud, temperature) triple — not the saturation
    equilibrium, which the Newton solve then finds (the 'plain' warm start)."""

    def __init__(self, seed=2, rh_min=0.2, rh_max=1.0, qmax=1e-3, xc=10000.0, zc=2000.0,
                 radius=2000.0, T0=288.0, lapse=0.0065):
        self.seed, self.rh_min, self.rh_max, self.qmax = seed, rh_min, rh_max, qmax
        self.xc, self.zc, self.radius = xc, zc, radius
        self.T0, self.lapse = T0, lapse

    def __call__(self, x, t, equations):
        eq = equations
        shape = x.shape[:-1]
        rng = np.random.Generator(np.random.Philox(self.seed))
        z = x[..., 1]
        T = self.T0 - self.lapse * z
        p = 1e5 * (T / self.T0) ** (eq.gravity / (eq.R_d * self.lapse))
        rh = rng.uniform(self.rh_min, self.rh_max, shape)
        r = np.sqrt((x[..., 0] - self.xc) ** 2 + (z - self.zc) ** 2)
        rh = np.where(r <= self.radius, 1.0, rh)
        rv = rh * eq.saturation_vapour_pressure(T) / (eq.R_v * T)
        rd = (p - rv * eq.R_v * T) / (eq.R_d * T)
        rc = rng.uniform(0.0, self.qmax, shape) * rd
        rr = rng.uniform(0.0, self.qmax, shape) * rd
        rm = rv + rc
        e = (eq.c_vd * rd + eq.c_vv * rv + eq.c_l * (rc + rr)) * T + rv * eq.ref_latent_heat_vap_temp
        z0 = np.zeros_like(T)
        return np.stack([rd, rm, rr, z0, z0, e, rv, rc, T], axis=-1)


# ---- CompressibleMoistEulerEquations2D ------------------------------------
def initial_condition_gemein_bubble(x, t, equations):
    """Warm bubble of examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl:20-51
    (Wicker & Skamarock 1998) for the moist equations without moisture: neutral
    theta_ref = 300 K background, cos^2 bubble of 2 K and radius 2 km at
    (10 km, 2 km), uniform v1 = 20 m/s."""
    eq = equations
    xc, zc, rc, theta_ref = 10000.0, 2000.0, 2000.0, 300.0
    r = np.sqrt((x[..., 0] - xc) ** 2 + (x[..., 1] - zc) ** 2)
    dtheta = np.where(r <= rc, 2.0 * np.cos(np.pi * (0.5 * r / rc)) ** 2, 0.0)
    theta = theta_ref + dtheta
    p = eq.p_0 * (1.0 - eq.kappa * eq.g * x[..., 1] / (eq.R_d * theta_ref)) ** (eq.c_pd / eq.R_d)
    rho = p / ((p / eq.p_0) ** eq.kappa * eq.R_d * theta)
    T = p / (eq.R_d * rho)
    v1 = 20.0
    z0 = np.zeros_like(rho)
    return np.stack([rho, rho * v1, z0, rho * eq.c_vd * T + 0.5 * rho * v1 * v1, z0, z0],
                    axis=-1)


def initial_condition_nonhydrostatic_gravity_wave(x, t, equations):
    """Mountain-triggered gravity wave (Gallus & Klemp 2000) of
    examples/euler/dry_air/buoyancy/elixir_gemein_nonhydrostatic_gravity_waves.jl:15-39
    for the moist equations without moisture: constant Brunt-Vaisala frequency
    N = 0.01 over theta_0 = T_0 = 280 K, hydrostatic pressure, uniform
    v1 = 10 m/s."""
    eq = equations
    z = x[..., 1]
    theta_0, N = 280.0, 0.01
    theta = theta_0 * np.exp(N * N * z / eq.g)
    p = eq.p_0 * (1.0 + eq.g * eq.g * (1.0 / (eq.c_pd * theta_0 * (N * N))) *
                  (np.exp(-z * (N * N) / eq.g) - 1.0)) ** (1.0 / eq.kappa)
    rho = p / ((p / eq.p_0) ** eq.kappa * eq.R_d * theta)
    T = p / (eq.R_d * rho)
    v1, v2 = 10.0, 0.0
    z0 = np.zeros_like(rho)
    return np.stack([rho, rho * v1, rho * v2, rho * eq.c_vd * T + 0.5 * rho * (v1 * v1 + v2 * v2),
                     z0, z0], axis=-1)


def initial_condition_convergence_test_dry(x, t, equations):
    """src/equations/compressible_moist_euler_2d.jl:173-200."""
    eq = equations
    ini = 2.0 + 0.1 * np.sin(np.pi * (x[..., 0] + x[..., 1] - t))
    T = (ini - 1.0) / eq.c_vd
    E = eq.c_vd * T + 1.0
    z0 = np.zeros_like(ini)
    return np.stack([ini, ini, ini, E * ini, z0, z0], axis=-1)


def initial_condition_convergence_test_moist(x, t, equations):
    """src/equations/compressible_moist_euler_2d.jl:244-272."""
    eq = equations
    ini = 2.0 + 0.1 * np.sin(np.pi * (x[..., 0] + x[..., 1] - t))
    qv = 100.0 / eq.L_00
    ql = qv / 10.0
    mu = (1.0 - qv - ql) * eq.c_vd + qv * eq.c_vv + ql * eq.c_pl
    T = (ini - 1.0) / mu + 10.0 / eq.c_vd + 40.0
    E = mu * T + qv * eq.L_00 + 1.0
    return np.stack([ini, ini, ini, E * ini, qv * ini, ql * ini], axis=-1)
