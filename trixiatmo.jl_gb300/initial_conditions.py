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
SMALL_EARTH_SCALING = 20                  # :46
SMALL_EARTH_RADIUS = EARTH_RADIUS / SMALL_EARTH_SCALING  # :53
SMALL_EARTH_ROTATION_RATE = EARTH_ROTATION_RATE * SMALL_EARTH_SCALING  # :61
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


def initial_condition_vortex_shedding(x, t, equations):
    """src/equations/initial_condition_compressible_euler_3d.jl:217-240 (DCMIP-2025
    test case 2 on the small Earth): solid-body rotation with u0 = 20 m/s in a
    stratified atmosphere of Brunt-Vaisala frequency N = 0.0182 1/s at
    T = 288 K; phi = g z with z = max(r - a, 0), a = SMALL_EARTH_RADIUS."""
    lon, lat, r = cartesian_to_sphere(x)
    a = SMALL_EARTH_RADIUS
    R = equations.c_p - equations.c_v
    k = R / equations.c_p
    u0 = 20.0
    v1 = -u0 * np.cos(lat) * np.sin(lon)
    v2 = u0 * np.cos(lat) * np.cos(lon)
    v3 = np.zeros_like(r)
    g = EARTH_GRAVITATIONAL_ACCELERATION
    T = 288.0
    om = SMALL_EARTH_ROTATION_RATE
    z = np.maximum(r - a, 0.0)
    phi = g * z
    N = 0.0182
    p = equations.p_0 * np.exp(-a * N ** 2 * u0 / (2 * g ** 2 * k) * (u0 / a + 2 * om) *
                               (np.sin(lat) ** 2 - 1) - N ** 2 / (g ** 2 * k) * phi)
    rho = p / (R * T)
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


class MountainWaveSetup:
    """Uniform flow u0 over a stratification of constant Brunt-Vaisala
    frequency N and surface potential temperature theta_0
    (src/equations/initial_condition_compressible_euler_2d.jl:107-200): called
    with (x, t, equations) it is the initial (and Dirichlet boundary) state,
    theta = theta_0 exp(N^2 z / g), Exner pressure
    1 + g^2 / (c_p theta_0 N^2) (exp(-N^2 z / g) - 1); passed as source_terms
    it is the Rayleigh damping towards that state in the absorbing layers
    (above z_damping_start, beyond +-x_damping_start)."""

    def __init__(self, *, theta_0, u0, brunt_vaisala_frequency, z_damping_start, z_damping_end,
                 x_damping_start, x_damping_end, damping_rate):
        self.theta_0, self.u0 = float(theta_0), float(u0)
        self.brunt_vaisala_frequency = float(brunt_vaisala_frequency)
        self.z_damping_start, self.z_damping_end = float(z_damping_start), float(z_damping_end)
        self.x_damping_start, self.x_damping_end = float(x_damping_start), float(x_damping_end)
        self.damping_rate = float(damping_rate)

    def params(self):
        """(theta_0, u0, N, z_damping_start, z_damping_end, x_damping_start,
        x_damping_end, damping_rate), the device source's parameters."""
        return [self.theta_0, self.u0, self.brunt_vaisala_frequency, self.z_damping_start,
                self.z_damping_end, self.x_damping_start, self.x_damping_end, self.damping_rate]

    def __call__(self, x, t, equations):
        eq = equations
        g, c_p, R = eq.g, eq.c_p, eq.R
        Nf = self.brunt_vaisala_frequency
        z = x[..., 1]
        exner = 1.0 + g * g / (c_p * self.theta_0 * (Nf * Nf)) * (np.exp(-(Nf * Nf) / g * z) - 1.0)
        p = eq.p_0 * exner ** (c_p / R)
        theta = self.theta_0 * np.exp((Nf * Nf) / g * z)
        T = theta * exner
        rho = p / (R * T)
        return eq.prim2cons(rho, self.u0 + 0.0 * rho, 0.0 * rho, p, g * z)

    def __repr__(self):
        return "MountainWaveSetup"


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


class AtmosphereLayers:
    """Saturated moist background atmosphere of constant equivalent potential
    temperature and total water (src/equations/compressible_moist_euler_2d.jl:1009-1104),
    tabulated every `preciseness` metres up to `total_height`.

    Each layer solves the seven equations of the reference's `moist_state`
    (:1009-1034) for y = (p, rho, T, r_t, r_v, rho_qv, theta_e): the discrete
    hydrostatic balance (p - p_below) / dz + g rho = 0, the gas law, the
    definition of theta_e (H = 1), r_t = r_t0, rho_qv = rho_d r_v,
    theta_e = theta_e0, and saturation in the form a + b - sqrt(a^2 + b^2) = 0
    (a the vapour deficit, b the liquid).  The surface layer is solved with
    dz = 0.01 from the guess (p0, rho0, theta_e0, r_t0, r_v0, rho0 r_v0,
    theta_e0); each next layer from the one below.  The reference calls NLsolve
    (trust region, tolerance 1e-8 on the residual); here a damped Newton
    iteration with a complex-step Jacobian (exact to rounding) runs to the
    root's last bits.  layer_data[i] = (rho, rho_theta, rho_qv, rho_ql) at
    z = i * preciseness."""

    def __init__(self, equations, total_height=10010, preciseness=10, ground_state=(1.4, 100000),
                 equivalent_potential_temperature=320, mixing_ratios=(0.02, 0.02)):
        eq = equations
        self.total_height = float(total_height)
        self.preciseness = int(preciseness)
        rho0, p0 = map(float, ground_state)
        r_t0, r_v0 = map(float, mixing_ratios)
        theta_e0 = float(equivalent_potential_temperature)
        n = int(round(total_height / preciseness))
        y = np.array([p0, rho0, theta_e0, r_t0, r_v0, rho0 * r_v0, theta_e0])
        data = np.zeros((n + 1, 4))
        for i in range(n + 1):
            dz = 0.01 if i == 0 else float(preciseness)
            y = self._solve(eq, y, dz, r_t0, theta_e0)
            p, rho, T, r_t, r_v, rho_qv, _ = y
            rho_d = rho / (1.0 + r_t)
            rho_ql = rho - rho_d - rho_qv
            kappa_M = (eq.R_d * rho_d + eq.R_v * rho_qv) / (
                eq.c_pd * rho_d + eq.c_pv * rho_qv + eq.c_pl * rho_ql)
            rho_theta = (rho * (p0 / p) ** kappa_M * T * (1.0 + (eq.R_v / eq.R_d) * r_v) /
                         (1.0 + r_t))
            data[i] = (rho, rho_theta, rho_qv, rho_ql)
        self.layer_data = data

    @staticmethod
    def _residual(eq, y, p_below, dz, r_t0, theta_e0):
        p, rho, T, r_t, r_v, rho_qv, theta_e = y
        rho_d = rho / (1.0 + r_t)
        p_d = eq.R_d * rho_d * T
        T_C = T - 273.15
        p_vs = 611.2 * np.exp(17.62 * T_C / (243.12 + T_C))
        L = eq.L_00 - (eq.c_pl - eq.c_pv) * T
        cm = eq.c_pd + eq.c_pl * r_t
        a = p_vs / (eq.R_v * T) - rho_qv
        b = rho - rho_qv - rho_d
        return np.stack([(p - p_below) / dz + eq.g * rho,
                         p - (eq.R_d * rho_d + eq.R_v * rho_qv) * T,
                         theta_e - T * (p_d / eq.p_0) ** (-eq.R_d / cm) * np.exp(L * r_v / (cm * T)),
                         r_t - r_t0 + 0.0 * p,
                         rho_qv - rho_d * r_v,
                         theta_e - theta_e0 + 0.0 * p,
                         a + b - np.sqrt(a * a + b * b)])

    @classmethod
    def _solve(cls, eq, y0, dz, r_t0, theta_e0):
        y = y0.copy()
        p_below = y0[0]
        scale = np.abs(y0) + 1e-3
        h = 1e-30
        for _ in range(100):
            F = cls._residual(eq, y, p_below, dz, r_t0, theta_e0)
            Yc = y[:, None] + 1j * h * scale[:, None] * np.eye(7)
            J = cls._residual(eq, Yc, p_below, dz, r_t0, theta_e0).imag / (h * scale[None, :])
            step = np.linalg.solve(J, -F)
            nF = np.abs(F).max()
            lam = 1.0
            while lam > 1e-4:
                yn = y + lam * step
                if np.all(np.isfinite(cls._residual(eq, yn, p_below, dz, r_t0, theta_e0))) and (
                        np.abs(cls._residual(eq, yn, p_below, dz, r_t0, theta_e0)).max() < nF
                        or nF < 1e-9):
                    break
                lam *= 0.5
            y = yn
            if np.all(np.abs(lam * step) <= 4e-16 * np.abs(y)):
                break
        return y


def _perturb_moist_profile(x, rho, rho_theta, rho_qv, rho_ql, eq):
    """perturb_moist_profile! (compressible_moist_euler_2d.jl:1148-1206), per
    node over arrays: the Bryan-Fritsch bubble (2 K of density potential
    temperature, radius 2 km at (10 km, 2 km)) at constant pressure, with the
    saturation adjustment by fixed-point iteration to 1e-12 (each node stops
    at its own first converged iterate).  Returns rho, rho_e, rho_qv, rho_ql, T."""
    xc, zc, rc, dtheta = 10000.0, 2000.0, 2000.0, 2.0
    r = np.sqrt((x[..., 0] - xc) ** 2 + (x[..., 1] - zc) ** 2)
    rho_d = rho - rho_qv - rho_ql
    kappa_M = (eq.R_d * rho_d + eq.R_v * rho_qv) / (eq.c_pd * rho_d + eq.c_pv * rho_qv +
                                                   eq.c_pl * rho_ql)
    p_loc = eq.p_0 * (eq.R_d * rho_theta / eq.p_0) ** (1.0 / (1.0 - kappa_M))
    T_loc = p_loc / (eq.R_d * rho_d + eq.R_v * rho_qv)
    rho_e = (eq.c_vd * rho_d + eq.c_vv * rho_qv + eq.c_pl * rho_ql) * T_loc + eq.L_00 * rho_qv
    b = np.nonzero(r < rc)[0]
    if b.size == 0:
        return rho, rho_e, rho_qv, rho_ql, T_loc
    rho, rho_e, rho_qv, rho_ql, T_loc = (a.copy() for a in (rho, rho_e, rho_qv, rho_ql, T_loc))
    th_dens = rho_theta[b] / rho[b] * (p_loc[b] / eq.p_0) ** (kappa_M[b] - eq.kappa)
    th_dens_new = th_dens * (1.0 + dtheta * np.cos(np.pi * (0.5 * r[b] / rc)) ** 2 / 300.0)
    rt = (rho_qv[b] + rho_ql[b]) / rho_d[b]
    rv = rho_qv[b] / rho_d[b]
    th_loc = th_dens_new * (1.0 + rt) / (1.0 + (eq.R_v / eq.R_d) * rv)
    pl = p_loc[b]
    T_b = np.zeros_like(th_loc)
    rvs = np.zeros_like(th_loc)
    rho_d_new = np.zeros_like(th_loc)
    dry = rt <= 0
    T_b[dry] = th_loc[dry] * (pl[dry] / eq.p_0) ** eq.kappa
    rho_d_new[dry] = pl[dry] / (eq.R_d * T_b[dry])
    act = np.nonzero(~dry)[0]
    for _ in range(1000):
        if act.size == 0:
            break
        T_a = th_loc[act] * (pl[act] / eq.p_0) ** eq.kappa
        T_C = T_a - 273.15
        pvs = 611.2 * np.exp(17.62 * T_C / (243.12 + T_C))
        rdn = (pl[act] - pvs) / (eq.R_d * T_a)
        rvs_a = pvs / (eq.R_v * rdn * T_a)
        th_new = th_dens_new[act] * (1.0 + rt[act]) / (1.0 + (eq.R_v / eq.R_d) * rvs_a)
        done = np.abs(th_new - th_loc[act]) <= th_loc[act] * 1.0e-12
        T_b[act], rvs[act], rho_d_new[act] = T_a, rvs_a, rdn
        th_loc[act[~done]] = th_new[~done]
        act = act[~done]
    else:
        raise RuntimeError("moist bubble: saturation adjustment did not converge")
    qv = rvs * rho_d_new
    ql = (rt - rvs) * rho_d_new
    rr = rho_d_new * (1.0 + rt)
    rd = rr - qv - ql
    rho[b], rho_qv[b], rho_ql[b], T_loc[b] = rr, qv, ql, T_b
    rho_e[b] = (eq.c_vd * rd + eq.c_vv * qv + eq.c_pl * ql) * T_b + eq.L_00 * qv
    return rho, rho_e, rho_qv, rho_ql, T_loc


def _moist_bubble_states(layers, x, eq):
    """initial_condition_moist_bubble (compressible_moist_euler_2d.jl:1106-1146)
    at nodes x[..., 2]: (rho, rho_v1, rho_v2, rho_E, rho_qv, rho_ql, T)."""
    data, dz, H = layers.layer_data, float(layers.preciseness), layers.total_height
    flat = np.asarray(x, dtype=np.float64).reshape(-1, 2)
    z = flat[:, 1]
    if np.any((z > H) & ~np.isclose(z, H, rtol=np.sqrt(np.finfo(float).eps), atol=0.0)):
        raise ValueError("the atmosphere does not match the simulation domain")
    n = np.floor((z + np.finfo(float).eps) / dz).astype(np.int64)  # 0-based layer below z
    z_l = n * dz
    z_r = (n + 1) * dz
    top = z_l == H
    z_r = np.where(top, z_l + dz, z_r)
    n = np.where(top, n - 1, n)
    rl, thl, qvl, qll = data[n].T
    rr, thr, qvr, qlr = data[n + 1].T
    rho = (rr * (z - z_l) + rl * (z_r - z)) / dz
    rho_theta = rho * (thr / rr * (z - z_l) + thl / rl * (z_r - z)) / dz
    rho_qv = rho * (qvr / rr * (z - z_l) + qvl / rl * (z_r - z)) / dz
    rho_ql = rho * (qlr / rr * (z - z_l) + qll / rl * (z_r - z)) / dz
    rho, rho_e, rho_qv, rho_ql, T = _perturb_moist_profile(flat, rho, rho_theta, rho_qv, rho_ql,
                                                           eq)
    z0 = np.zeros_like(rho)
    out = np.stack([rho, z0, z0, rho_e + 0.5 * rho * 0.0, rho_qv, rho_ql, T], axis=-1)
    return out.reshape(np.shape(x)[:-1] + (7,))


def initial_condition_moist_bubble(atmosphere_layers):
    """Moist bubble of Bryan & Fritsch (2002)
    (compressible_moist_euler_2d.jl:1106-1146): the layer data interpolated
    linearly in z (rho; rho_theta, rho_qv, rho_ql per unit rho), then the
    perturbation; at rest.  Returns the initial condition (x, t, equations)."""
    def ic(x, t, equations):
        return _moist_bubble_states(atmosphere_layers, x, equations)[..., :6]

    return ic


def initial_condition_moist_bubble_rainy(atmosphere_layers, moist_equations):
    """The moist bubble as a state of the rainy equations
    (examples/euler/moist_air/buoyancy/elixir_hoeck_bubble.jl:16-25):
    (rho_dry, rho_vapour + rho_cloud, rho_rain = 0, rho_v1, rho_v2, energy,
    rho_vapour, rho_cloud, T), the bubble computed with the moist equations'
    constants."""
    def ic(x, t, equations):
        s = _moist_bubble_states(atmosphere_layers, x, moist_equations)
        rho, qv, ql = s[..., 0], s[..., 4], s[..., 5]
        z0 = np.zeros_like(rho)
        return np.stack([rho - qv - ql, qv + ql, z0, s[..., 1], s[..., 2], s[..., 3], qv, ql,
                         s[..., 6]], axis=-1)

    return ic


# ---- the rainy bubble with precipitation (elixir_hoeck_bubble.jl) ------------
def _theta_d_rainy(z, eq):
    """Hydrostatic dry potential temperature of the rainy bubble
    (src/equations/compressible_rainy_euler_2d.jl:1062-1078): 283 K at 850 hPa,
    stratification 1.3e-5 1/m."""
    theta0 = 283.0 * (eq.ref_pressure / 85000.0) ** (eq.R_d / eq.c_pd)
    return theta0 * np.exp(1.3e-5 * z)


def _complex_step_newton(residual, y, scale, tol_rel=4e-16, maxit=60):
    """Newton's method on independent small systems y[..., k] (k unknowns per
    point) with the Jacobian by complex steps (exact to rounding), iterated to
    the root's last bits.  The reference's NLsolve stops at a residual
    tolerance; both find the same isolated root."""
    y = np.array(y, dtype=np.float64)
    k = y.shape[-1]
    h = 1e-30
    eye = np.eye(k)
    norm = lambda F: np.abs(F).max(axis=-1)  # noqa: E731
    for _ in range(maxit):
        F = residual(y)
        yc = y[..., None, :] + 1j * h * (scale[..., None, :] * eye)
        # row c of the complex evaluation perturbs unknown c: dF/dy_c * h * scale_c
        J = np.swapaxes(residual(yc).imag / (h * scale[..., :, None]), -1, -2)
        step = np.linalg.solve(J, -F[..., None])[..., 0]
        # halve the step where it does not reduce the residual (far from the root)
        lam = np.ones(y.shape[:-1])
        for _ in range(30):
            Fn = residual(y + lam[..., None] * step)
            bad = ~(np.isfinite(Fn).all(axis=-1) & ((norm(Fn) < norm(F)) | (norm(F) < 1e-12)))
            if not np.any(bad):
                break
            lam = np.where(bad, 0.5 * lam, lam)
        y = y + lam[..., None] * step
        if np.all(np.abs(lam[..., None] * step) <= tol_rel * np.abs(y)):
            break
    return y


class AtmosphereLayersRainyBubble:
    """Hydrostatic background of the rainy bubble
    (src/equations/compressible_rainy_euler_2d.jl:1087-1129): layer_data[i] =
    (p, rho_dry, rho_vapour, T) at z = 0.01 + i * precision, each layer solving
    the discrete hydrostatic balance (p - p_below)/dz + (rho_dry + rho_vapour) g
    = 0, the gas law, the dry potential temperature profile and 20 % relative
    humidity from the layer below (the surface layer with dz = 0.01 from
    (850 hPa, 1.4, 0.04, 300 K))."""

    def __init__(self, equations, total_height, precision=1.0):
        eq = equations
        self.total_height = float(total_height)
        self.precision = float(precision)
        n = int(round(self.total_height / self.precision))
        h0 = 0.2
        data = np.zeros((n + 1, 4))
        z, dz = 0.01, 0.01
        guess = np.array([85000.0, 1.4, 0.04, 300.0])
        data[0] = self._solve(eq, guess, 85000.0, h0, z, dz)
        dz = self.precision
        for i in range(n):
            z += dz
            data[i + 1] = self._solve(eq, data[i], data[i, 0], h0, z, dz)
        self.layer_data = data

    @staticmethod
    def _solve(eq, guess, p_below, h0, z, dz):
        eps = eq.R_d / eq.R_v
        th = _theta_d_rainy(z, eq)

        def res(y):
            p, rd, rv, T = y[..., 0], y[..., 1], y[..., 2], y[..., 3]
            rvs = eq.saturation_vapour_pressure(T) / (eq.R_v * T)
            return np.stack([(p - p_below) / dz + (rd + rv) * eq.gravity,
                             p - T * (rd * eq.R_d + rv * eq.R_v),
                             th - T * (eq.ref_pressure / p) ** (eq.R_d / eq.c_pd),
                             (rvs * (rd + rv / eps) * h0 - rv * (rd + rvs / eps)) * 1000.0],
                            axis=-1)
        y = np.asarray(guess, dtype=np.float64)
        return _complex_step_newton(res, y, np.abs(y) + 1e-3)


def initial_condition_bubble_rainy(x, t, equations, atmosphere_layers):
    """src/equations/compressible_rainy_euler_2d.jl:1131-1202: a humid bubble
    (relative humidity 1 inside r = 200 m, a cos^2 ramp to the background 0.2 at
    r = 300 m around (1200 m, 800 m)) in the hydrostatic background; per node
    the pressure is interpolated between the layers around z and
    (rho_dry, rho_vapour, T) solve the humidity, dry potential temperature and
    pressure equations from the lower layer's values.  State (rho_dry,
    rho_vapour, 0, 0, 0, energy, rho_vapour, 0, T), all moisture as vapour."""
    eq = equations
    x = np.asarray(x, dtype=np.float64)
    r = np.sqrt((x[..., 0] - 1200.0) ** 2 + (x[..., 1] - 800.0) ** 2)
    hb = 0.2
    hum = np.where(r > 300.0, hb,
                   np.where(r > 200.0,
                            hb + (1.0 - hb) * np.cos(np.pi * (r - 200.0) / (2 * 100.0)) ** 2,
                            1.0))
    L = atmosphere_layers
    dz = L.precision
    z = x[..., 1]
    n = np.floor((z + np.finfo(np.float64).eps) / dz).astype(np.int64) + 1  # Julia's 1-based row
    z_lower = (n - 1) * dz
    z_upper = n * dz
    top = z_lower == L.total_height
    z_upper = np.where(top, z_lower + dz, z_upper)
    n = np.where(top, n - 1, n)
    n = np.where(n == 0, 1, n)
    if np.any(z > L.total_height + 1e-9 * L.total_height):
        raise ValueError("The atmosphere does not match the simulation domain")
    lo, up = L.layer_data[n - 1], L.layer_data[n]
    p_h = (up[..., 0] * (z - z_lower) + lo[..., 0] * (z_upper - z)) / dz
    eps = eq.R_d / eq.R_v
    th = _theta_d_rainy(z, eq)

    def res(y):
        rd, rv, T = y[..., 0], y[..., 1], y[..., 2]
        # the node fields broadcast over the Jacobian's extra axis
        b = lambda a: a.reshape(a.shape + (1,) * (rd.ndim - a.ndim))  # noqa: E731
        rvs = eq.saturation_vapour_pressure(T) / (eq.R_v * T)
        p = (rd * eq.R_d + rv * eq.R_v) * T
        return np.stack([(rvs * (rd + rv / eps) * b(hum) - rv * (rd + rvs / eps)) * 30.0,
                         b(th) - T * (eq.ref_pressure / b(p_h)) ** (eq.R_d / eq.c_pd),
                         b(p_h) - p], axis=-1)
    y0 = lo[..., 1:4].copy()
    y = _complex_step_newton(res, y0, np.abs(y0) + 1e-3)
    rd, rv, T = y[..., 0], y[..., 1], y[..., 2]
    energy = (eq.c_vd * rd + eq.c_vv * rv) * T + rv * eq.ref_latent_heat_vap_temp
    zero = np.zeros_like(rd)
    return np.stack([rd, rv, zero, zero, zero, energy, rv, zero, T], axis=-1)
