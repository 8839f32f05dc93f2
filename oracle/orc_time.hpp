// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Explicit time integrators used by the reference's elixirs and tests.
// * CarpenterKennedy2N54 (OrdinaryDiffEqLowStorageRK, external): the
//   five-stage fourth-order 2N-storage scheme "RK4(3)5[2N] solution 3" of
//   M. H. Carpenter, C. A. Kennedy, NASA TM-109112 (1994). Per stage s:
//     du = f(u, t + c_s dt);  k = A_s k + dt du;  u = u + B_s k.
//   Used by e.g. examples/euler/moist_air/buoyancy/elixir_gemein_bubble.jl:121.
// * SSPRK43 (OrdinaryDiffEqSSPRK, external): the four-stage third-order SSP
//   scheme with SSP coefficient 2 (J. F. B. M. Kraaijevanger, BIT 31 (1991);
//   R. J. Spiteri, S. J. Ruuth, SINUM 40 (2002)), run with adaptive = false
//   by examples/euler/dry_air/buoyancy/elixir_energy_inertia_gravity_waves.jl:74-78:
//     u1 = u + dt/2 f(u, t);          u2 = u1 + dt/2 f(u1, t + dt/2)
//     u3 = 2/3 u + 1/3 (u2 + dt/2 f(u2, t + dt));  u+ = u3 + dt/2 f(u3, t + dt/2)
#pragma once
#include <cstddef>
#include <vector>

namespace orc {

struct CK2N54 {
  static constexpr int stages = 5;
  static constexpr double A[5] = {0.0,
                                  -567301805773.0 / 1357537059087.0,
                                  -2404267990393.0 / 2016746695238.0,
                                  -3550918686646.0 / 2091501179385.0,
                                  -1275806237668.0 / 842570457699.0};
  static constexpr double B[5] = {1432997174477.0 / 9575080441755.0,
                                  5161836677717.0 / 13612068292357.0,
                                  1720146321549.0 / 2090206949498.0,
                                  3134564353537.0 / 4481467310338.0,
                                  2277821191437.0 / 14882151754819.0};
  static constexpr double c[5] = {0.0,
                                  1432997174477.0 / 9575080441755.0,
                                  2526269341429.0 / 6820363962896.0,
                                  2006345519317.0 / 3224310063776.0,
                                  2802321613138.0 / 2924317926251.0};
};

// One CK2N54 step; `rhs(u, du, t)` evaluates the semidiscretization.
template <class Rhs>
void ck2n54_step(Rhs&& rhs, double* u, double* k, double* du, size_t N, double t, double dt) {
  for (int s = 0; s < CK2N54::stages; ++s) {
    rhs(u, du, t + CK2N54::c[s] * dt);
    const double a = CK2N54::A[s], bb = CK2N54::B[s];
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)N; ++q) {
      k[q] = a * k[q] + dt * du[q];
      u[q] = u[q] + bb * k[q];
    }
  }
}

// One SSPRK43 step (Kraaijevanger 1991, Shu-Osher form); `lim(v)` is the
// stage limiter applied to every stage value (a no-op without one).
template <class Rhs, class Lim>
void ssprk43_step(Rhs&& rhs, Lim&& lim, double* u, double* tmp, double* du, double* u0, size_t N,
                  double t, double dt) {
  const double h = 0.5 * dt;
  for (size_t q = 0; q < N; ++q) u0[q] = u[q];
  rhs(u, du, t);
  for (size_t q = 0; q < N; ++q) tmp[q] = u[q] + h * du[q];
  lim(tmp);
  rhs(tmp, du, t + h);
  for (size_t q = 0; q < N; ++q) tmp[q] = tmp[q] + h * du[q];
  lim(tmp);
  rhs(tmp, du, t + dt);
  for (size_t q = 0; q < N; ++q) tmp[q] = (2.0 / 3.0) * u0[q] + (1.0 / 3.0) * (tmp[q] + h * du[q]);
  lim(tmp);
  rhs(tmp, du, t + h);
  for (size_t q = 0; q < N; ++q) u[q] = tmp[q] + h * du[q];
  lim(u);
}

template <class Rhs>
void ssprk43_step(Rhs&& rhs, double* u, double* tmp, double* du, double* u0, size_t N, double t,
                  double dt) {
  ssprk43_step(rhs, [](double*) {}, u, tmp, du, u0, N, t, dt);
}

// One SSPRK33 step (Shu & Osher 1988, Shu-Osher form), stage limiter `lim`.
template <class Rhs, class Lim>
void ssprk33_step(Rhs&& rhs, Lim&& lim, double* u, double* tmp, double* du, double* u0, size_t N,
                  double t, double dt) {
  for (size_t q = 0; q < N; ++q) u0[q] = u[q];
  rhs(u, du, t);
  for (size_t q = 0; q < N; ++q) tmp[q] = u[q] + dt * du[q];
  lim(tmp);
  rhs(tmp, du, t + dt);
  for (size_t q = 0; q < N; ++q) tmp[q] = 0.75 * u0[q] + 0.25 * (tmp[q] + dt * du[q]);
  lim(tmp);
  rhs(tmp, du, t + 0.5 * dt);
  for (size_t q = 0; q < N; ++q) u[q] = (1.0 / 3.0) * u0[q] + (2.0 / 3.0) * (tmp[q] + dt * du[q]);
  lim(u);
}

// `nsteps` steps of SSPRK43 (scheme 1) or SSPRK33 (scheme 2), adaptive = false:
// dt = cfl * max_dt(u) before each step (or fixed_dt > 0), the last one
// shortened to land on t_end (> 0).  Returns the new time.
template <class Rhs, class MaxDt, class Lim>
double ssp_steps(Rhs&& rhs, MaxDt&& max_dt, Lim&& lim, double* u, size_t N, double t, double cfl,
                 int nsteps, int scheme, double fixed_dt, double t_end) {
  std::vector<double> tmp(N), du(N), u0(N);
  for (int s = 0; s < nsteps; ++s) {
    if (t_end > 0 && t >= t_end) break;
    double dt = fixed_dt > 0 ? fixed_dt : cfl * max_dt(u);
    if (t_end > 0 && t + dt > t_end) dt = t_end - t;
    if (scheme == 2)
      ssprk33_step(rhs, lim, u, tmp.data(), du.data(), u0.data(), N, t, dt);
    else
      ssprk43_step(rhs, lim, u, tmp.data(), du.data(), u0.data(), N, t, dt);
    t += dt;
  }
  return t;
}

}  // namespace orc
