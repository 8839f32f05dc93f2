// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Explicit time integrators used by the reference's elixirs and tests.
// * CarpenterKennedy2N54 (OrdinaryDiffEqLowStorageRK, external): the
//   five-stage fourth-order 2N-storage scheme "RK4(3)5[2N] solution 3" of
//   M. H. Carpenter, C. A. Kennedy, NASA TM-109112 (1994). Per stage s:
//     du = f(u, t + c_s dt);  k = A_s k + dt du;  u = u + B_s k.
//   Used by e.g. examples/euler/moist_air/buoyancy/elixir_gemein_bubble.jl:100-102.
// * SSPRK43 (OrdinaryDiffEqSSPRK, external): the four-stage third-order SSP
//   scheme with SSP coefficient 2 (J. F. B. M. Kraaijevanger, BIT 31 (1991);
//   R. J. Spiteri, S. J. Ruuth, SINUM 40 (2002)), run with adaptive = false
//   by examples/euler/dry_air/buoyancy/elixir_energy_inertia_gravity_waves.jl:74-78:
//     u1 = u + dt/2 f(u, t);          u2 = u1 + dt/2 f(u1, t + dt/2)
//     u3 = 2/3 u + 1/3 (u2 + dt/2 f(u2, t + dt));  u+ = u3 + dt/2 f(u3, t + dt/2)
#pragma once
#include <algorithm>
#include <cmath>
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

#ifndef ORC_FLOP_COUNTING  // the operation-count build needs only the fixed-step schemes
// Adaptive SSPRK43 as OrdinaryDiffEq runs it by default (solve(ode,
// SSPRK43(); abstol, reltol), OrdinaryDiffEqSSPRK, external; used without a
// StepsizeCallback by e.g. examples/euler/dry_air/mountain_flow/
// elixir_potential_temperature_linear_hydrostatic.jl:83-86).  Restated from the
// published algorithms:
// * Step: the Shu-Osher form above.  Error estimate: the difference to the
//   embedded second-order method with weights b^ = (1/4, 1/4, 1/4, 1/4) on the
//   four stage derivatives (the SSPRK(4,3) pair of I. Higueras / D. Conde et
//   al., "Embedded pairs for optimal explicit SSP RK methods", 2022), i.e.
//   u^ = (u+ + (u/3 + 2/3 (u2 + dt/2 f(u2))))/2.
// * Error norm: EEst = sqrt(mean_i (e_i / (abstol + max(|u_i|, |u+_i|) reltol))^2)
//   over every entry of the state.
// * PI step-size control (Hairer, Norsett, Wanner; Gustafsson 1991) with
//   beta1 = 7/(10 p), beta2 = 2/(5 p), p = 3; q = EEst^beta1 / qold^beta2,
//   clamped to [1/qmax, 1/qmin] after division by gamma = 0.9 (qmin = 1/5,
//   qmax = 10); accepted (EEst <= 1): dt_new = dt / q, qold = max(EEst, 1e-4);
//   rejected: dt /= min(1/qmin, EEst^beta1 / gamma).
// * Initial step: Hairer, Norsett, Wanner (1993) II.4: d0 = |u0/sk|,
//   d1 = |f0/sk|, dt0 = 0.01 d0/d1 (1e-6 if either is below 1e-5), one Euler
//   step, d2 = |(f1 - f0)/sk| / dt0, dt1 = (0.01 / max(d1, d2))^(1/p_init)
//   (max(1e-6, 1e-3 dt0) if max(d1, d2) <= 1e-15), dt = min(100 dt0, dt1),
//   with sk = abstol + |u0| reltol and the same root-mean-square norm.
// * Stops: a step never passes the next stop (the save times and the end);
//   the controller's next proposal uses the step actually taken.
// `variant` selects alternatives while the restatement is pinned to the
// reference's goldens: bit 0 the embedded weights (1/3, 1/3, 1/3, 0); bit 1
// p_init = order + 1; bit 2 beta from the embedded order 2.
struct AdaptiveStats {
  long accepted = 0, rejected = 0, rhs_calls = 0;
  double dt_first = 0.0, dt_last = 0.0;
};

template <class Rhs, class Lim>
double ssprk43_adaptive(Rhs&& rhs, Lim&& lim, double* u, size_t N, double t, double t_end,
                        const double* stops, int nstops, double abstol, double reltol,
                        int variant, AdaptiveStats* st) {
  AdaptiveStats stats;
  const int p = (variant & 4) ? 2 : 3;
  const double beta1 = 7.0 / (10.0 * p), beta2 = 2.0 / (5.0 * p);
  const double qmin = 0.2, qmax = 10.0, gamma = 0.9, qoldinit = 1e-4;
  const double p_init = (variant & 2) ? 4.0 : 3.0;
  std::vector<double> f0(N), k(N), tmp(N), w(N), unew(N), err(N);
  auto rms = [&](auto&& term) {
    double s = 0.0;
    for (size_t q = 0; q < N; ++q) {
      const double x = term(q);
      s += x * x;
    }
    return std::sqrt(s / (double)N);
  };
  rhs(u, f0.data(), t);
  ++stats.rhs_calls;
  // initial step
  double dt;
  {
    auto sk = [&](size_t q) { return abstol + std::fabs(u[q]) * reltol; };
    const double d0 = rms([&](size_t q) { return u[q] / sk(q); });
    const double d1 = rms([&](size_t q) { return f0[q] / sk(q); });
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    dt0 = std::min(dt0, t_end - t);
    for (size_t q = 0; q < N; ++q) tmp[q] = u[q] + dt0 * f0[q];
    rhs(tmp.data(), k.data(), t + dt0);
    ++stats.rhs_calls;
    const double d2 = rms([&](size_t q) { return (k[q] - f0[q]) / sk(q); }) / dt0;
    const double m = std::max(d1, d2);
    const double dt1 = m <= 1e-15 ? std::max(1e-6, dt0 * 1e-3)
                                  : std::pow(10.0, -(2.0 + std::log10(m)) / p_init);
    dt = std::min(std::min(100.0 * dt0, dt1), t_end - t);
  }
  stats.dt_first = dt;
  double qold = qoldinit;
  int next_stop = 0;
  while (t < t_end) {
    while (next_stop < nstops && stops[next_stop] <= t) ++next_stop;
    const double stop = next_stop < nstops ? std::min(stops[next_stop], t_end) : t_end;
    const double h_dt = std::min(dt, stop - t);
    const double h = 0.5 * h_dt;
    // stages
    for (size_t q = 0; q < N; ++q) tmp[q] = u[q] + h * f0[q];
    lim(tmp.data());
    rhs(tmp.data(), k.data(), t + h);
    for (size_t q = 0; q < N; ++q) tmp[q] = tmp[q] + h * k[q];
    lim(tmp.data());
    rhs(tmp.data(), k.data(), t + h_dt);
    for (size_t q = 0; q < N; ++q) {
      w[q] = tmp[q] + h * k[q];  // u2 + dt/2 f(u2)
      tmp[q] = (2.0 / 3.0) * u[q] + (1.0 / 3.0) * w[q];
    }
    lim(tmp.data());
    rhs(tmp.data(), k.data(), t + h);
    for (size_t q = 0; q < N; ++q) unew[q] = tmp[q] + h * k[q];
    lim(unew.data());
    stats.rhs_calls += 3;
    for (size_t q = 0; q < N; ++q) {
      const double lo = (1.0 / 3.0) * u[q] + (2.0 / 3.0) * w[q];
      const double ut = (variant & 1) ? lo : 0.5 * (lo + unew[q]);
      err[q] = unew[q] - ut;
    }
    const double eest = rms([&](size_t q) {
      return err[q] / (abstol + std::max(std::fabs(u[q]), std::fabs(unew[q])) * reltol);
    });
    const double q11 = std::pow(eest, beta1);
    if (eest <= 1.0) {
      double q = eest == 0.0 ? 1.0 / qmax : q11 / std::pow(qold, beta2);
      if (eest != 0.0) q = std::max(1.0 / qmax, std::min(1.0 / qmin, q / gamma));
      t = (h_dt == stop - t) ? stop : t + h_dt;
      for (size_t q2 = 0; q2 < N; ++q2) u[q2] = unew[q2];
      rhs(u, f0.data(), t);
      ++stats.rhs_calls;
      qold = std::max(eest, qoldinit);
      dt = h_dt / q;
      stats.dt_last = h_dt;
      ++stats.accepted;
    } else {
      dt = h_dt / std::min(1.0 / qmin, q11 / gamma);
      ++stats.rejected;
    }
  }
  if (st) *st = stats;
  return t;
}
#endif  // ORC_FLOP_COUNTING

}  // namespace orc
