// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Covariant shallow-water equations on a 2D manifold (the cubed sphere),
// restating src/equations/covariant_shallow_water.jl,
// src/equations/covariant_shallow_water_split.jl, the Lax-Friedrichs
// dissipation of src/equations/equations.jl:243-257, and the covariant DGSEM
// pipeline of src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl
// (weak form :98-131, flux differencing :135-234, interface fluxes with the
// neighbour state transformed through global coordinates :239-432, sources
// :435-452, apply_jacobian :461-478) and the covariant max_dt of
// src/callbacks_step/stepsize_dg2d.jl:47-71.
// Auxiliary variables per node: the reference's 26-entry layout
// (src/equations/equations.jl:139-215).
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "orc_basis.hpp"
#include "orc_dg2d.hpp"

namespace orc {

struct CovSWE {
  using State = std::array<double, 3>;
  double g = 9.80616, omega = 7.292e-5;
  bool split = false;
  // aux accessors (0-based offsets of the reference layout)
  static double J(const double* a) { return a[12]; }
  static double Gcov(const double* a, int i, int j) {
    return (i == 0 && j == 0) ? a[13] : (i == 1 && j == 1) ? a[15] : a[14];
  }
  static double Gcon(const double* a, int i, int j) {
    return (i == 0 && j == 0) ? a[16] : (i == 1 && j == 1) ? a[18] : a[17];
  }
  static double hs(const double* a) { return a[19]; }
  // Christoffel symbols Gamma^k_ij as a symmetric matrix
  static double Gam(const double* a, int k, int i, int j) {
    const double* c = a + 20 + 3 * k;
    return (i == 0 && j == 0) ? c[0] : (i == 1 && j == 1) ? c[2] : c[1];
  }
  // covariant basis A[r][c] (3x2, column-major at a[0..5]); contravariant
  // basis Acon[r][c] (2x3, column-major at a[6..11])
  static double A(const double* a, int r, int c) { return a[c * 3 + r]; }
  static double Acon(const double* a, int r, int c) { return a[6 + c * 2 + r]; }

  // state of another node expressed in the contravariant basis of `to`
  // (contravariant2global then global2contravariant)
  static State transform(const State& u, const double* from, const double* to) {
    double gl[3];
    for (int r = 0; r < 3; ++r) gl[r] = A(from, r, 0) * u[1] + A(from, r, 1) * u[2];
    State s;
    s[0] = u[0];
    for (int r = 0; r < 2; ++r) s[r + 1] = Acon(to, r, 0) * gl[0] + Acon(to, r, 1) * gl[1] + Acon(to, r, 2) * gl[2];
    return s;
  }

  // flux(u, aux, orientation): covariant_shallow_water.jl:155-176 (standard),
  // covariant_shallow_water_split.jl:64-72 (split: no pressure term)
  State flux(const State& u, const double* a, int o) const {
    const double Jv = J(a);
    const double vo = u[1 + o] / u[0];
    if (split) {
      const double m = Jv * u[1 + o];
      return {m, m * (u[1] / u[0]), m * (u[2] / u[0])};
    }
    const double gt = 0.5 * g * u[0] * u[0];
    return {Jv * u[1 + o], Jv * (u[1] * vo + Gcon(a, 0, o) * gt), Jv * (u[2] * vo + Gcon(a, 1, o) * gt)};
  }

  // flux_ec (split, :101-116)
  static State flux_ec(const State& ua, const State& ub, const double* aa, const double* ab, int o) {
    const double m = 0.5 * (J(aa) * ua[1 + o] + J(ab) * ub[1 + o]);
    return {m, 0.5 * (ua[1] / ua[0] + ub[1] / ub[0]) * m, 0.5 * (ua[2] / ua[0] + ub[2] / ub[0]) * m};
  }

  State flux_central(const State& ua, const State& ub, const double* aa, const double* ab, int o) const {
    const State fa = flux(ua, aa, o), fb = flux(ub, ab, o);
    return {0.5 * (fa[0] + fb[0]), 0.5 * (fa[1] + fb[1]), 0.5 * (fa[2] + fb[2])};
  }

  // flux_nonconservative_ec (split, :142-162)
  State noncons_ec(const State& ua, const State& ub, const double* aa, const double* ab, int o) const {
    const double jump = hs(ab) - hs(aa);
    const double vb[2] = {ub[1] / ub[0], ub[2] / ub[0]};
    const double vcov[2] = {Gcov(ab, 0, 0) * vb[0] + Gcov(ab, 0, 1) * vb[1],
                            Gcov(ab, 1, 0) * vb[0] + Gcov(ab, 1, 1) * vb[1]};
    State f{0.0, 0.0, 0.0};
    for (int r = 0; r < 2; ++r) {
      const double geo = 0.5 * ua[1 + o] * (Gcon(aa, r, 0) * vcov[0] + Gcon(aa, r, 1) * vcov[1] - vb[r]);
      const double pr = g * Gcon(aa, r, o) * ua[0] * (ub[0] + jump);
      f[1 + r] = J(aa) * (geo + pr);
    }
    return f;
  }

  // flux_nonconservative_surface_simplified (split, :205-220)
  State noncons_simplified(const State& ua, const State& ub, const double* aa, const double*, int o) const {
    State f{0.0, 0.0, 0.0};
    for (int r = 0; r < 2; ++r) f[1 + r] = J(aa) * (g * Gcon(aa, r, o) * ua[0] * ub[0]);
    return f;
  }

  // max_abs_speed with an orientation (covariant_shallow_water.jl:246-265)
  double max_abs_speed(const State& ua, const State& ub, const double* aa, const double* ab, int o) const {
    return std::max(std::fabs(ua[1 + o] / ua[0]) + std::sqrt(Gcon(aa, o, o) * ua[0] * g),
                    std::fabs(ub[1 + o] / ub[0]) + std::sqrt(Gcon(ab, o, o) * ub[0] * g));
  }

  // source_terms_geometric_coriolis: standard :216-243, split :273-302
  State source(const State& u, const double* x, const double* a) const {
    const double hv[2] = {u[1], u[2]};
    const double v[2] = {u[1] / u[0], u[2] / u[0]};
    const double f = 2.0 * omega * x[2] / std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    double sg[2];
    if (!split) {
      const double gt = 0.5 * g * u[0] * u[0];
      for (int k = 0; k < 2; ++k) {
        double s = 0.0;
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) s += Gam(a, k, i, j) * (hv[i] * v[j] + gt * Gcon(a, i, j));
        sg[k] = s;
      }
    } else {
      double T[2][2], C[2][2];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) T[i][j] = hv[i] * v[j];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) C[i][j] = Gcov(a, i, 0) * T[0][j] + Gcov(a, i, 1) * T[1][j];
      double w[2];
      for (int i = 0; i < 2; ++i)
        w[i] = (Gam(a, 0, i, 0) * C[0][0] + Gam(a, 0, i, 1) * C[0][1]) +
               (Gam(a, 1, i, 0) * C[1][0] + Gam(a, 1, i, 1) * C[1][1]);
      for (int k = 0; k < 2; ++k) {
        double s = 0.0;
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j) s += Gam(a, k, i, j) * T[i][j];
        sg[k] = 0.5 * (s - (Gcon(a, k, 0) * w[0] + Gcon(a, k, 1) * w[1]));
      }
    }
    const double Jv = J(a);
    const double s1 = sg[0] + f * Jv * (Gcon(a, 0, 1) * hv[0] - Gcon(a, 0, 0) * hv[1]);
    const double s2 = sg[1] + f * Jv * (Gcon(a, 1, 1) * hv[0] - Gcon(a, 1, 0) * hv[1]);
    return {0.0, -s1, -s2};
  }

  void max_abs_speeds(const State& u, const double* a, double& l1, double& l2) const {
    l1 = std::fabs(u[1] / u[0]) + std::sqrt(Gcon(a, 0, 0) * u[0] * g);
    l2 = std::fabs(u[2] / u[0]) + std::sqrt(Gcon(a, 1, 1) * u[0] * g);
  }
};

// Flux choices.  Volume: weak form, or flux differencing with a symmetric
// flux (central / ec) and optionally flux_nonconservative_ec.  Surface: a
// symmetric flux (central / ec) plus optional local Lax-Friedrichs dissipation,
// plus an optional nonconservative flux (ec / surface_simplified).
struct CovFluxes {
  int volume = 0;   // 0 weak form, 1 flux differencing
  int vol_sym = 0;  // 0 flux_central, 1 flux_ec
  int vol_nc = 0;   // 0 none, 1 flux_nonconservative_ec
  int surf_sym = 0; // 0 flux_central, 1 flux_ec
  int surf_diss = 1;// 0 none, 1 DissipationLocalLaxFriedrichs
  int surf_nc = 0;  // 0 none, 1 flux_nonconservative_ec, 2 surface_simplified
};

struct CovDG {
  using State = CovSWE::State;
  CovSWE eq;
  CovFluxes fx;
  Basis b;
  int n = 0, nelem = 0;
  std::vector<double> aux, xyz;
  std::vector<int> if_e0, if_f0, if_e1, if_f1, if_flip;
  std::vector<double> sfv;

  size_t node(int i, int j, int e) const { return (size_t)(e * n + j) * n + i; }
  State get(const double* u, int i, int j, int e) const {
    const double* p = u + node(i, j, e) * 3;
    return {p[0], p[1], p[2]};
  }
  const double* ax(int i, int j, int e) const { return &aux[node(i, j, e) * 26]; }

  State vol_sym(const State& a, const State& c, const double* aa, const double* ac, int o) const {
    return fx.vol_sym == 1 ? CovSWE::flux_ec(a, c, aa, ac, o) : eq.flux_central(a, c, aa, ac, o);
  }

  void volume(const double* u, double* du, int e) const {
    if (fx.volume == 0) {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const State ui = get(u, i, j, e);
          const State f1 = eq.flux(ui, ax(i, j, e), 0), f2 = eq.flux(ui, ax(i, j, e), 1);
          for (int ii = 0; ii < n; ++ii)
            for (int v = 0; v < 3; ++v) du[node(ii, j, e) * 3 + v] += b.dh(ii, i) * f1[v];
          for (int jj = 0; jj < n; ++jj)
            for (int v = 0; v < 3; ++v) du[node(i, jj, e) * 3 + v] += b.dh(jj, j) * f2[v];
        }
      return;
    }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State ui = get(u, i, j, e);
        for (int ii = i + 1; ii < n; ++ii) {
          const State f = vol_sym(ui, get(u, ii, j, e), ax(i, j, e), ax(ii, j, e), 0);
          for (int v = 0; v < 3; ++v) {
            du[node(i, j, e) * 3 + v] += b.ds(i, ii) * f[v];
            du[node(ii, j, e) * 3 + v] += b.ds(ii, i) * f[v];
          }
        }
        for (int jj = j + 1; jj < n; ++jj) {
          const State f = vol_sym(ui, get(u, i, jj, e), ax(i, j, e), ax(i, jj, e), 1);
          for (int v = 0; v < 3; ++v) {
            du[node(i, j, e) * 3 + v] += b.ds(j, jj) * f[v];
            du[node(i, jj, e) * 3 + v] += b.ds(jj, j) * f[v];
          }
        }
      }
    if (fx.vol_nc == 0) return;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State ui = get(u, i, j, e);
        State acc{0.0, 0.0, 0.0};
        for (int ii = 0; ii < n; ++ii) {
          const State g = eq.noncons_ec(ui, get(u, ii, j, e), ax(i, j, e), ax(ii, j, e), 0);
          for (int v = 0; v < 3; ++v) acc[v] += b.ds(i, ii) * g[v];
        }
        for (int jj = 0; jj < n; ++jj) {
          const State g = eq.noncons_ec(ui, get(u, i, jj, e), ax(i, j, e), ax(i, jj, e), 1);
          for (int v = 0; v < 3; ++v) acc[v] += b.ds(j, jj) * g[v];
        }
        for (int v = 0; v < 3; ++v) du[node(i, j, e) * 3 + v] += 0.5 * acc[v];
      }
  }

  // surface_flux (+ 0.5 nonconservative) of states a (left) and c (right)
  // with both sides' auxiliary variables those of `own`
  State surface(const State& a, const State& c, const double* own, int o) const {
    State f = fx.surf_sym == 1 ? CovSWE::flux_ec(a, c, own, own, o) : eq.flux_central(a, c, own, own, o);
    if (fx.surf_diss) {
      const double lam = eq.max_abs_speed(a, c, own, own, o);
      for (int v = 0; v < 3; ++v) f[v] += -0.5 * CovSWE::J(own) * lam * (c[v] - a[v]);
    }
    if (fx.surf_nc) {
      const State g = fx.surf_nc == 1 ? eq.noncons_ec(a, c, own, own, o) : eq.noncons_simplified(a, c, own, own, o);
      for (int v = 0; v < 3; ++v) f[v] += 0.5 * g[v];
    }
    return f;
  }

  // outward flux of one side: direction index (1-based) f + 1 odd <=> f even
  State side_flux(const State& mine, const State& other_in_mine, const double* own, int f) const {
    const int o = f >> 1;
    if ((f & 1) == 0) {
      const State s = surface(other_in_mine, mine, own, o);
      return {-s[0], -s[1], -s[2]};
    }
    return surface(mine, other_in_mine, own, o);
  }

  void interface(const double* u, int k) {
    const int e0 = if_e0[k], f0 = if_f0[k], e1 = if_e1[k], f1 = if_f1[k];
    for (int l = 0; l < n; ++l) {
      const int l1 = if_flip[k] ? n - 1 - l : l;
      int i0, j0, i1, j1;
      face_node(f0, l, n, i0, j0);
      face_node(f1, l1, n, i1, j1);
      const State ul = get(u, i0, j0, e0), ur = get(u, i1, j1, e1);
      const double *al = ax(i0, j0, e0), *ar = ax(i1, j1, e1);
      const State fp = side_flux(ul, CovSWE::transform(ur, ar, al), al, f0);
      const State fs = side_flux(ur, CovSWE::transform(ul, al, ar), ar, f1);
      for (int v = 0; v < 3; ++v) {
        sfv[(((size_t)e0 * 4 + f0) * n + l) * 3 + v] = fp[v];
        sfv[(((size_t)e1 * 4 + f1) * n + l1) * 3 + v] = fs[v];
      }
    }
  }

  void surface_jacobian_sources(const double* u, double* du, int e) const {
    for (int f = 0; f < 4; ++f)
      for (int l = 0; l < n; ++l) {
        int i, j;
        face_node(f, l, n, i, j);
        const double winv = 1.0 / b.w[(f % 2) ? n - 1 : 0];
        for (int v = 0; v < 3; ++v)
          du[node(i, j, e) * 3 + v] += sfv[(((size_t)e * 4 + f) * n + l) * 3 + v] * winv;
      }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double fac = -1.0 / CovSWE::J(ax(i, j, e));
        for (int v = 0; v < 3; ++v) du[node(i, j, e) * 3 + v] *= fac;
      }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State s = eq.source(get(u, i, j, e), &xyz[node(i, j, e) * 3], ax(i, j, e));
        for (int v = 0; v < 3; ++v) du[node(i, j, e) * 3 + v] += s[v];
      }
  }

  void rhs(const double* u, double* du) {
    const size_t N = (size_t)nelem * n * n * 3;
    std::fill(du, du + N, 0.0);
    if (sfv.size() != (size_t)nelem * 4 * n * 3) sfv.assign((size_t)nelem * 4 * n * 3, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nelem; ++e) volume(u, du, e);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < (int)if_e0.size(); ++k) interface(u, k);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nelem; ++e) surface_jacobian_sources(u, du, e);
  }

  double max_dt(const double* u) const {
    double ms = std::nextafter(0.0, 1.0);
#pragma omp parallel for reduction(max : ms)
    for (int e = 0; e < nelem; ++e) {
      double m1 = 0.0, m2 = 0.0;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double l1, l2;
          eq.max_abs_speeds(get(u, i, j, e), ax(i, j, e), l1, l2);
          m1 = std::max(m1, l1);
          m2 = std::max(m2, l2);
        }
      ms = std::max(ms, m1 + m2);
    }
    return 2.0 / (n * ms);
  }
};

}  // namespace orc
