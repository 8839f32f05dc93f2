// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// DGSEM right-hand side on a 2D curvilinear quadrilateral mesh, restated from
// the strong-form split DGSEM with flux differencing (Gassner, Winters, Kopriva,
// JCP 327 (2016); Trixi.jl `rhs!` phases as listed in TrixiAtmo's own override
// src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:8-71):
//   reset du -> volume integral (flux differencing, :134-234) -> interface flux
//   -> boundary flux -> surface integral -> apply_jacobian (:461-478) -> sources.
// The symmetric two-point flux uses the average of the two nodes' contravariant
// vectors as normal; the nonconservative part is 0.5 * sum_ii Dsplit[i,ii] g(...)
// (:188-234 restated for Cartesian metric terms).
//
// Layouts follow Trixi's column-major arrays (variable fastest):
//   u[v, i, j, e]                   -> u[((e*n + j)*n + i)*nv + v]
//   contravariant_vectors[c, d, i, j, e] -> Ja[(((e*n + j)*n + i)*2 + d)*2 + c]
//   inverse_jacobian[i, j, e]        -> invJ[(e*n + j)*n + i]
//   node_coordinates[c, i, j, e]     -> xy[((e*n + j)*n + i)*2 + c]
// Faces are 0 = xi-, 1 = xi+, 2 = eta-, 3 = eta+ (Trixi directions 1..4).
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>
#include "orc_basis.hpp"

namespace orc {

struct Mesh2D {
  int n = 0, nelem = 0;
  std::vector<double> Ja, invJ, xy;
  // interfaces: primary (elem, face), secondary (elem, face), flip of the
  // secondary's face-node order
  std::vector<int> if_e0, if_f0, if_e1, if_f1, if_flip;
  // boundary faces: elem, face, kind (1 = slip wall, StructuredMesh semantics;
  // 2 = slip wall, P4estMesh semantics; 4 = Dirichlet, P4estMesh semantics)
  std::vector<int> bd_e, bd_f, bd_kind;
  // Dirichlet states [B][n][nv] of the kind-4 faces (Trixi's
  // BoundaryConditionDirichlet: surface flux of the inner and the given state)
  std::vector<double> bd_values;
};

// Face node (i, j) of face f at face index l.
inline void face_node(int f, int l, int n, int& i, int& j) {
  switch (f) {
    case 0: i = 0; j = l; break;
    case 1: i = n - 1; j = l; break;
    case 2: i = l; j = 0; break;
    default: i = l; j = n - 1; break;
  }
}

// StructuredMesh on a rectangle [x0,x1] x [y0,y1] with nx x ny cells; node
// coordinates by the affine cell map, metric terms by collocation
// differentiation of the node coordinates (Kopriva 2006 for 2D:
// Ja^1 = (y_eta, -x_eta), Ja^2 = (-y_xi, x_xi), J = x_xi y_eta - x_eta y_xi).
inline Mesh2D structured_rectangle(const Basis& b, int nx, int ny, double x0, double x1,
                                   double y0, double y1, bool periodic_x, bool periodic_y,
                                   int wall_kind = 1) {
  Mesh2D m;
  const int n = b.n;
  m.n = n;
  m.nelem = nx * ny;
  m.xy.assign((size_t)m.nelem * n * n * 2, 0.0);
  m.Ja.assign((size_t)m.nelem * n * n * 4, 0.0);
  m.invJ.assign((size_t)m.nelem * n * n, 0.0);
  const double dxr = 2.0 / nx, dyr = 2.0 / ny;
  for (int cy = 0; cy < ny; ++cy)
    for (int cx = 0; cx < nx; ++cx) {
      const int e = cx + nx * cy;
      const double ox = -1.0 + cx * dxr + 0.5 * dxr, oy = -1.0 + cy * dyr + 0.5 * dyr;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double xi = ox + 0.5 * dxr * b.x[i], eta = oy + 0.5 * dyr * b.x[j];
          const size_t k = ((size_t)(e * n + j) * n + i) * 2;
          m.xy[k + 0] = x0 + 0.5 * (xi + 1.0) * (x1 - x0);
          m.xy[k + 1] = y0 + 0.5 * (eta + 1.0) * (y1 - y0);
        }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double x_xi = 0, y_xi = 0, x_eta = 0, y_eta = 0;
          for (int k = 0; k < n; ++k) {
            const size_t a = ((size_t)(e * n + j) * n + k) * 2;
            const size_t c = ((size_t)(e * n + k) * n + i) * 2;
            x_xi += b.d(i, k) * m.xy[a];
            y_xi += b.d(i, k) * m.xy[a + 1];
            x_eta += b.d(j, k) * m.xy[c];
            y_eta += b.d(j, k) * m.xy[c + 1];
          }
          const size_t q = ((size_t)(e * n + j) * n + i) * 4;
          m.Ja[q + 0] = y_eta;   // Ja^1_x
          m.Ja[q + 1] = -x_eta;  // Ja^1_y
          m.Ja[q + 2] = -y_xi;   // Ja^2_x
          m.Ja[q + 3] = x_xi;    // Ja^2_y
          m.invJ[(size_t)(e * n + j) * n + i] = 1.0 / (x_xi * y_eta - x_eta * y_xi);
        }
    }
  for (int cy = 0; cy < ny; ++cy)
    for (int cx = 0; cx < nx; ++cx) {
      const int e = cx + nx * cy;
      if (cx < nx - 1 || periodic_x) {
        m.if_e0.push_back(e); m.if_f0.push_back(1);
        m.if_e1.push_back((cx + 1) % nx + nx * cy); m.if_f1.push_back(0);
        m.if_flip.push_back(0);
      }
      if (cy < ny - 1 || periodic_y) {
        m.if_e0.push_back(e); m.if_f0.push_back(3);
        m.if_e1.push_back(cx + nx * ((cy + 1) % ny)); m.if_f1.push_back(2);
        m.if_flip.push_back(0);
      }
      if (!periodic_x && cx == 0) { m.bd_e.push_back(e); m.bd_f.push_back(0); m.bd_kind.push_back(wall_kind); }
      if (!periodic_x && cx == nx - 1) { m.bd_e.push_back(e); m.bd_f.push_back(1); m.bd_kind.push_back(wall_kind); }
      if (!periodic_y && cy == 0) { m.bd_e.push_back(e); m.bd_f.push_back(2); m.bd_kind.push_back(wall_kind); }
      if (!periodic_y && cy == ny - 1) { m.bd_e.push_back(e); m.bd_f.push_back(3); m.bd_kind.push_back(wall_kind); }
    }
  return m;
}

template <class Phys>
struct DG2D {
  using State = typename Phys::State;
  static constexpr int nv = Phys::nv;
  const Phys& phys;
  const Basis& b;
  const Mesh2D& m;
  int n;
  std::vector<double> sfv;  // outward surface flux [e][face][l][v]

  DG2D(const Phys& p, const Basis& bb, const Mesh2D& mm) : phys(p), b(bb), m(mm), n(bb.n) {
    sfv.assign((size_t)m.nelem * 4 * n * nv, 0.0);
  }

  size_t node(int i, int j, int e) const { return (size_t)(e * n + j) * n + i; }
  State get(const double* u, int i, int j, int e) const {
    State s;
    for (int v = 0; v < nv; ++v) s[v] = u[node(i, j, e) * nv + v];
    return s;
  }
  void ja(int d, int i, int j, int e, double* out) const {
    const size_t q = node(i, j, e) * 4 + 2 * d;
    out[0] = m.Ja[q];
    out[1] = m.Ja[q + 1];
  }
  double& sf(int e, int f, int l, int v) { return sfv[(((size_t)e * 4 + f) * n + l) * nv + v]; }

  bool weak_form = false;  // VolumeIntegralWeakForm instead of flux differencing

  // weak form (:100-130 pattern): du[ii] += D_hat[ii, i] * f~(u_i)
  void volume_integral_weak(const double* u, double* du, int e) const {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State ui = get(u, i, j, e);
        double a1[2], a2[2];
        ja(0, i, j, e, a1);
        ja(1, i, j, e, a2);
        const State f1 = phys.flux(ui, a1), f2 = phys.flux(ui, a2);
        for (int ii = 0; ii < n; ++ii)
          for (int v = 0; v < nv; ++v) du[node(ii, j, e) * nv + v] += b.dh(ii, i) * f1[v];
        for (int jj = 0; jj < n; ++jj)
          for (int v = 0; v < nv; ++v) du[node(i, jj, e) * nv + v] += b.dh(jj, j) * f2[v];
      }
  }

  void volume_integral(const double* u, double* du, int e) const {
    if (weak_form) {
      volume_integral_weak(u, du, e);
      return;
    }
    // symmetric two-point flux, each pair once (:148-181 pattern)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State ui = get(u, i, j, e);
        double ja_i[2], ja_ii[2], navg[2];
        ja(0, i, j, e, ja_i);
        for (int ii = i + 1; ii < n; ++ii) {
          const State uii = get(u, ii, j, e);
          ja(0, ii, j, e, ja_ii);
          navg[0] = 0.5 * (ja_i[0] + ja_ii[0]);
          navg[1] = 0.5 * (ja_i[1] + ja_ii[1]);
          const State f = phys.volume_flux(ui, uii, navg);
          for (int v = 0; v < nv; ++v) {
            du[node(i, j, e) * nv + v] += b.ds(i, ii) * f[v];
            du[node(ii, j, e) * nv + v] += b.ds(ii, i) * f[v];
          }
        }
        ja(1, i, j, e, ja_i);
        for (int jj = j + 1; jj < n; ++jj) {
          const State ujj = get(u, i, jj, e);
          ja(1, i, jj, e, ja_ii);
          navg[0] = 0.5 * (ja_i[0] + ja_ii[0]);
          navg[1] = 0.5 * (ja_i[1] + ja_ii[1]);
          const State f = phys.volume_flux(ui, ujj, navg);
          for (int v = 0; v < nv; ++v) {
            du[node(i, j, e) * nv + v] += b.ds(j, jj) * f[v];
            du[node(i, jj, e) * nv + v] += b.ds(jj, j) * f[v];
          }
        }
      }
    if (!Phys::has_noncons) return;
    // nonconservative part, 0.5 * sum over the full line (:202-231 pattern)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const State ui = get(u, i, j, e);
        double ja_i[2], ja_ii[2], navg[2];
        State acc{};
        ja(0, i, j, e, ja_i);
        for (int ii = 0; ii < n; ++ii) {
          const State uii = get(u, ii, j, e);
          ja(0, ii, j, e, ja_ii);
          navg[0] = 0.5 * (ja_i[0] + ja_ii[0]);
          navg[1] = 0.5 * (ja_i[1] + ja_ii[1]);
          const State g = phys.volume_noncons(ui, uii, navg);
          for (int v = 0; v < nv; ++v) acc[v] += b.ds(i, ii) * g[v];
        }
        ja(1, i, j, e, ja_i);
        for (int jj = 0; jj < n; ++jj) {
          const State ujj = get(u, i, jj, e);
          ja(1, i, jj, e, ja_ii);
          navg[0] = 0.5 * (ja_i[0] + ja_ii[0]);
          navg[1] = 0.5 * (ja_i[1] + ja_ii[1]);
          const State g = phys.volume_noncons(ui, ujj, navg);
          for (int v = 0; v < nv; ++v) acc[v] += b.ds(j, jj) * g[v];
        }
        for (int v = 0; v < nv; ++v) du[node(i, j, e) * nv + v] += 0.5 * acc[v];
      }
  }

  // outward normal (unnormalised) of face f at face index l of element e
  void outward_normal(int e, int f, int l, double* nrm) const {
    int i, j;
    face_node(f, l, n, i, j);
    ja(f / 2, i, j, e, nrm);
    const double s = (m.invJ[node(i, j, e)] < 0 ? -1.0 : 1.0) * ((f % 2) ? 1.0 : -1.0);
    nrm[0] *= s;
    nrm[1] *= s;
  }

  void interface_flux(const double* u, int k) {
    const int e0 = m.if_e0[k], f0 = m.if_f0[k], e1 = m.if_e1[k], f1 = m.if_f1[k];
    for (int l = 0; l < n; ++l) {
      const int l1 = m.if_flip[k] ? n - 1 - l : l;
      int i0, j0, i1, j1;
      face_node(f0, l, n, i0, j0);
      face_node(f1, l1, n, i1, j1);
      const State ul = get(u, i0, j0, e0), ur = get(u, i1, j1, e1);
      double nrm[2];
      outward_normal(e0, f0, l, nrm);
      const State fl = phys.surface_flux(ul, ur, nrm);
      const State g0 = phys.surface_noncons(ul, ur, nrm);
      const State g1 = phys.surface_noncons(ur, ul, nrm);
      for (int v = 0; v < nv; ++v) {
        sf(e0, f0, l, v) = fl[v] + 0.5 * g0[v];
        sf(e1, f1, l1, v) = -(fl[v] + 0.5 * g1[v]);
      }
    }
  }

  void boundary_flux(const double* u, int k, double t) {
    const int e = m.bd_e[k], f = m.bd_f[k];
    for (int l = 0; l < n; ++l) {
      int i, j;
      face_node(f, l, n, i, j);
      const State ui = get(u, i, j, e);
      double nrm[2];
      State fl;
      if (m.bd_kind[k] == 1) {
        // StructuredMesh: normal in the +xi/+eta sense, flux stored likewise
        ja(f / 2, i, j, e, nrm);
        const double sj = m.invJ[node(i, j, e)] < 0 ? -1.0 : 1.0;
        nrm[0] *= sj; nrm[1] *= sj;
        fl = phys.bc_structured(ui, nrm, f + 1);
        const double s = sj * ((f % 2) ? 1.0 : -1.0);  // to outward
        for (int v = 0; v < nv; ++v) sf(e, f, l, v) = s * fl[v];
      } else if (m.bd_kind[k] == 4) {
        // BoundaryConditionDirichlet, P4estMesh method: surface flux (plus half
        // the nonconservative surface flux) of the inner and the boundary state
        outward_normal(e, f, l, nrm);
        State ub;
        for (int v = 0; v < nv; ++v) ub[v] = m.bd_values[((size_t)k * n + l) * nv + v];
        fl = phys.surface_flux(ui, ub, nrm);
        if (Phys::has_noncons) {
          const State g = phys.surface_noncons(ui, ub, nrm);
          for (int v = 0; v < nv; ++v) fl[v] += 0.5 * g[v];
        }
        for (int v = 0; v < nv; ++v) sf(e, f, l, v) = fl[v];
      } else {
        outward_normal(e, f, l, nrm);
        fl = phys.bc_normal(ui, nrm);
        for (int v = 0; v < nv; ++v) sf(e, f, l, v) = fl[v];
      }
    }
    (void)t;
  }

  void surface_jacobian_sources(const double* u, double* du, int e, double t) const {
    for (int f = 0; f < 4; ++f)
      for (int l = 0; l < n; ++l) {
        int i, j;
        face_node(f, l, n, i, j);
        const double winv = 1.0 / b.w[(f % 2) ? n - 1 : 0];
        for (int v = 0; v < nv; ++v)
          du[node(i, j, e) * nv + v] += sfv[(((size_t)e * 4 + f) * n + l) * nv + v] * winv;
      }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double f = -m.invJ[node(i, j, e)];
        for (int v = 0; v < nv; ++v) du[node(i, j, e) * nv + v] *= f;
      }
    if (Phys::has_sources) {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const State ui = get(u, i, j, e);
          const double* x = &m.xy[node(i, j, e) * 2];
          State s = phys.source(ui, x, t);
          for (int v = 0; v < nv; ++v) du[node(i, j, e) * nv + v] += s[v];
        }
    }
  }

  void rhs(const double* u, double* du, double t) {
    const size_t N = (size_t)m.nelem * n * n * nv;
    std::fill(du, du + N, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < m.nelem; ++e) volume_integral(u, du, e);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < (int)m.if_e0.size(); ++k) interface_flux(u, k);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < (int)m.bd_e.size(); ++k) boundary_flux(u, k, t);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < m.nelem; ++e) surface_jacobian_sources(u, du, e, t);
  }

  // max_dt, restating src/callbacks_step/stepsize_dg2d.jl:5-44 for 2 components
  double max_dt(const double* u) const {
    double max_scaled = std::nextafter(0.0, 1.0);
#pragma omp parallel for reduction(max : max_scaled)
    for (int e = 0; e < m.nelem; ++e) {
      double ml1 = 0, ml2 = 0;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double l1, l2, a[2], c[2];
          phys.max_abs_speeds(get(u, i, j, e), l1, l2);
          ja(0, i, j, e, a);
          ja(1, i, j, e, c);
          const double ij = std::fabs(m.invJ[node(i, j, e)]);
          ml1 = std::max(ml1, std::fabs(a[0] * l1 + a[1] * l2) * ij);
          ml2 = std::max(ml2, std::fabs(c[0] * l1 + c[1] * l2) * ij);
        }
      max_scaled = std::max(max_scaled, ml1 + ml2);
    }
    return 2.0 / (n * max_scaled);
  }
};

}  // namespace orc
