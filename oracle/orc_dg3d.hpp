// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// DGSEM right-hand side on a 3D curvilinear hexahedral mesh with general
// (P4estMesh-like) connectivity: the same phases as the 2D oracle
// (orc_dg2d.hpp), with three reference directions and face-to-face
// orientations.  Geometry (contravariant vectors, inverse Jacobian, node
// coordinates) and connectivity are inputs, built by the host mirror exactly
// as they are passed to the C ABI:
//   u[v, i, j, k, e]                          -> u[(((e*n + k)*n + j)*n + i)*nv + v]
//   contravariant_vectors[c, d, i, j, k, e]    -> Ja[(node*3 + d)*3 + c]
//   inverse_jacobian[i, j, k, e], node_coordinates[c, i, j, k, e]
// Faces: 0/1 = xi-/+, 2/3 = eta-/+, 4/5 = zeta-/+.  Face-local indices
// (l1, l2) are (j, k), (i, k), (i, j) for the xi, eta, zeta faces.  The
// orientation code o maps the primary's (l1, l2) to the secondary's (s1, s2):
// swap when o & 1, then s1 = n-1-s1 when o & 2, s2 = n-1-s2 when o & 4.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>
#include "orc_basis.hpp"

namespace orc {

struct Mesh3D {
  int n = 0, nelem = 0;
  const double* Ja = nullptr;
  const double* invJ = nullptr;
  const double* xyz = nullptr;
  std::vector<int> if_e0, if_f0, if_e1, if_f1, if_orient;
  std::vector<int> bd_e, bd_f;
};

inline void face_node3d(int f, int l1, int l2, int n, int& i, int& j, int& k) {
  const int end = (f & 1) ? n - 1 : 0;
  switch (f >> 1) {
    case 0: i = end; j = l1; k = l2; break;
    case 1: i = l1; j = end; k = l2; break;
    default: i = l1; j = l2; k = end; break;
  }
}

inline void orient_map(int o, int l1, int l2, int n, int& s1, int& s2) {
  int a = l1, b = l2;
  if (o & 1) std::swap(a, b);
  if (o & 2) a = n - 1 - a;
  if (o & 4) b = n - 1 - b;
  s1 = a;
  s2 = b;
}

template <class Phys>
struct DG3D {
  using State = typename Phys::State;
  static constexpr int nv = Phys::nv;
  const Phys& phys;
  const Basis& b;
  const Mesh3D& m;
  int n;
  std::vector<double> sfv;  // outward surface flux [e][face][l2][l1][v]

  DG3D(const Phys& p, const Basis& bb, const Mesh3D& mm) : phys(p), b(bb), m(mm), n(bb.n) {
    sfv.assign((size_t)m.nelem * 6 * n * n * nv, 0.0);
  }

  size_t node(int i, int j, int k, int e) const { return (((size_t)e * n + k) * n + j) * n + i; }
  State get(const double* u, size_t q) const {
    State s;
    for (int v = 0; v < nv; ++v) s[v] = u[q * nv + v];
    return s;
  }
  void ja(int d, size_t q, double* out) const {
    for (int c = 0; c < 3; ++c) out[c] = m.Ja[(q * 3 + d) * 3 + c];
  }
  size_t line_node(int d, int a, int p1, int p2, int e) const {
    // node a along direction d; (p1, p2) index the other two directions
    if (d == 0) return node(a, p1, p2, e);
    if (d == 1) return node(p1, a, p2, e);
    return node(p1, p2, a, e);
  }
  double& sf(int e, int f, int l1, int l2, int v) {
    return sfv[((((size_t)e * 6 + f) * n + l2) * n + l1) * nv + v];
  }

  void volume_integral(const double* u, double* du, int e) const {
    for (int d = 0; d < 3; ++d)
      for (int p2 = 0; p2 < n; ++p2)
        for (int p1 = 0; p1 < n; ++p1)
          for (int a = 0; a < n; ++a) {
            const size_t qa = line_node(d, a, p1, p2, e);
            const State ua = get(u, qa);
            double ja_a[3], ja_b[3], nav[3];
            ja(d, qa, ja_a);
            for (int bb = a + 1; bb < n; ++bb) {
              const size_t qb = line_node(d, bb, p1, p2, e);
              const State ub = get(u, qb);
              ja(d, qb, ja_b);
              for (int c = 0; c < 3; ++c) nav[c] = 0.5 * (ja_a[c] + ja_b[c]);
              const State f = phys.volume_flux(ua, ub, nav);
              for (int v = 0; v < nv; ++v) {
                du[qa * nv + v] += b.ds(a, bb) * f[v];
                du[qb * nv + v] += b.ds(bb, a) * f[v];
              }
            }
          }
    if (!Phys::has_noncons) return;
    for (int kk = 0; kk < n; ++kk)
      for (int jj = 0; jj < n; ++jj)
        for (int ii = 0; ii < n; ++ii) {
          const size_t q = node(ii, jj, kk, e);
          const State uq = get(u, q);
          State acc{};
          const int idx[3] = {ii, jj, kk};
          for (int d = 0; d < 3; ++d) {
            const int p1 = d == 0 ? jj : ii;
            const int p2 = d == 2 ? jj : kk;
            double ja_a[3], ja_b[3], nav[3];
            ja(d, q, ja_a);
            for (int bb = 0; bb < n; ++bb) {
              const size_t qb = line_node(d, bb, p1, p2, e);
              ja(d, qb, ja_b);
              for (int c = 0; c < 3; ++c) nav[c] = 0.5 * (ja_a[c] + ja_b[c]);
              const State g = phys.volume_noncons(uq, get(u, qb), nav);
              for (int v = 0; v < nv; ++v) acc[v] += b.ds(idx[d], bb) * g[v];
            }
          }
          for (int v = 0; v < nv; ++v) du[q * nv + v] += 0.5 * acc[v];
        }
  }

  void outward_normal(int e, int f, int l1, int l2, double* nrm) const {
    int i, j, k;
    face_node3d(f, l1, l2, n, i, j, k);
    const size_t q = node(i, j, k, e);
    ja(f >> 1, q, nrm);
    const double s = (m.invJ[q] < 0 ? -1.0 : 1.0) * ((f & 1) ? 1.0 : -1.0);
    for (int c = 0; c < 3; ++c) nrm[c] *= s;
  }

  void interface_flux(const double* u, int it) {
    const int e0 = m.if_e0[it], f0 = m.if_f0[it], e1 = m.if_e1[it], f1 = m.if_f1[it];
    for (int l2 = 0; l2 < n; ++l2)
      for (int l1 = 0; l1 < n; ++l1) {
        int s1, s2, i0, j0, k0, i1, j1, k1;
        orient_map(m.if_orient[it], l1, l2, n, s1, s2);
        face_node3d(f0, l1, l2, n, i0, j0, k0);
        face_node3d(f1, s1, s2, n, i1, j1, k1);
        const State ul = get(u, node(i0, j0, k0, e0)), ur = get(u, node(i1, j1, k1, e1));
        double nrm[3];
        outward_normal(e0, f0, l1, l2, nrm);
        const State fl = phys.surface_flux(ul, ur, nrm);
        const State g0 = phys.surface_noncons(ul, ur, nrm);
        const State g1 = phys.surface_noncons(ur, ul, nrm);
        for (int v = 0; v < nv; ++v) {
          sf(e0, f0, l1, l2, v) = fl[v] + 0.5 * g0[v];
          sf(e1, f1, s1, s2, v) = -(fl[v] + 0.5 * g1[v]);
        }
      }
  }

  void boundary_flux(const double* u, int kb) {
    const int e = m.bd_e[kb], f = m.bd_f[kb];
    for (int l2 = 0; l2 < n; ++l2)
      for (int l1 = 0; l1 < n; ++l1) {
        int i, j, k;
        face_node3d(f, l1, l2, n, i, j, k);
        double nrm[3];
        outward_normal(e, f, l1, l2, nrm);
        const State fl = phys.bc_normal(get(u, node(i, j, k, e)), nrm);
        for (int v = 0; v < nv; ++v) sf(e, f, l1, l2, v) = fl[v];
      }
  }

  void surface_jacobian_sources(const double* u, double* du, int e, double t) const {
    for (int f = 0; f < 6; ++f)
      for (int l2 = 0; l2 < n; ++l2)
        for (int l1 = 0; l1 < n; ++l1) {
          int i, j, k;
          face_node3d(f, l1, l2, n, i, j, k);
          const double winv = 1.0 / b.w[(f & 1) ? n - 1 : 0];
          const size_t q = node(i, j, k, e);
          for (int v = 0; v < nv; ++v)
            du[q * nv + v] += sfv[((((size_t)e * 6 + f) * n + l2) * n + l1) * nv + v] * winv;
        }
    for (int q0 = 0; q0 < n * n * n; ++q0) {
      const size_t q = (size_t)e * n * n * n + q0;
      const double fjac = -m.invJ[q];
      for (int v = 0; v < nv; ++v) du[q * nv + v] *= fjac;
      if (Phys::has_sources) {
        const State s = phys.source(get(u, q), m.xyz ? &m.xyz[q * 3] : nullptr, t);
        for (int v = 0; v < nv; ++v) du[q * nv + v] += s[v];
      }
    }
  }

  void rhs(const double* u, double* du, double t) {
    const size_t N = (size_t)m.nelem * n * n * n * nv;
    std::fill(du, du + N, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < m.nelem; ++e) volume_integral(u, du, e);
#pragma omp parallel for schedule(static)
    for (int it = 0; it < (int)m.if_e0.size(); ++it) interface_flux(u, it);
#pragma omp parallel for schedule(static)
    for (int kb = 0; kb < (int)m.bd_e.size(); ++kb) boundary_flux(u, kb);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < m.nelem; ++e) surface_jacobian_sources(u, du, e, t);
  }

  // max_dt: 2 / (n * max_e (sum_d max_nodes |Ja^d . lambda| |invJ|)), the 3D
  // form of src/callbacks_step/stepsize_dg2d.jl:5-44
  double max_dt(const double* u) const {
    double max_scaled = std::nextafter(0.0, 1.0);
#pragma omp parallel for reduction(max : max_scaled)
    for (int e = 0; e < m.nelem; ++e) {
      double ml[3] = {0, 0, 0};
      for (int q0 = 0; q0 < n * n * n; ++q0) {
        const size_t q = (size_t)e * n * n * n + q0;
        double lam[3];
        phys.max_abs_speeds(get(u, q), lam);
        const double ij = std::fabs(m.invJ[q]);
        for (int d = 0; d < 3; ++d) {
          double a[3];
          ja(d, q, a);
          ml[d] = std::max(ml[d], std::fabs(a[0] * lam[0] + a[1] * lam[1] + a[2] * lam[2]) * ij);
        }
      }
      max_scaled = std::max(max_scaled, ml[0] + ml[1] + ml[2]);
    }
    return 2.0 / (n * max_scaled);
  }
};

}  // namespace orc
