// Covariant metric terms of the cubed-sphere manifold, computed on the device:
// the 26 auxiliary variables per node and the node coordinates that the
// reference's cache builds on the host (init_auxiliary_node_variables!,
// src/solvers/dgsem_p4est/containers_2d_manifold_in_3d_covariant.jl:232-489).
//
// Per node (xi1, xi2) of an element with corner vertices v1..v4 (element-local
// mapping, Guba et al. 2014, appendix A): the covariant basis A (3x2) of the
// radially projected bilinear map, in global Cartesian components (product
// and quotient rule, :306-327) or in spherical components (:334-375); the
// covariant metric G = A^T A, its inverse, the contravariant basis G^-1 A^T,
// the area element J = sqrt(det G); the Christoffel symbols
// Gamma^i_jk = G^il (d_j G_lk + d_k G_lj - d_l G_jk) / 2 (:417-441) from the
// metric derivatives, either exact (forward-mode dual numbers through the
// mapping: ChristoffelSymbolsAutodiff) or by the collocation derivative of the
// nodal metric (ChristoffelSymbolsCollocationDerivative).  The bottom
// topography (slot 19) is left to the caller, which evaluates its own
// function at the returned coordinates.
#include <string>
#include <vector>

#include "tag_common.cuh"

namespace tag {
namespace {

// value and derivatives with respect to xi1 and xi2
struct Dual {
  double v, d1, d2;
};

TAG_DEV Dual mk(double v) { return Dual{v, 0.0, 0.0}; }
TAG_DEV Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d1 + b.d1, a.d2 + b.d2}; }
TAG_DEV Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d1 - b.d1, a.d2 - b.d2}; }
TAG_DEV Dual operator-(Dual a) { return Dual{-a.v, -a.d1, -a.d2}; }
TAG_DEV Dual operator*(Dual a, Dual b) {
  return Dual{a.v * b.v, a.d1 * b.v + a.v * b.d1, a.d2 * b.v + a.v * b.d2};
}
TAG_DEV Dual operator/(Dual a, Dual b) {
  const double q = b.v * b.v;
  return Dual{a.v / b.v, (a.d1 * b.v - a.v * b.d1) / q, (a.d2 * b.v - a.v * b.d2) / q};
}
TAG_DEV Dual operator*(double s, Dual a) { return mk(s) * a; }
TAG_DEV Dual operator+(double s, Dual a) { return mk(s) + a; }
TAG_DEV Dual operator-(double s, Dual a) { return mk(s) - a; }
TAG_DEV Dual dsqrt(Dual a) {
  const double s = sqrt(a.v);
  return Dual{s, a.d1 / (2 * s), a.d2 / (2 * s)};
}
TAG_DEV Dual dsin(Dual a) {
  const double c = cos(a.v);
  return Dual{sin(a.v), c * a.d1, c * a.d2};
}
TAG_DEV Dual dcos(Dual a) {
  const double s = sin(a.v);
  return Dual{cos(a.v), -s * a.d1, -s * a.d2};
}
TAG_DEV Dual dasin(Dual a) {
  const double r = sqrt(1 - a.v * a.v);
  return Dual{asin(a.v), a.d1 / r, a.d2 / r};
}
TAG_DEV Dual datan2(Dual y, Dual x) {
  const double r2 = x.v * x.v + y.v * y.v;
  return Dual{atan2(y.v, x.v), (x.v * y.d1 - y.v * x.d1) / r2, (x.v * y.d2 - y.v * x.d2) / r2};
}

// Covariant basis A[r][c] (r: global component, c: a_1, a_2) at (xi1, xi2),
// derivatives carried along; v: the element's vertices [4][3].
TAG_DEV void basis_covariant(const double* v, Dual xi1, Dual xi2, double radius, bool spherical,
                             Dual A[3][2]) {
  const double* v1 = v;
  const double* v2 = v + 3;
  const double* v3 = v + 6;
  const double* v4 = v + 9;
  Dual xe[3];
  for (int k = 0; k < 3; ++k)
    xe[k] = 0.25 * ((1.0 - xi1) * (1.0 - xi2) * mk(v1[k]) + (1.0 + xi1) * (1.0 - xi2) * mk(v2[k]) +
                    (1.0 + xi1) * (1.0 + xi2) * mk(v3[k]) + (1.0 - xi1) * (1.0 + xi2) * mk(v4[k]));
  if (!spherical) {
    Dual d1[3], d2[3];
    for (int k = 0; k < 3; ++k) {
      d1[k] = 0.25 * (-((1.0 - xi2) * mk(v1[k])) + (1.0 - xi2) * mk(v2[k]) +
                      (1.0 + xi2) * mk(v3[k]) - (1.0 + xi2) * mk(v4[k]));
      d2[k] = 0.25 * (-((1.0 - xi1) * mk(v1[k])) - (1.0 + xi1) * mk(v2[k]) +
                      (1.0 + xi1) * mk(v3[k]) + (1.0 - xi1) * mk(v4[k]));
    }
    const Dual nrm = dsqrt(xe[0] * xe[0] + xe[1] * xe[1] + xe[2] * xe[2]);
    const Dual dot1 = xe[0] * d1[0] + xe[1] * d1[1] + xe[2] * d1[2];
    const Dual dot2 = xe[0] * d2[0] + xe[1] * d2[1] + xe[2] * d2[2];
    const Dual n2 = nrm * nrm;
    for (int k = 0; k < 3; ++k) {
      A[k][0] = mk(radius) / nrm * (d1[k] - dot1 / n2 * xe[k]);
      A[k][1] = mk(radius) / nrm * (d2[k] - dot2 / n2 * xe[k]);
    }
    return;
  }
  const Dual sf = mk(radius) / dsqrt(xe[0] * xe[0] + xe[1] * xe[1] + xe[2] * xe[2]);
  Dual x[3];
  for (int k = 0; k < 3; ++k) x[k] = sf * xe[k];
  const Dual lon = datan2(x[1], x[0]), lat = dasin(x[2] / mk(radius));
  const Dual sl = dsin(lon), cl = dcos(lon), st = dsin(lat), ct = dcos(lat);
  const Dual P[3][3] = {{sl * sl * ct * ct + st * st, -(sl * cl * ct * ct), -(cl * st * ct)},
                        {-(sl * cl * ct * ct), cl * cl * ct * ct + st * st, -(sl * st * ct)},
                        {-(cl * st), -(sl * st), ct}};
  const Dual S[2][3] = {{-sl, cl, mk(0.0)}, {mk(0.0), mk(0.0), mk(1.0)}};
  const Dual W[4][2] = {{-1.0 + xi2, -1.0 + xi1}, {1.0 - xi2, -1.0 - xi1},
                        {1.0 + xi2, 1.0 + xi1}, {-1.0 - xi2, 1.0 - xi1}};
  const double* V[4] = {v1, v2, v3, v4};
  Dual M[3][2], PM[3][2];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 2; ++c) {
      Dual s = mk(V[0][k]) * W[0][c];
      for (int q = 1; q < 4; ++q) s = s + mk(V[q][k]) * W[q][c];
      M[k][c] = s;
    }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) {
      Dual s = P[r][0] * M[0][c];
      for (int k = 1; k < 3; ++k) s = s + P[r][k] * M[k][c];
      PM[r][c] = s;
    }
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) {
      Dual s = S[r][0] * PM[0][c];
      for (int k = 1; k < 3; ++k) s = s + S[r][k] * PM[k][c];
      A[r][c] = 0.25 * sf * s;
    }
  A[2][0] = A[2][1] = mk(0.0);
}

// One block per element, one thread per node.  D: derivative matrix,
// D[i + n k] = l_k'(x_i) (collocation Christoffel symbols only).
__global__ void k_cov_metric(const double* __restrict__ vertices, int n,
                             const double* __restrict__ nodes, const double* __restrict__ D,
                             double radius, int spherical, int collocation,
                             double* __restrict__ aux, double* __restrict__ xyz,
                             int* __restrict__ nonfinite) {
  __shared__ double sv[12];
  __shared__ double sG[3 * kMaxNodes * kMaxNodes];
  const long e = blockIdx.x;
  const int node = threadIdx.x, nn = n * n;
  if (node < 12) sv[node] = vertices[e * 12 + node];
  __syncthreads();
  const bool act = node < nn;
  const int i = node % n, j = node / n;
  double* a = aux + (e * nn + node) * 26;
  double G11_1 = 0, G12_1 = 0, G22_1 = 0, G11_2 = 0, G12_2 = 0, G22_2 = 0;
  double g[3] = {0, 0, 0};
  if (act) {
    const Dual xi1{nodes[i], 1.0, 0.0}, xi2{nodes[j], 0.0, 1.0};
    Dual A[3][2];
    basis_covariant(sv, xi1, xi2, radius, spherical != 0, A);
    const Dual G11 = A[0][0] * A[0][0] + A[1][0] * A[1][0] + A[2][0] * A[2][0];
    const Dual G12 = A[0][0] * A[0][1] + A[1][0] * A[1][1] + A[2][0] * A[2][1];
    const Dual G22 = A[0][1] * A[0][1] + A[1][1] * A[1][1] + A[2][1] * A[2][1];
    const double det = G11.v * G22.v - G12.v * G12.v;
    const double gi11 = G22.v / det, gi22 = G11.v / det, gi12 = -G12.v / det;
    for (int r = 0; r < 3; ++r) {  // A column-major 3x2, contravariant basis column-major 2x3
      a[r] = A[r][0].v;
      a[3 + r] = A[r][1].v;
      a[6 + 2 * r] = gi11 * A[r][0].v + gi12 * A[r][1].v;
      a[7 + 2 * r] = gi12 * A[r][0].v + gi22 * A[r][1].v;
    }
    a[12] = sqrt(det);
    a[13] = G11.v;
    a[14] = G12.v;
    a[15] = G22.v;
    a[16] = gi11;
    a[17] = gi12;
    a[18] = gi22;
    a[19] = 0.0;
    g[0] = G11.v;
    g[1] = G12.v;
    g[2] = G22.v;
    G11_1 = G11.d1; G12_1 = G12.d1; G22_1 = G22.d1;
    G11_2 = G11.d2; G12_2 = G12.d2; G22_2 = G22.d2;
    // node coordinates: the radial projection of the bilinear map
    double xb[3];
    for (int k = 0; k < 3; ++k)
      xb[k] = 0.25 * ((1 - xi1.v) * (1 - xi2.v) * sv[k] + (1 + xi1.v) * (1 - xi2.v) * sv[3 + k] +
                      (1 + xi1.v) * (1 + xi2.v) * sv[6 + k] + (1 - xi1.v) * (1 + xi2.v) * sv[9 + k]);
    const double nr = sqrt(xb[0] * xb[0] + xb[1] * xb[1] + xb[2] * xb[2]);
    for (int k = 0; k < 3; ++k) xyz[(e * nn + node) * 3 + k] = radius * xb[k] / nr;
    for (int c = 0; c < 3; ++c) sG[c * nn + node] = g[c];
  }
  if (collocation) {
    __syncthreads();
    if (act) {
      double s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
      for (int k = 0; k < n; ++k) {
        const double di = D[i + n * k], dj = D[j + n * k];
        for (int c = 0; c < 3; ++c) {
          s1[c] += di * sG[c * nn + j * n + k];
          s2[c] += dj * sG[c * nn + k * n + i];
        }
      }
      G11_1 = s1[0]; G12_1 = s1[1]; G22_1 = s1[2];
      G11_2 = s2[0]; G12_2 = s2[1]; G22_2 = s2[2];
    }
  }
  if (!act) return;
  // Christoffel symbols of the first kind, raised with G^-1
  const double g1_00 = 0.5 * G11_1, g1_01 = 0.5 * G11_2, g1_11 = G12_2 - 0.5 * G22_1;
  const double g2_00 = G12_1 - 0.5 * G11_2, g2_01 = 0.5 * G22_1, g2_11 = 0.5 * G22_2;
  const double c11 = a[16], c12 = a[17], c22 = a[18];
  a[20] = c11 * g1_00 + c12 * g2_00;
  a[21] = c11 * g1_01 + c12 * g2_01;
  a[22] = c11 * g1_11 + c12 * g2_11;
  a[23] = c12 * g1_00 + c22 * g2_00;
  a[24] = c12 * g1_01 + c22 * g2_01;
  a[25] = c12 * g1_11 + c22 * g2_11;
  bool ok = true;
  for (int k = 0; k < 26; ++k) ok = ok && isfinite(a[k]);
  if (!ok) atomicOr(nonfinite, 1);
}

}  // namespace
}  // namespace tag

using namespace tag;

extern "C" int tag_cov_metric_terms(const double* vertices, int32_t nelements, int32_t polydeg,
                                    double radius, int32_t spherical, int32_t collocation,
                                    const double* nodes, const double* derivative_matrix,
                                    double* aux, double* xyz) {
  const int n = polydeg + 1;
  if (!vertices || !nodes || !aux || !xyz || nelements <= 0 || n < 2 || n > kMaxNodes ||
      !(radius > 0.0) || (collocation && !derivative_matrix)) {
    set_last_error("tag_cov_metric_terms: bad argument");
    return TAG_E_INVALID;
  }
  const size_t E = (size_t)nelements, nodes_all = E * n * n;
  double *d_v = nullptr, *d_x = nullptr, *d_D = nullptr, *d_aux = nullptr, *d_xyz = nullptr;
  int* d_flag = nullptr;
  int rc = TAG_OK, flag = 0;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == TAG_OK) {
      rc = TAG_E_CUDA;
      set_last_error(std::string("tag_cov_metric_terms: ") + cudaGetErrorString(e));
    }
    return rc == TAG_OK;
  };
  if (ok(cudaMalloc(&d_v, sizeof(double) * E * 12)) && ok(cudaMalloc(&d_x, sizeof(double) * n)) &&
      ok(cudaMalloc(&d_D, sizeof(double) * n * n)) &&
      ok(cudaMalloc(&d_aux, sizeof(double) * nodes_all * 26)) &&
      ok(cudaMalloc(&d_xyz, sizeof(double) * nodes_all * 3)) && ok(cudaMalloc(&d_flag, sizeof(int))) &&
      ok(cudaMemcpy(d_v, vertices, sizeof(double) * E * 12, cudaMemcpyHostToDevice)) &&
      ok(cudaMemcpy(d_x, nodes, sizeof(double) * n, cudaMemcpyHostToDevice)) &&
      ok(cudaMemset(d_D, 0, sizeof(double) * n * n)) &&
      (!collocation ||
       ok(cudaMemcpy(d_D, derivative_matrix, sizeof(double) * n * n, cudaMemcpyHostToDevice))) &&
      ok(cudaMemset(d_flag, 0, sizeof(int)))) {
    k_cov_metric<<<(unsigned)E, 64>>>(d_v, n, d_x, d_D, radius, spherical, collocation, d_aux,
                                      d_xyz, d_flag);
    if (ok(cudaGetLastError()) &&
        ok(cudaMemcpy(aux, d_aux, sizeof(double) * nodes_all * 26, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(xyz, d_xyz, sizeof(double) * nodes_all * 3, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost)) && flag) {
      rc = TAG_E_INVALID;
      set_last_error("the metric terms are singular at a node (spherical global coordinates are "
                     "singular at the poles; use GlobalCartesianCoordinates)");
    }
  }
  cudaFree(d_v);
  cudaFree(d_x);
  cudaFree(d_D);
  cudaFree(d_aux);
  cudaFree(d_xyz);
  cudaFree(d_flag);
  return rc;
}
