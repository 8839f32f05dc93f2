// ORACLE — test infrastructure only. CPU restatement used as the checker for
// the CUDA path; never linked into or called by the product library.
//
// Legendre-Gauss-Lobatto (LGL) nodal basis on [-1, 1], restated from
// D. A. Kopriva, "Implementing Spectral Methods for Partial Differential
// Equations" (Springer 2009): Alg. 22 (Legendre polynomial and derivative),
// Alg. 25 (LGL nodes and weights by Newton iteration on q = L_{N+1} - L_{N-1}),
// Alg. 30 (barycentric weights) and Alg. 37 (first-derivative matrix).
// The split-form operator D_split = 2 D - M^{-1} B and the weak-form operator
// D_hat = -M^{-1} D^T M are the operators Trixi.jl's `LobattoLegendreBasis`
// exposes as `derivative_split` / `derivative_hat`, which TrixiAtmo's kernels
// consume (src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:104,140).
#pragma once
#include <cmath>
#include <vector>

namespace orc {

struct Basis {
  int n = 0;                 // number of nodes per direction (polydeg + 1)
  std::vector<double> x, w;  // nodes, quadrature weights
  std::vector<double> D;     // D[i*n + j] = l_j'(x_i)
  std::vector<double> Dsplit;
  std::vector<double> Dhat;
  double d(int i, int j) const { return D[i * n + j]; }
  double ds(int i, int j) const { return Dsplit[i * n + j]; }
  double dh(int i, int j) const { return Dhat[i * n + j]; }
};

// L_N(x), L_N'(x) by the three-term recurrence.
inline void legendre_and_derivative(int N, double x, double& L, double& dL) {
  if (N == 0) { L = 1.0; dL = 0.0; return; }
  if (N == 1) { L = x; dL = 1.0; return; }
  double Lm2 = 1.0, Lm1 = x, dLm2 = 0.0, dLm1 = 1.0;
  for (int k = 2; k <= N; ++k) {
    L = (2.0 * k - 1.0) / k * x * Lm1 - (k - 1.0) / k * Lm2;
    dL = dLm2 + (2.0 * k - 1.0) * Lm1;
    Lm2 = Lm1; Lm1 = L; dLm2 = dLm1; dLm1 = dL;
  }
}

// q(x) = L_{N+1} - L_{N-1}, q'(x), and L_N(x)  (Kopriva Alg. 24).
inline void q_and_L(int N, double x, double& q, double& dq, double& LN) {
  double Lnp1, dLnp1, Lnm1, dLnm1, dLN;
  legendre_and_derivative(N + 1, x, Lnp1, dLnp1);
  legendre_and_derivative(N - 1, x, Lnm1, dLnm1);
  legendre_and_derivative(N, x, LN, dLN);
  q = Lnp1 - Lnm1;
  dq = dLnp1 - dLnm1;
}

inline Basis make_lgl_basis(int polydeg) {
  const int N = polydeg;
  Basis b;
  b.n = N + 1;
  b.x.assign(b.n, 0.0);
  b.w.assign(b.n, 0.0);
  const double pi = 3.14159265358979323846;
  if (N == 1) {
    b.x = {-1.0, 1.0};
    b.w = {1.0, 1.0};
  } else {
    b.x[0] = -1.0; b.w[0] = 2.0 / (N * (N + 1.0));
    b.x[N] = 1.0;  b.w[N] = b.w[0];
    for (int j = 1; j <= (N + 1) / 2 - 1; ++j) {
      double xj = -std::cos((j + 0.25) * pi / N - 3.0 / (8.0 * N * pi * (j + 0.25)));
      double q, dq, LN;
      for (int it = 0; it < 100; ++it) {
        q_and_L(N, xj, q, dq, LN);
        double delta = -q / dq;
        xj += delta;
        if (std::fabs(delta) <= 4e-16 * std::fabs(xj)) break;
      }
      q_and_L(N, xj, q, dq, LN);
      b.x[j] = xj;
      b.x[N - j] = -xj;
      b.w[j] = 2.0 / (N * (N + 1.0) * LN * LN);
      b.w[N - j] = b.w[j];
    }
    if (N % 2 == 0) {
      double q, dq, LN;
      q_and_L(N, 0.0, q, dq, LN);
      b.x[N / 2] = 0.0;
      b.w[N / 2] = 2.0 / (N * (N + 1.0) * LN * LN);
    }
  }
  const int n = b.n;
  // barycentric weights (Alg. 30)
  std::vector<double> lam(n, 1.0);
  for (int j = 1; j < n; ++j)
    for (int k = 0; k < j; ++k) {
      lam[k] *= (b.x[k] - b.x[j]);
      lam[j] *= (b.x[j] - b.x[k]);
    }
  for (int j = 0; j < n; ++j) lam[j] = 1.0 / lam[j];
  // derivative matrix (Alg. 37, negative-sum trick on the diagonal)
  b.D.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      double v = lam[j] / lam[i] / (b.x[i] - b.x[j]);
      b.D[i * n + j] = v;
      diag -= v;
    }
    b.D[i * n + i] = diag;
  }
  // D_split = 2 D - M^{-1} B,  B = diag(-1, 0, ..., 0, 1)
  b.Dsplit.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) b.Dsplit[i * n + j] = 2.0 * b.D[i * n + j];
  b.Dsplit[0] += 1.0 / b.w[0];
  b.Dsplit[(n - 1) * n + (n - 1)] -= 1.0 / b.w[n - 1];
  // D_hat = -M^{-1} D^T M
  b.Dhat.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) b.Dhat[i * n + j] = -b.D[j * n + i] * b.w[j] / b.w[i];
  return b;
}

// Polynomial interpolation matrix from the nodes `from` to the points `to`
// (barycentric form, Kopriva Alg. 32).
inline std::vector<double> interpolation_matrix(const std::vector<double>& from,
                                                const std::vector<double>& to) {
  const int n = (int)from.size(), m = (int)to.size();
  std::vector<double> lam(n, 1.0);
  for (int j = 1; j < n; ++j)
    for (int k = 0; k < j; ++k) {
      lam[k] *= (from[k] - from[j]);
      lam[j] *= (from[j] - from[k]);
    }
  for (int j = 0; j < n; ++j) lam[j] = 1.0 / lam[j];
  std::vector<double> V(m * n, 0.0);
  for (int k = 0; k < m; ++k) {
    bool match = false;
    for (int j = 0; j < n; ++j)
      if (to[k] == from[j]) { V[k * n + j] = 1.0; match = true; }
    if (match) continue;
    double s = 0.0;
    for (int j = 0; j < n; ++j) {
      double t = lam[j] / (to[k] - from[j]);
      V[k * n + j] = t;
      s += t;
    }
    for (int j = 0; j < n; ++j) V[k * n + j] /= s;
  }
  return V;
}

}  // namespace orc
