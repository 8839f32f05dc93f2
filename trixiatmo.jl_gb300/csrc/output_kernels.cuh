// Solution variables for output (SaveSolutionCallback): the conversions that
// the reference's convert_variables applies node by node before writing a
// solution file, computed on the device into the variable-major layout of
// the file (row v = variable v over the nodes of the selected range).
//
// Reference: src/callbacks_step/save_solution_covariant.jl (convert_variables
// :5-33, cons2prim_and_vorticity :64-74, calc_vorticity_node :93-118,
// varnames :122-125); src/equations/covariant_shallow_water.jl (varnames
// :83-100, cons2prim :113-118, contravariant2global :140-145);
// src/equations/equations.jl (aux-variable slots :210-244).
#pragma once
#include "cov_kernels.cuh"

namespace tag {

// cons2cons of any equation system: out[v][t] = u[q0 + t][v]
__global__ void k_state_rows(const double* __restrict__ u, int nv, long q0, long nq,
                             double* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  const double* uq = u + (q0 + t) * nv;
  for (int v = 0; v < nv; ++v) out[(long)v * nq + t] = uq[v];
}

// Row a of the plain derivative matrix D at column c, from the split form
// D_split = 2 D - M^{-1} B held by the basis (B = diag(-1, 0, .., 0, 1)).
TAG_DEV double cov_derivative(const BasisDev& b, int n, int a, int c) {
  double d = b.Ds[a * n + c];
  if (a == c && a == 0) d -= b.winv0;
  if (a == c && a == n - 1) d += b.winvN;
  return 0.5 * d;
}

// covariant velocity components v_k = G_kl v^l of node q (aux slots 13-15:
// G_11, G_12, G_22)
TAG_DEV void cov_velocity_covariant(const double* __restrict__ u, const double* __restrict__ aux,
                                    long q, double& w1, double& w2) {
  const double* uq = u + q * 3;
  const double* a = aux + q * 26;
  const double ih = 1.0 / uq[0];
  const double c1 = uq[1] * ih, c2 = uq[2] * ih;
  w1 = a[13] * c1 + a[14] * c2;
  w2 = a[14] * c1 + a[15] * c2;
}

// Covariant shallow water: one thread per node of [q0, q0 + nq).
// kind TAG_SOLVAR_CONS2CONS (h, h_vcon1, h_vcon2), _CONS2PRIM (H, vcon1,
// vcon2), _CONTRAVARIANT2GLOBAL (h, h_v1, h_v2, h_v3), _CONS2PRIM_AND_VORTICITY
// (H, v1, v2, v3, b, vorticity); aux slots 0-5 hold the covariant basis
// (columns a_1, a_2), 12 the area element J, 19 the bottom topography.
__global__ void k_cov_solution_rows(const CovGroups* __restrict__ G,
                                    const BasisDev* __restrict__ bases,
                                    const double* __restrict__ u, const double* __restrict__ aux,
                                    int kind, long q0, long nq, double* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  const long q = q0 + t;
  int gi = 0;
  for (int k = 1; k < G->count; ++k)
    if (G->g[k].node0 <= q) gi = k;
  const CovGroup& g = G->g[gi];
  const double* uq = u + q * 3;
  const double* a = aux + q * 26;
  const double h = uq[0], m1 = uq[1], m2 = uq[2];
  double r[6];
  int nr = 3;
  if (kind == 0) {
    r[0] = h; r[1] = m1; r[2] = m2;
  } else if (kind == 1) {
    r[0] = h + a[19]; r[1] = m1 / h; r[2] = m2 / h;
  } else if (kind == 2) {
    nr = 4;
    r[0] = h;
#pragma unroll
    for (int c = 0; c < 3; ++c) r[1 + c] = a[c] * m1 + a[3 + c] * m2;
  } else {
    nr = 6;
    const double c1 = m1 / h, c2 = m2 / h;
    r[0] = h + a[19];
#pragma unroll
    for (int c = 0; c < 3; ++c) r[1 + c] = a[c] * c1 + a[3 + c] * c2;
    r[4] = a[19];
    // relative vorticity (d v_2 / d xi^1 - d v_1 / d xi^2) / J along the
    // node's two grid lines
    const int n = g.n, nn = n * n;
    const BasisDev& b = bases[g.basis];
    const long ql = q - g.node0;
    const long e0 = g.node0 + (ql / nn) * nn;
    const int rr = (int)(ql % nn), i = rr % n, j = rr / n;
    double d21 = 0.0, d12 = 0.0, w1, w2;
    for (int ii = 0; ii < n; ++ii) {
      cov_velocity_covariant(u, aux, e0 + (long)j * n + ii, w1, w2);
      d21 += cov_derivative(b, n, i, ii) * w2;
    }
    for (int jj = 0; jj < n; ++jj) {
      cov_velocity_covariant(u, aux, e0 + (long)jj * n + i, w1, w2);
      d12 += cov_derivative(b, n, j, jj) * w1;
    }
    r[5] = (d21 - d12) / a[12];
  }
  for (int v = 0; v < nr; ++v) out[(long)v * nq + t] = r[v];
}

}  // namespace tag
