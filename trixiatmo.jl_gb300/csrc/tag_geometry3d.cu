// Geometry of the cubed-sphere shell, computed on the device: what the
// reference's cache builds on the host for P4estMeshCubedSphereTopography.
//
// Node coordinates: the equiangular cubed-sphere map of each cube face
// (src/meshes/p4est_cubed_sphere_topography.jl:596-620): with alpha = xi pi/4,
// beta = eta pi/4, x = tan alpha, y = tan beta, the face's cube vector c(x, y)
// of length r = sqrt(1 + x^2 + y^2) is scaled to radius inner_radius + z with
// z = thickness (zeta + 1) / 2, or, over a topography, z moved by the
// Gal-Chen / Sleve vertical coordinate (:7-79) from the ground height z_s of
// the node's column (given per column node by the caller, who evaluates its
// topography function there).  Metric terms as Trixi builds them for curved
// P4estMesh{3} meshes: the Jacobian matrix by the collocation derivative of
// the node coordinates, J its determinant, and the contravariant vectors in
// the invariant curl form of D. A. Kopriva, J. Sci. Comput. 26 (2006) 301-327,
//   (Ja^i)_n = -1/2 e_i . curl_xi I^N( X_l grad_xi X_m - X_m grad_xi X_l ),
// (n, m, l) cyclic, which satisfies the discrete metric identities.  One CTA
// per element; the element's nodal fields live in shared memory.
// Element order: e = cz + layers (cx + trees (cy + trees face)), faces 0..5 as
// the reference's directions 1..6 (-z, +x, +y, -x, -y, +z); node order
// [e][k][j][i]; outputs xyz[e][k][j][i][c], Ja[e][k][j][i][d][c] (d the
// reference direction, c the Cartesian component), invJ[e][k][j][i].
#include <string>

#include "tag_common.cuh"

namespace tag {
namespace {

struct ShellArgs {
  int trees, layers, n, vertical;  // vertical: 0 Gal-Chen, 1 Sleve
  double inner_radius, thickness, sleve_eta_h, sleve_s;
};

TAG_DEV void cube_vector(int face, double x, double y, double* c) {
  switch (face) {
    case 0: c[0] = -y; c[1] = -x; c[2] = -1.0; break;
    case 1: c[0] = 1.0; c[1] = x; c[2] = y; break;
    case 2: c[0] = -x; c[1] = 1.0; c[2] = y; break;
    case 3: c[0] = -1.0; c[1] = -x; c[2] = y; break;
    case 4: c[0] = x; c[1] = -1.0; c[2] = y; break;
    default: c[0] = x; c[1] = y; c[2] = 1.0; break;
  }
}

// derivative along direction d (0: i, 1: j, 2: k) of the nodal field f at
// node (i, j, k) with the collocation derivative matrix D[a * n + b]
TAG_DEV double dnodal(const double* f, const double* D, int n, int d, int i, int j, int k) {
  double s = 0.0;
  const int p = d == 0 ? i : (d == 1 ? j : k);
  for (int a = 0; a < n; ++a) {
    const int q = d == 0 ? (k * n + j) * n + a : (d == 1 ? (k * n + a) * n + i : (a * n + j) * n + i);
    s = fma(D[p * n + a], f[q], s);
  }
  return s;
}

__global__ void k_shell_geometry(ShellArgs A, const double* __restrict__ nodes,
                                 const double* __restrict__ D, const double* __restrict__ zs,
                                 double* __restrict__ xyz, double* __restrict__ Ja,
                                 double* __restrict__ invJ, int* __restrict__ flag) {
  extern __shared__ double sm[];
  const int n = A.n, nnn = n * n * n;
  double* X = sm;              // [3][nnn]
  double* G = X + 3 * nnn;     // [3 (c)][3 (d)][nnn]: dX_c / dxi_d
  double* W = G + 9 * nnn;     // [3][nnn]
  double* sD = W + 3 * nnn;    // [n][n]
  const int e = blockIdx.x;
  const int cz = e % A.layers, cx = (e / A.layers) % A.trees;
  const int cy = (e / (A.layers * A.trees)) % A.trees, face = e / (A.layers * A.trees * A.trees);
  const double dx = 2.0 / A.trees, dz = 2.0 / A.layers;
  const double pi = 3.14159265358979323846;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) sD[t] = D[t];
  for (int q = threadIdx.x; q < nnn; q += blockDim.x) {
    const int i = q % n, j = (q / n) % n, k = q / (n * n);
    const double xi = -1.0 + cx * dx + 0.5 * dx + 0.5 * dx * nodes[i];
    const double eta = -1.0 + cy * dx + 0.5 * dx + 0.5 * dx * nodes[j];
    const double zeta = -1.0 + cz * dz + 0.5 * dz + 0.5 * dz * nodes[k];
    const double x = tan(xi * pi / 4.0), y = tan(eta * pi / 4.0);
    double c[3];
    cube_vector(face, x, y, c);
    const double r = sqrt(1.0 + x * x + y * y);
    double z = A.thickness * 0.5 * (zeta + 1.0);
    if (zs) {
      const double h = zs[(size_t)e * n * n + j * n + i], H = A.thickness;
      if (A.vertical == 0) {
        z = z + (H - z) * h / H;
      } else {
        const double et = z / H;
        z = et <= A.sleve_eta_h
                ? et * H + h * sinh((A.sleve_eta_h - et) / A.sleve_s / A.sleve_eta_h) /
                               sinh(1.0 / A.sleve_s)
                : et * H;
      }
    }
    const double s = (A.inner_radius + z) / r;
    for (int d = 0; d < 3; ++d) {
      X[d * nnn + q] = s * c[d];
      xyz[((size_t)e * nnn + q) * 3 + d] = s * c[d];
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nnn; q += blockDim.x) {
    const int i = q % n, j = (q / n) % n, k = q / (n * n);
    double m[9];
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) {
        m[c * 3 + d] = dnodal(X + c * nnn, sD, n, d, i, j, k);
        G[(c * 3 + d) * nnn + q] = m[c * 3 + d];
      }
    const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                       m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (!(det != 0.0) || !isfinite(det)) atomicOr(flag, 1);
    invJ[(size_t)e * nnn + q] = 1.0 / det;
  }
  __syncthreads();
  for (int nc = 0; nc < 3; ++nc) {
    const int mm = (nc + 1) % 3, l = (nc + 2) % 3;
    // W = X_l grad X_m - X_m grad X_l, then (Ja^d)_nc = -1/2 (curl W)_d
    for (int q = threadIdx.x; q < nnn; q += blockDim.x)
      for (int f = 0; f < 3; ++f)
        W[f * nnn + q] = X[l * nnn + q] * G[(mm * 3 + f) * nnn + q] -
                         X[mm * nnn + q] * G[(l * 3 + f) * nnn + q];
    __syncthreads();
    for (int q = threadIdx.x; q < nnn; q += blockDim.x) {
      const int i = q % n, j = (q / n) % n, k = q / (n * n);
      const double c0 = dnodal(W + 2 * nnn, sD, n, 1, i, j, k) - dnodal(W + nnn, sD, n, 2, i, j, k);
      const double c1 = dnodal(W, sD, n, 2, i, j, k) - dnodal(W + 2 * nnn, sD, n, 0, i, j, k);
      const double c2 = dnodal(W + nnn, sD, n, 0, i, j, k) - dnodal(W, sD, n, 1, i, j, k);
      double* o = Ja + ((size_t)e * nnn + q) * 9 + nc;
      o[0] = -0.5 * c0;
      o[3] = -0.5 * c1;
      o[6] = -0.5 * c2;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace tag

using namespace tag;

extern "C" int tag_shell_geometry(int32_t trees, int32_t layers, double inner_radius,
                                  double thickness, int32_t polydeg, const double* nodes,
                                  const double* derivative_matrix, const double* ground_height,
                                  int32_t vertical, double sleve_eta_h, double sleve_s,
                                  double* xyz, double* Ja, double* invJ) {
  const int n = polydeg + 1;
  if (trees < 1 || layers < 1 || n < 2 || n > kMaxNodes || !(inner_radius > 0.0) ||
      !(thickness > 0.0) || !nodes || !derivative_matrix || !xyz || !Ja || !invJ ||
      (ground_height && vertical != 0 &&
       (vertical != 1 || !(sleve_eta_h > 0.0) || !(sleve_s > 0.0)))) {
    set_last_error("tag_shell_geometry: bad argument");
    return TAG_E_INVALID;
  }
  const size_t E = (size_t)6 * trees * trees * layers, nnn = (size_t)n * n * n;
  ShellArgs A{trees, layers, n, vertical, inner_radius, thickness, sleve_eta_h, sleve_s};
  double *d_nodes = nullptr, *d_D = nullptr, *d_zs = nullptr, *d_xyz = nullptr, *d_Ja = nullptr,
         *d_invJ = nullptr;
  int* d_flag = nullptr;
  int rc = TAG_OK, flag = 0;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == TAG_OK) {
      rc = TAG_E_CUDA;
      set_last_error(std::string("tag_shell_geometry: ") + cudaGetErrorString(e));
    }
    return rc == TAG_OK;
  };
  const size_t smem = sizeof(double) * (15 * nnn + (size_t)n * n);
  if (ok(cudaMalloc(&d_nodes, sizeof(double) * n)) && ok(cudaMalloc(&d_D, sizeof(double) * n * n)) &&
      (!ground_height || ok(cudaMalloc(&d_zs, sizeof(double) * E * n * n))) &&
      ok(cudaMalloc(&d_xyz, sizeof(double) * E * nnn * 3)) &&
      ok(cudaMalloc(&d_Ja, sizeof(double) * E * nnn * 9)) &&
      ok(cudaMalloc(&d_invJ, sizeof(double) * E * nnn)) && ok(cudaMalloc(&d_flag, sizeof(int))) &&
      ok(cudaMemcpy(d_nodes, nodes, sizeof(double) * n, cudaMemcpyHostToDevice)) &&
      ok(cudaMemcpy(d_D, derivative_matrix, sizeof(double) * n * n, cudaMemcpyHostToDevice)) &&
      (!ground_height ||
       ok(cudaMemcpy(d_zs, ground_height, sizeof(double) * E * n * n, cudaMemcpyHostToDevice))) &&
      ok(cudaMemset(d_flag, 0, sizeof(int))) &&
      ok(cudaFuncSetAttribute(k_shell_geometry, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem))) {
    k_shell_geometry<<<(unsigned)E, 128, smem>>>(A, d_nodes, d_D, d_zs, d_xyz, d_Ja, d_invJ,
                                                 d_flag);
    if (ok(cudaGetLastError()) &&
        ok(cudaMemcpy(xyz, d_xyz, sizeof(double) * E * nnn * 3, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(Ja, d_Ja, sizeof(double) * E * nnn * 9, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(invJ, d_invJ, sizeof(double) * E * nnn, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost)) && flag) {
      rc = TAG_E_INVALID;
      set_last_error("tag_shell_geometry: singular Jacobian at a node");
    }
  }
  cudaFree(d_nodes);
  cudaFree(d_D);
  cudaFree(d_zs);
  cudaFree(d_xyz);
  cudaFree(d_Ja);
  cudaFree(d_invJ);
  cudaFree(d_flag);
  return rc;
}
