// Analysis of the resident solution on the device: integrals of the conserved
// variables, of the entropy and of the total energy; the entropy time
// derivative; l2 / linf error norms against an exact solution the caller
// evaluates at the analysis nodes.  All reductions run in a fixed order, so
// repeated calls on the same state return the same bits.
//
// Reference: Trixi's AnalysisCallback as TrixiAtmo drives it.  Covariant
// equations: src/callbacks_step/analysis_covariant.jl (integrate_via_indices
// :53-85, quadrature weights times the exact area element J from the
// auxiliary variables; entropy_timederivative :87-105, sum of
// cons2entropy(u, aux) . du; calc_error_norms :143-189, at the solution
// nodes).  Cartesian meshes: the same quadrature with |1 / inverse_jacobian|;
// error norms on the Legendre-Gauss-Lobatto nodes of degree 2N (the default
// analysis polydeg), to which the solution and J are interpolated.
#pragma once
#include "tag_common.cuh"

namespace tag {

enum AnalysisPhys : int {
  kAnEnergy2D = 0, kAnEnergy3D, kAnRainy2D, kAnMoist2D, kAnPT2D, kAnCov, kAnPT3D,
  kAnIE2D
};

// One analysis call.  Node ranges of the members are [mbeg[m], mend[m])
// (device arrays; members occupy contiguous ranges).
struct AnalysisArgs {
  int phys;
  const void* params;  // the physics' Params (host copy, passed by value to kernels)
  int quantity;        // TAG_AQ_*
  int nmembers;
  const double* u;     // resident state [nodes][nv]
  const double* du;    // time derivative (entropy time derivative), else null
  const double* aux;   // covariant: aux_node_vars [nodes][26], else null
  const double* wj;    // quadrature weight x |J| per node
  const long* mbeg;
  const long* mend;
};

// Values per member of a quantity (nv conserved variables, or one value);
// -1 when the equations do not define it.
int analysis_values(int phys, int quantity);

// rows: [nmembers][nchunks][analysis_values + 1] (the last column the
// volume); chunk nodes per block.
int analysis_node_rows(const AnalysisArgs& a, int nchunks, long chunk, double* rows,
                       cudaStream_t s);

// Error-norm rows of Cartesian elements, one row [2 nv + 1] per element:
// sum wJ d^2 (nv), max |d| (nv), sum wJ, with d = u_exact - u at the analysis
// nodes.  V [m][n] interpolates from the solution to the analysis nodes, wa the
// analysis weights; u_exact [E][m^dim][nv].
int analysis_element_error_rows(int phys, int dim, int n, int m, int nelem, const double* u,
                                const double* invJ, const double* V, const double* wa,
                                const double* u_exact, double* rows, cudaStream_t s);

// Error-norm rows at the solution nodes (covariant): rows [nmembers][nchunks][2 nv + 1].
int analysis_node_error_rows(const AnalysisArgs& a, const double* u_exact, int nchunks, long chunk,
                             double* rows, cudaStream_t s);

// Reduces rows [rbeg[m], rend[m]) of width nq per member in a fixed order
// (columns [max_lo, max_hi) by max, the others by sum) into out [nmembers][nq].
// With rbeg == null the members' rows are [m * stride, (m + 1) * stride).
int analysis_reduce_rows(const double* rows, int nq, int max_lo, int max_hi, const long* rbeg,
                         const long* rend, long stride, int nmembers, double* out, cudaStream_t s);

// wj for Cartesian elements of npe = n^dim nodes: w_i w_j (w_k) |1 / invJ|.
int analysis_weights_cartesian(const double* invJ, const double* w, int n, int dim, long nodes,
                               double* wj, cudaStream_t s);
// wj for a run of covariant elements of n x n nodes: w_i w_j J (aux slot 12).
int analysis_weights_covariant(const double* aux, const double* w, int n, long node0, long count,
                               double* wj, cudaStream_t s);

// Coordinates of the analysis nodes [E][m^dim][dim] interpolated from the
// solution nodes' coordinates xyz [E][n^dim][dim].
int analysis_coordinates(int dim, int n, int m, int nelem, const double* xyz, const double* V,
                         double* out, cudaStream_t s);

// Legendre-Gauss-Lobatto nodes and weights of degree N on [-1, 1] (host).
void lgl_nodes_weights(int N, double* x, double* w);
// Lagrange interpolation matrix V[a][i] from nodes xf (nf) to xt (nt), barycentric form (host).
void interpolation_matrix(const double* xf, int nf, const double* xt, int nt, double* V);

}  // namespace tag
