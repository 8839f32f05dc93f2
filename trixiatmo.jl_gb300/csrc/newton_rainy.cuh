// Rainy-Euler saturation Newton solve (the reference's stage limiter,
// src/callbacks_stage/nonlinear_solve_dg2d.jl:6-44, with residual and Jacobian
// from src/equations/compressible_rainy_euler_2d.jl:738-809), one thread per
// node, with an optional learned initial guess from a small FP32 MLP.
#pragma once
#include "phys_rainy_2d.cuh"

namespace tag {

// FP32 MLP 5 -> 32 -> 32 -> 1 (tanh hidden layers).  Flat parameter layout:
//   W1[32][5], b1[32], W2[32][32], b2[32], W3[32], b3,      (1281 trainable)
//   in_mean[5], in_scale[5], out_mean, out_scale           (12 normalisation)
constexpr int kMlpIn = 5, kMlpH = 32;
constexpr int kMlpTrain = kMlpH * kMlpIn + kMlpH + kMlpH * kMlpH + kMlpH + kMlpH + 1;  // 1281
constexpr int kMlpParams = kMlpTrain + 2 * kMlpIn + 2;                                   // 1293
constexpr int oW1 = 0, oB1 = oW1 + kMlpH * kMlpIn, oW2 = oB1 + kMlpH, oB2 = oW2 + kMlpH * kMlpH,
              oW3 = oB2 + kMlpH, oB3 = oW3 + kMlpH, oInMean = oB3 + 1,
              oInScale = oInMean + kMlpIn, oOutMean = oInScale + kMlpIn,
              oOutScale = oOutMean + 1;

// Temperature of the unsaturated equilibrium (all moisture as vapour):
// e_int = (c_vd rho_d + c_vv rho_m + c_l rho_r) T + rho_m L, e_int the internal
// energy E - |rho v|^2 / (2 rho).  It is the exact solution of the saturation
// system when e_s(T) / (R_v T) >= rho_m there, and a lower bound otherwise.
TAG_DEV double rainy_t_unsat(const double* u, double& e_int) {
  using C = RainyConst;
  const double rho = u[0] + u[1] + u[2];
  e_int = u[5] - 0.5 * (u[3] * u[3] + u[4] * u[4]) / rho;
  return (e_int - u[1] * C::ref_L) / (C::c_vd * u[0] + C::c_vv * u[1] + C::c_l * u[2]);
}

// Network inputs of a rainy state: (rho_dry, rho_moist, rho_rain, internal
// energy, unsaturated-equilibrium temperature).  The network predicts the
// latent-heat offset T* - T_unsat of nodes that are saturated at equilibrium.
// Cloud water is an unknown of the saturation system, not an input, so the
// conserved moist density stands in for (rho_v, rho_c).
TAG_DEV void mlp_inputs(const double* u, double e_int, double t_unsat, float* x) {
  x[0] = (float)u[0];
  x[1] = (float)u[1];
  x[2] = (float)u[2];
  x[3] = (float)e_int;
  x[4] = (float)t_unsat;
}

TAG_DEV float mlp_forward(const float* __restrict__ P, const float* xin) {
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) x[k] = (xin[k] - P[oInMean + k]) * P[oInScale + k];
  float h1[kMlpH];
#pragma unroll
  for (int o = 0; o < kMlpH; ++o) {
    float s = P[oB1 + o];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) s = fmaf(P[oW1 + o * kMlpIn + k], x[k], s);
    h1[o] = tanhf(s);
  }
  float y = P[oB3];
  for (int o = 0; o < kMlpH; ++o) {
    float s = P[oB2 + o];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) s = fmaf(P[oW2 + o * kMlpH + k], h1[k], s);
    y = fmaf(P[oW3 + o], tanhf(s), y);
  }
  return P[oOutMean] + P[oOutScale] * y;
}

struct NewtonArgs {
  int mode;          // 0: max|res| < tol (reference); 1: relative to E_int and 1e7 rho_moist
  int maxit;         // Newton updates allowed
  int polish;        // canonical finish: Newton updates from the converged iterate snapped
                     // to a fixed grid (0: stop at the criterion, as the reference does)
  int learned;       // start: 0 the warm start (slots 7-9, as the reference); 1 the closed-form
                     // unsaturated equilibrium where valid, else the MLP guess; 2 the closed
                     // form where valid, else the warm start; 3 the closed form where valid,
                     // else whichever of the MLP guess and the warm start has the smaller
                     // residual.  A guessed start that has not converged after
                     // maxit_learned updates falls back to the warm start.
  int maxit_learned; // 8
  double tol;
  const float* mlp;  // device parameters (kMlpParams floats) or null
  int* iters;        // per-node Newton updates, or null
  unsigned long long* counters;  // [0] updates, [1] fallbacks, [2] not converged, or null
  double* sink;      // the limited state of every node is also stored here (mapped host
                     // memory; the limiter after the last stage of a step), or null
};

// Residual of the saturation system at x, given svp = e_s(x[2]).
TAG_DEV void rainy_residual_at(const double* u, const double* x, double svp, double* r) {
  using C = RainyConst;
  const double rho = u[0] + u[1] + u[2];
  const double ri = 1.0 / rho;
  const double v1 = u[3] * ri, v2 = u[4] * ri;
  double r1 = (C::c_vd * u[0] + C::c_vv * x[0] + C::c_l * (x[1] + u[2])) * x[2];
  r1 += x[0] * C::ref_L;
  r1 -= (u[5] - rho * 0.5 * (v1 * v1 + v2 * v2));
  double r2 = fmin(svp / (C::R_v * x[2]), u[1]);
  r2 -= x[0];
  r2 *= 1.0e7;
  double r3 = u[1];
  r3 -= x[0] + x[1];
  r3 *= 1.0e7;
  r[0] = r1;
  r[1] = r2;
  r[2] = r3;
}

// Residual of the saturation system at x; returns e_s(x[2]), which the
// Newton update at the same x reuses.
TAG_DEV double rainy_residual(const double* u, const double* x, double* r) {
  const double svp = rainy_e_s(x[2]);
  rainy_residual_at(u, x, svp, r);
  return svp;
}

// Newton update dx = J^{-1} r with the reference Jacobian (Cramer's rule);
// svp = e_s(x[2]) as the residual at x returned it
TAG_DEV void rainy_newton_step(const double* u, const double* x, const double* r, double svp,
                               double* dx) {
  using C = RainyConst;
  const double svp_t = rainy_e_s_T_from(x[2], svp);
  const double a = C::c_vv * x[2] + C::ref_L, b = C::c_l * x[2];
  const double c = C::c_vd * u[0] + C::c_vv * x[0] + C::c_l * (x[1] + u[2]);
  const double d = -10000000.0, e = 0.0;
  const double f = (svp / (C::R_v * x[2]) < u[1]) ? (svp_t * x[2] - svp) / (C::R_v * x[2] * x[2]) * 1.0e7 : 0.0;
  const double g = -10000000.0, h = -10000000.0, i = 0.0;
  const double A = e * i - f * h, B = -(d * i - f * g), Cc = d * h - e * g;
  const double id = 1.0 / (a * A + b * B + c * Cc);
  dx[0] = (A * r[0] + (c * h - b * i) * r[1] + (b * f - c * e) * r[2]) * id;
  dx[1] = (B * r[0] + (a * i - c * g) * r[1] + (c * d - a * f) * r[2]) * id;
  dx[2] = (Cc * r[0] + (b * g - a * h) * r[1] + (a * e - b * d) * r[2]) * id;
}

TAG_DEV bool rainy_newton_done(const double* u, const double* r, int mode, double tol) {
  if (mode == 0) return fmax(fabs(r[0]), fmax(fabs(r[1]), fabs(r[2]))) < tol;
  const double rho = u[0] + u[1] + u[2];
  const double e_int = u[5] - 0.5 * (u[3] * u[3] + u[4] * u[4]) / rho;
  const double s2 = tol * 1.0e7 * fabs(u[1]);
  return fabs(r[0]) < tol * fabs(e_int) && fabs(r[1]) <= s2 && fabs(r[2]) <= s2;
}

// Size of a residual in the units of the stopping criterion: max |r| for
// mode 0; for mode 1 each component over its own scale (|E_int| for the
// energy, 1e7 rho_moist for the two mass rows), so that a size below tol is
// convergence in both modes.
TAG_DEV double rainy_residual_size(const double* u, const double* r, int mode) {
  if (mode == 0) return fmax(fabs(r[0]), fmax(fabs(r[1]), fabs(r[2])));
  const double rho = u[0] + u[1] + u[2];
  const double e_int = u[5] - 0.5 * (u[3] * u[3] + u[4] * u[4]) / rho;
  const double sm = 1.0e7 * fabs(u[1]);
  return fmax(fabs(r[0]) / fabs(e_int), fmax(fabs(r[1]), fabs(r[2])) / sm);
}

// Snaps a converged iterate to a grid fixed by the node's state: vapour and
// cloud to 2^-24 of the power of two above rho_moist, temperature to 2^-18 K.
// Two runs converged from different starts land on the same grid point unless
// they straddle a cell edge (their distance is ~1e-12 of a cell at the
// tolerance); Newton updates from that common point then agree bit for bit.
TAG_DEV void rainy_snap(const double* u, double* x) {
  int e;
  frexp(fabs(u[1]), &e);
  const double gm = ldexp(1.0, e - 24), gt = ldexp(1.0, -18);
  x[0] = rint(x[0] / gm) * gm;
  x[1] = rint(x[1] / gm) * gm;
  x[2] = rint(x[2] / gt) * gt;
}

// Newton from x; returns updates until the criterion held (maxit if never).
// With polish > 0 a converged iterate is snapped (rainy_snap) and `polish`
// further updates are taken from there; if the criterion then fails, the
// iterate before the snap is kept.  svp0 > 0 is e_s(x[2]) of the start when
// the caller has it already (a guess computed it), else 0.
TAG_DEV int rainy_newton_run(const double* u, double* x, int mode, double tol, int maxit,
                             int polish, bool& converged, double svp0 = 0.0) {
  double r[3], dx[3];
  int it = 0;
  converged = false;
  for (; it < maxit; ++it) {
    double svp;
    if (it == 0 && svp0 > 0.0) {
      svp = svp0;
      rainy_residual_at(u, x, svp, r);
    } else {
      svp = rainy_residual(u, x, r);
    }
    if (rainy_newton_done(u, r, mode, tol)) {
      converged = true;
      break;
    }
    rainy_newton_step(u, x, r, svp, dx);
    x[0] -= dx[0];
    x[1] -= dx[1];
    x[2] -= dx[2];
  }
  if (!converged) {
    rainy_residual(u, x, r);
    converged = rainy_newton_done(u, r, mode, tol);
  }
  if (polish > 0 && converged) {
    double y[3] = {x[0], x[1], x[2]};
    rainy_snap(u, y);
    for (int p = 0; p < polish; ++p) {
      const double svp = rainy_residual(u, y, r);
      rainy_newton_step(u, y, r, svp, dx);
      y[0] -= dx[0];
      y[1] -= dx[1];
      y[2] -= dx[2];
    }
    rainy_residual(u, y, r);
    if (rainy_newton_done(u, r, mode, tol)) {
      x[0] = y[0];
      x[1] = y[1];
      x[2] = y[2];
    }
  }
  return it;
}

// The closed-form unsaturated equilibrium (all moisture as vapour at T_unsat)
// when it is valid, i.e. when the vapour fits under the saturation density;
// returns false for a saturated node.  svp = e_s(T_unsat) (0 if T_unsat <= 0).
TAG_DEV bool rainy_closed_form_guess(const double* u, double* x, double& tu, double& e_int,
                                     double& svp) {
  using C = RainyConst;
  tu = rainy_t_unsat(u, e_int);
  svp = tu > 0.0 ? rainy_e_s(tu) : 0.0;
  if (tu > 0.0 && svp / (C::R_v * tu) >= u[1]) {
    x[0] = u[1];
    x[1] = 0.0;
    x[2] = tu;
    return true;
  }
  return false;
}

// Learned start: the closed-form unsaturated equilibrium where it is valid,
// else T_unsat plus the network's latent-heat offset, with vapour and cloud
// from the saturation relation at that temperature.
// Returns true where the closed form was taken; svp = e_s(x[2]).
TAG_DEV bool rainy_learned_guess(const float* __restrict__ P, const double* u, double* x,
                                 double& svp) {
  using C = RainyConst;
  double e_int, tu;
  if (rainy_closed_form_guess(u, x, tu, e_int, svp)) return true;
  float xin[kMlpIn];
  mlp_inputs(u, e_int, tu, xin);
  const double T = tu + fmax((double)mlp_forward(P, xin), 0.0);
  svp = rainy_e_s(T);
  x[2] = T;
  x[0] = fmin(svp / (C::R_v * T), u[1]);
  x[1] = u[1] - x[0];
  return false;
}

// The stage limiter at one node: the node's saturation solve from the start
// that NewtonArgs::learned selects, the guessed start falling back to the
// warm start (slots 7-9) when it has not converged after maxit_learned
// updates.  Writes slots 7-9 (and clamps negative rain); returns the Newton
// updates taken, with whether a fallback happened and whether it converged.
TAG_DEV int newton_rainy_node(const float* sp, double* __restrict__ un, const NewtonArgs& a,
                              int& fallback, bool& conv) {
  // the node's conserved variables (slots 1-6), copied before the rain
  // clamp; the solve reads no other slot
  double s[6];
#pragma unroll
  for (int v = 0; v < 6; ++v) s[v] = un[v];
  if (un[2] < 0.0) un[2] = 0.0;
  double x[3] = {un[6], un[7], un[8]};
  conv = false;
  fallback = 0;
  int its = 0;
  double xg[3], svp_g = 0.0;
  bool guessed = false;
  if (a.learned == 1 && a.mlp) {
    rainy_learned_guess(sp, s, xg, svp_g);
    guessed = true;
  } else if (a.learned == 3 && a.mlp) {
    guessed = rainy_learned_guess(sp, s, xg, svp_g);
    if (!guessed) {
      // saturated node: keep the MLP guess only where it starts closer
      double rg[3], rw[3];
      rainy_residual_at(s, xg, svp_g, rg);
      rainy_residual(s, x, rw);
      const double sg = rainy_residual_size(s, rg, a.mode);
      guessed = isfinite(sg) && sg < rainy_residual_size(s, rw, a.mode);
    }
  } else if (a.learned == 2) {
    double tu, e_int;
    guessed = rainy_closed_form_guess(s, xg, tu, e_int, svp_g);
  }
  if (guessed) {
    its = rainy_newton_run(s, xg, a.mode, a.tol, a.maxit_learned, a.polish, conv, svp_g);
    if (conv && isfinite(xg[2])) {
      x[0] = xg[0];
      x[1] = xg[1];
      x[2] = xg[2];
    } else {
      fallback = 1;
      conv = false;
    }
  }
  if (!conv) its += rainy_newton_run(s, x, a.mode, a.tol, a.maxit, a.polish, conv);
  un[6] = x[0];
  un[7] = x[1];
  un[8] = x[2];
  return its;
}

// The stage limiter over all nodes, one thread per node, 256 threads per CTA
// (launch through launch_newton_rainy); the network's parameters are staged
// in shared memory for starts 1 and 3.
static __global__ void __launch_bounds__(256) k_newton_rainy(double* __restrict__ u, long nodes,
                                                      NewtonArgs a, unsigned* __restrict__ status) {
  __shared__ float sp[kMlpParams];
  if ((a.learned == 1 || a.learned == 3) && a.mlp) {
    for (int t = threadIdx.x; t < kMlpParams; t += blockDim.x) sp[t] = a.mlp[t];
    __syncthreads();
  }
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  // every lane stays to the end for the warp's counter reduction; lanes past
  // the last node do no work and contribute zeros
  unsigned its = 0, fallbacks = 0, unconverged = 0;
  if (q < nodes) {
    int fb;
    bool conv;
    its = (unsigned)newton_rainy_node(sp, u + q * 9, a, fb, conv);
    if (a.iters) a.iters[q] = (int)its;
    if (!conv) atomicOr(status, TAG_S_NEWTON_MAXIT);
    fallbacks = (unsigned)fb;
    unconverged = conv ? 0u : 1u;
  }
  if (a.sink != nullptr) {
    // the step's result to the registered sink (host memory over the host
    // link).  A warp's nodes are consecutive, so their 32 x 9 values are 288
    // consecutive doubles: lane l stores doubles l + 32 k (k = 0..8), each
    // fetched from its node's lane, so that every store is contiguous
    const long w_first = q - (threadIdx.x & 31);
    const long valid = nodes - w_first;  // the warp's nodes in range
    double fin[9];
#pragma unroll
    for (int v = 0; v < 9; ++v) fin[v] = q < nodes ? u[q * 9 + v] : 0.0;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int d = lane + 32 * k, src = d / 9, c = d % 9;
      double val = 0.0;
#pragma unroll
      for (int v = 0; v < 9; ++v) {
        const double x = __shfl_sync(0xffffffffu, fin[v], src);
        if (v == c) val = x;
      }
      if (src < valid) a.sink[w_first * 9 + d] = val;
    }
  }
  if (a.counters) {
    // one atomic per warp and counter instead of one per node
    its = __reduce_add_sync(0xffffffffu, its);
    fallbacks = __reduce_add_sync(0xffffffffu, fallbacks);
    unconverged = __reduce_add_sync(0xffffffffu, unconverged);
    if ((threadIdx.x & 31) == 0) {
      if (its) atomicAdd(a.counters, (unsigned long long)its);
      if (fallbacks) atomicAdd(a.counters + 1, (unsigned long long)fallbacks);
      if (unconverged) atomicAdd(a.counters + 2, (unsigned long long)unconverged);
    }
  }
}

// Launches k_newton_rainy over `nodes` nodes (u[nodes][9]) on `stream`.
static inline cudaError_t launch_newton_rainy(double* u, long nodes, const NewtonArgs& a,
                                              unsigned* status, cudaStream_t stream) {
  k_newton_rainy<<<(unsigned)((nodes + 255) / 256), 256, 0, stream>>>(u, nodes, a, status);
  return cudaGetLastError();
}

}  // namespace tag
