// Shared device helpers for the DGSEM kernels (FP64 on CUDA cores).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/trixiatmo_gpu.h"

#define TAG_DEV __device__ __forceinline__

namespace tag {

// Sets the message tag_last_error() returns on this thread (defined in tag_api.cu).
void set_last_error(const std::string& msg);

constexpr int kMaxNodes = 8;  // n = polydeg + 1 supported up to polydeg 7

// Logarithmic mean and its inverse in the form of Ranocha et al., ACM TOMS 49
// (2023), arXiv:2112.10517: a 4-term series in f2 = ((x-y)/(x+y))^2 when
// f2 < 1e-4, else (y-x)/log(y/x).  Trixi.ln_mean / Trixi.inv_ln_mean are the
// reference's definitions (imported at src/TrixiAtmo.jl:37).
TAG_DEV double ln_mean(double x, double y) {
  const double f2 = (x * (x - 2.0 * y) + y * y) / (x * (x + 2.0 * y) + y * y);
  if (f2 < 1.0e-4) {
    return (x + y) * 52.5 / (105.0 + f2 * (35.0 + f2 * (21.0 + f2 * 15.0)));
  }
  return (y - x) / log(y / x);
}

TAG_DEV double inv_ln_mean(double x, double y) {
  const double f2 = (x * (x - 2.0 * y) + y * y) / (x * (x + 2.0 * y) + y * y);
  if (f2 < 1.0e-4) {
    return (105.0 + f2 * (35.0 + f2 * (21.0 + f2 * 15.0))) / (52.5 * (x + y));
  }
  return log(y / x) / (y - x);
}

// Both logarithmic means of one node pair with a single reciprocal and no
// logarithm in the common case.  With f2 = ((y-x)/(y+x))^2 and z = sqrt(f2):
//   ln_mean(x, y)     = (x+y)/2 * z/atanh(z) = (x+y)/2 * R(f2)
//   inv_ln_mean(x, y) = 2/(x+y) * atanh(z)/z = 2/(x+y) * Q(f2)
// Q(f2) = sum_k f2^k/(2k+1); R = 1/Q, its Taylor coefficients derived exactly
// from that definition.  Eight terms each are exact to ~1e-18 relative for
// f2 < 0.01, so they agree with the reference's definition (4-term form below
// f2 = 1e-4, (y-x)/log(y/x) above) to rounding.  For f2 >= 0.01 the exact
// logarithmic form is used.
//   rho_mean = ln_mean(xa, xb), inv_beta_mean = inv_ln_mean(ya, yb).
// For f2 >= 0.01 the logarithmic form (y - x)/log(y/x) is evaluated with the
// per-node logarithms Lx = log x, Ly = log y (log(y/x) = Ly - Lx; with
// |y/x - 1| > 0.2 there the difference is accurate to ~1e-14 relative).  The
// caller guarantees the logarithms are valid whenever a pair can leave the
// series range (see kLogMeanRange).
constexpr double kSeriesF2 = 1.0e-2;
// An element whose node values x satisfy ((max-min)/(max+min))^2 below this
// bound never leaves the series range (margin for rounding of f2).
constexpr double kLogMeanRange = 0.9e-2;

// The eight-term series R(f2) and Q(f2) described above
TAG_DEV double ln_series_R(double f2) {
  return 1.0 + f2 * (-1.0 / 3.0 + f2 * (-4.0 / 45.0 + f2 * (-44.0 / 945.0 +
         f2 * (-428.0 / 14175.0 + f2 * (-10196.0 / 467775.0 +
         f2 * (-10719068.0 / 638512875.0 + f2 * (-25865068.0 / 1915538625.0)))))));
}
TAG_DEV double ln_series_Q(double f2) {
  return 1.0 + f2 * (1.0 / 3.0 + f2 * (1.0 / 5.0 + f2 * (1.0 / 7.0 +
         f2 * (1.0 / 9.0 + f2 * (1.0 / 11.0 + f2 * (1.0 / 13.0 + f2 * (1.0 / 15.0)))))));
}
// Below kShortF2 the first four terms are exact to < 2e-17 relative.
constexpr double kShortF2 = 1.0e-4;

// The rare branch, kept out of line so that the common path is not predicated
// with its extra reciprocal; the series are evaluated only for a mean that is
// still in range.
static __device__ __noinline__ void ln_mean_pair_log(double sx, double dx, double sy, double dy,
                                                     double f2x, double f2y, double Lxa,
                                                     double Lxb, double Lya, double Lyb,
                                                     double& rho_mean, double& inv_beta_mean) {
  const bool lx = f2x >= kSeriesF2, ly = f2y >= kSeriesF2;
  const double nx = lx ? dx : 0.5 * sx * ln_series_R(f2x);
  const double ex = lx ? Lxb - Lxa : 1.0;
  const double ny = ly ? Lyb - Lya : 2.0 * ln_series_Q(f2y);
  const double ey = ly ? dy : sy;
  const double r2 = 1.0 / (ex * ey);
  rho_mean = nx * ey * r2;
  inv_beta_mean = ny * ex * r2;
}

// kNodeLogs: true when the caller supplies per-node logarithms (elements
// whose pairs often leave the series range, e.g. tall 3D elements); false to
// take the logarithms inside the rare branch (2D elements rarely need them).
// kShort: take the four-term series below kShortF2.  Worth it only where a
// warp's pairs share one direction (the 3D kernel); in the 2D kernel a warp
// mixes horizontal and vertical pairs and the extra branch diverges.
template <bool kNodeLogs, bool kShort = kNodeLogs>
TAG_DEV void ln_mean_pair(double xa, double xb, double ya, double yb, double Lxa, double Lxb,
                          double Lya, double Lyb, double& rho_mean, double& inv_beta_mean) {
  const double sx = xa + xb, dx = xb - xa;
  const double sy = ya + yb, dy = yb - ya;
  const double r = 1.0 / (sx * sy);
  const double isx = sy * r, isy = sx * r;
  const double tx = dx * isx, ty = dy * isy;
  const double f2x = tx * tx, f2y = ty * ty;
  const double fm = fmax(f2x, f2y);
  if (kShort && fm < kShortF2) {
    // nearly equal values (e.g. horizontal pairs of a smooth atmosphere)
    rho_mean = 0.5 * sx * (1.0 + f2x * (-1.0 / 3.0 + f2x * (-4.0 / 45.0 + f2x * (-44.0 / 945.0))));
    inv_beta_mean = 2.0 * isy * (1.0 + f2y * (1.0 / 3.0 + f2y * (1.0 / 5.0 + f2y * (1.0 / 7.0))));
  } else if (fm < kSeriesF2) {
    rho_mean = 0.5 * sx * ln_series_R(f2x);
    inv_beta_mean = 2.0 * isy * ln_series_Q(f2y);
  } else if constexpr (kNodeLogs) {
    ln_mean_pair_log(sx, dx, sy, dy, f2x, f2y, Lxa, Lxb, Lya, Lyb, rho_mean, inv_beta_mean);
  } else {
    rho_mean = f2x < kSeriesF2 ? 0.5 * sx * ln_series_R(f2x) : dx / log(xb / xa);
    inv_beta_mean = f2y < kSeriesF2 ? 2.0 * isy * ln_series_Q(f2y) : log(yb / ya) / dy;
  }
}

// The same series R and Q to sixteen terms: exact to < 1e-18 relative for
// f2 < kLongF2 = 0.09 (node values within a factor 1.86 of each other), which
// covers every pair of a tall atmospheric element without logarithms (a 3.75 km
// layer of an isothermal 250 K atmosphere reaches f2 = 0.064).  Coefficients:
// Q_k = 1/(2k+1); R = 1/Q by exact series inversion, correctly rounded.
constexpr double kLongF2 = 0.09;
// An element whose node values satisfy ((max-min)/(max+min))^2 below this bound
// keeps every pair inside kLongF2 (margin for the rounding of f2).
constexpr double kLongLogRange = 0.08;

TAG_DEV double ln_series_R16(double f2) {
  double r = -0.004746430692874202;
  r = fma(r, f2, -0.005208475658374312);
  r = fma(r, f2, -0.005756954446288888);
  r = fma(r, f2, -0.006417063031397296);
  r = fma(r, f2, -0.007224464737393906);
  r = fma(r, f2, -0.008231206567350501);
  r = fma(r, f2, -0.009516073194527899);
  r = fma(r, f2, -0.011203745637718733);
  r = fma(r, f2, -0.013502765051265932);
  r = fma(r, f2, -0.016787551856334924);
  r = fma(r, f2, -0.021796804019026242);
  r = fma(r, f2, -0.030194003527336862);
  r = fma(r, f2, -0.04656084656084656);
  r = fma(r, f2, -0.08888888888888889);
  r = fma(r, f2, -0.3333333333333333);
  return fma(r, f2, 1.0);
}
TAG_DEV double ln_series_Q16(double f2) {
  double r = 1.0 / 31.0;
  r = fma(r, f2, 1.0 / 29.0);
  r = fma(r, f2, 1.0 / 27.0);
  r = fma(r, f2, 1.0 / 25.0);
  r = fma(r, f2, 1.0 / 23.0);
  r = fma(r, f2, 1.0 / 21.0);
  r = fma(r, f2, 1.0 / 19.0);
  r = fma(r, f2, 1.0 / 17.0);
  r = fma(r, f2, 1.0 / 15.0);
  r = fma(r, f2, 1.0 / 13.0);
  r = fma(r, f2, 1.0 / 11.0);
  r = fma(r, f2, 1.0 / 9.0);
  r = fma(r, f2, 1.0 / 7.0);
  r = fma(r, f2, 1.0 / 5.0);
  r = fma(r, f2, 1.0 / 3.0);
  return fma(r, f2, 1.0);
}

// Out-of-line branch of ln_mean_pair_halved for a pair with f2 at or above
// the series range `lim` in either mean (elements flagged by needs_logs give
// per-node logarithms Lxa = log(xa/2) ...; kLogsInline takes log(y/x)
// here instead, for kernels whose elements rarely need them; differences of
// logarithms do not see the halving).  One reciprocal serves both means:
// rho_mean = nx/ex and inv_beta_mean = ny/ey.
template <int kTerms, bool kLogsInline>
static __device__ __noinline__ void ln_mean_pair_halved_log(double sx, double dx, double sy,
                                                            double dy, double f2x, double f2y,
                                                            double Lxa, double Lxb, double Lya,
                                                            double Lyb, double& rho_mean,
                                                            double& inv_beta_mean) {
  constexpr double lim = kTerms == 16 ? kLongF2 : kSeriesF2;
  const bool lx = f2x >= lim, ly = f2y >= lim;
  const double Rx = kTerms == 16 ? ln_series_R16(f2x) : ln_series_R(f2x);
  const double Qy = kTerms == 16 ? ln_series_Q16(f2y) : ln_series_Q(f2y);
  const double nx = lx ? 2.0 * dx : sx * Rx;
  const double ny = ly ? (kLogsInline ? log((sy + dy) / (sy - dy)) : Lyb - Lya) : Qy;
  const double ex = lx ? (kLogsInline ? log((sx + dx) / (sx - dx)) : Lxb - Lxa) : 1.0;
  const double ey = ly ? 2.0 * dy : sy;
  const double r2 = 1.0 / (ex * ey);
  rho_mean = nx * ey * r2;
  inv_beta_mean = ny * ex * r2;
}

// ln_mean(x_a, x_b) and inv_ln_mean(y_a, y_b) from HALVED node values
// (hx = x/2, hy = y/2, which saves the factors 1/2 and 2 of the series forms:
// ln_mean = (hx_a + hx_b) R(f2x), inv_ln_mean = Q(f2y) / (hy_a + hy_b)), one
// reciprocal per pair.  The number of series terms follows the pair's own f2
// (four below kShortF2 when kShort, else kTerms = 8 below kSeriesF2 or 16
// below kLongF2, logarithms beyond), so a pair's result does not depend on
// which pairs share its warp; the branch tests compare the bit patterns of
// the non-negative f2 on the integer pipe.  kShort pays where a warp's pairs
// share one direction (the 3D kernel); in the 2D kernel a warp mixes
// horizontal and vertical pairs, and the extra branch would diverge.
template <bool kShort = true, int kTerms = 16, bool kLogsInline = false>
TAG_DEV void ln_mean_pair_halved(double hxa, double hxb, double hya, double hyb, double Lxa,
                                 double Lxb, double Lya, double Lyb, double& rho_mean,
                                 double& inv_beta_mean) {
  static_assert(kTerms == 8 || kTerms == 16, "eight or sixteen series terms");
  constexpr double lim = kTerms == 16 ? kLongF2 : kSeriesF2;
  const double sx = hxa + hxb, dx = hxb - hxa;
  const double sy = hya + hyb, dy = hyb - hya;
  const double r = 1.0 / (sx * sy);
  const double isx = sy * r, isy = sx * r;
  const double tx = dx * isx, ty = dy * isy;
  const double f2x = tx * tx, f2y = ty * ty;
  const long long fb = max(__double_as_longlong(f2x), __double_as_longlong(f2y));
  if (kShort && fb < __double_as_longlong(kShortF2)) {
    rho_mean = sx * fma(f2x, fma(f2x, fma(f2x, -44.0 / 945.0, -4.0 / 45.0), -1.0 / 3.0), 1.0);
    inv_beta_mean = isy * fma(f2y, fma(f2y, fma(f2y, 1.0 / 7.0, 1.0 / 5.0), 1.0 / 3.0), 1.0);
  } else if (fb < __double_as_longlong(lim)) {
    rho_mean = sx * (kTerms == 16 ? ln_series_R16(f2x) : ln_series_R(f2x));
    inv_beta_mean = isy * (kTerms == 16 ? ln_series_Q16(f2y) : ln_series_Q(f2y));
  } else {
    ln_mean_pair_halved_log<kTerms, kLogsInline>(sx, dx, sy, dy, f2x, f2y, Lxa, Lxb, Lya, Lyb,
                                                 rho_mean, inv_beta_mean);
  }
}

// One logarithmic mean (or its inverse) with its own reciprocal: the series of
// ln_mean_pair in the common range, the reference's (y-x)/log(y/x) outside.
TAG_DEV double ln_mean_single(double x, double y) {
  const double s = x + y, d = y - x;
  const double t = d / s, f2 = t * t;
  if (f2 < kSeriesF2) {
    const double R = 1.0 + f2 * (-1.0 / 3.0 + f2 * (-4.0 / 45.0 + f2 * (-44.0 / 945.0 +
                     f2 * (-428.0 / 14175.0 + f2 * (-10196.0 / 467775.0 +
                     f2 * (-10719068.0 / 638512875.0 + f2 * (-25865068.0 / 1915538625.0)))))));
    return 0.5 * s * R;
  }
  return d / log(y / x);
}

TAG_DEV double inv_ln_mean_single(double x, double y) {
  const double s = x + y, d = y - x;
  const double t = d / s, f2 = t * t;
  if (f2 < kSeriesF2) {
    const double Q = 1.0 + f2 * (1.0 / 3.0 + f2 * (1.0 / 5.0 + f2 * (1.0 / 7.0 +
                     f2 * (1.0 / 9.0 + f2 * (1.0 / 11.0 + f2 * (1.0 / 13.0 + f2 * (1.0 / 15.0)))))));
    return 2.0 * Q / s;
  }
  return log(y / x) / d;
}

// Whether the values of one element can push a node pair out of the series
// range of ln_mean_pair.
TAG_DEV bool needs_logs(double vmin, double vmax, double range = kLogMeanRange) {
  const double t = (vmax - vmin) / (vmax + vmin);
  return t * t >= range;
}

// Face node (i, j) of face f (0 = xi-, 1 = xi+, 2 = eta-, 3 = eta+) at index l.
TAG_DEV void face_node(int f, int l, int n, int& i, int& j) {
  if (f < 2) {
    i = (f == 0) ? 0 : n - 1;
    j = l;
  } else {
    i = l;
    j = (f == 2) ? 0 : n - 1;
  }
}

// Atomic max of a non-negative double stored as its IEEE bit pattern.
TAG_DEV void atomic_max_nonneg(double* addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(addr),
            static_cast<unsigned long long>(__double_as_longlong(v)));
}

// Carpenter-Kennedy RK4(3)5[2N] coefficients (NASA TM-109112, 1994).
struct CK2N54 {
  double A[5], B[5], c[5];
};

__host__ __device__ inline CK2N54 ck2n54() {
  return CK2N54{{0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                 -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0},
                {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                 1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                 2277821191437.0 / 14882151754819.0},
                {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                 2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0}};
}

// One stage of a time integrator in the form the element kernels apply:
//   2N (ssp = 0):  k = A k + dt du,  u = u + B k
//   SSP (ssp = 1): w = u + (B dt) du,  u = A k + C w  (u = w where A = 0),
//                  k = u at the first stage (save), the step's starting state.
// The SSP schemes are the Shu-Osher forms of SSPRK43 (Kraaijevanger 1991;
// h = dt/2: u1 = u + h L(u), u2 = u1 + h L(u1), u3 = 2/3 u + 1/3 (u2 + h L(u2)),
// u_new = u3 + h L(u3)) and SSPRK33 (Shu & Osher 1988: u1 = u + dt L(u),
// u2 = 3/4 u + 1/4 (u1 + dt L(u1)), u_new = 1/3 u + 2/3 (u2 + dt L(u2))).
struct StageCoef {
  double A, B, C, c;  // c: stage time fraction
  int ssp, save;
};

inline int rk_stages(int scheme) {
  return scheme == TAG_RK_SSPRK43 ? 4 : scheme == TAG_RK_SSPRK33 ? 3 : 5;
}

inline StageCoef rk_stage(int scheme, int s) {
  if (scheme == TAG_RK_SSPRK43) {
    static const double c[4] = {0.0, 0.5, 1.0, 0.5};
    if (s == 2) return StageCoef{2.0 / 3.0, 0.5, 1.0 / 3.0, c[s], 1, 0};
    return StageCoef{0.0, 0.5, 1.0, c[s], 1, s == 0};
  }
  if (scheme == TAG_RK_SSPRK33) {
    static const double c[3] = {0.0, 1.0, 0.5};
    if (s == 1) return StageCoef{0.75, 1.0, 0.25, c[s], 1, 0};
    if (s == 2) return StageCoef{1.0 / 3.0, 1.0, 2.0 / 3.0, c[s], 1, 0};
    return StageCoef{0.0, 1.0, 1.0, c[s], 1, 1};
  }
  const CK2N54 ck = ck2n54();
  return StageCoef{ck.A[s], ck.B[s], 0.0, ck.c[s], 0, 0};
}

// Step control shared by all ensemble members (device memory, so a captured
// graph picks up new values without re-instantiation).
struct StepCtl {
  double cfl;
  double fixed_dt;
};

// Per-member step scalars, each an array of nmembers doubles in device memory.
struct MemberScalars {
  double* t;          // start time of the current step
  double* dt;         // current step size
  double* max_speed;  // running max over elements of (max lambda1 + max lambda2)
};

}  // namespace tag
