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
// Q(f2) = sum_k f2^k/(2k+1) and R = 1/Q.  Below kShortF2 the four-term Taylor
// forms are exact to < 2e-17 relative.  On the wider ranges [0, F] R and Q are
// polynomials 1 + f2 (c0 + f2 (c1 + ...)), Chebyshev economizations of their
// Taylor series (C. Lanczos, J. Math. Phys. 17 (1938) 123-199; coefficients
// made and checked by csrc/log_mean_series.py): six coefficients each for
// F = kSeriesF2 = 0.01 (exact to < 5e-19 relative), nine (R) and ten (Q) for
// F = kLongF2 = 0.09 (< 4e-18).  So they agree with the reference's definition
// (a 4-term series below f2 = 1e-4, (y-x)/log(y/x) above) to rounding.
//   rho_mean = ln_mean(xa, xb), inv_beta_mean = inv_ln_mean(ya, yb).
// Beyond the series range the logarithmic form (y - x)/log(y/x) is evaluated,
// from per-node logarithms Lx = log x, Ly = log y where the caller supplies
// them (log(y/x) = Ly - Lx; with |y/x - 1| > 0.2 there the difference is
// accurate to ~1e-14 relative).  Such a caller guarantees the logarithms are
// valid whenever a pair can leave the series range (see kLogMeanRange).
constexpr double kShortF2 = 1.0e-4;
constexpr double kSeriesF2 = 1.0e-2;
// An element whose node values x satisfy ((max-min)/(max+min))^2 below this
// bound never leaves the series range (margin for rounding of f2).
constexpr double kLogMeanRange = 0.9e-2;
constexpr double kLongF2 = 0.09;
// The same bound for kLongF2: a 3.75 km layer of an isothermal 250 K
// atmosphere reaches f2 = 0.064, so tall shell elements stay in range.
constexpr double kLongLogRange = 0.08;

TAG_DEV double ln_short_R(double f2) {
  return fma(f2, fma(f2, fma(f2, -44.0 / 945.0, -4.0 / 45.0), -1.0 / 3.0), 1.0);
}
TAG_DEV double ln_short_Q(double f2) {
  return fma(f2, fma(f2, fma(f2, 1.0 / 7.0, 1.0 / 5.0), 1.0 / 3.0), 1.0);
}

// R and Q on [0, kSeriesF2]
TAG_DEV double ln_series_R(double f2) {
  double r = -0.01719901874634888;
  r = fma(r, f2, -0.021792151641765893);
  r = fma(r, f2, -0.030194027707754922);
  r = fma(r, f2, -0.0465608465041037);
  r = fma(r, f2, -0.08888888888893755);
  r = fma(r, f2, -0.3333333333333333);
  return fma(r, f2, 1.0);
}
TAG_DEV double ln_series_Q(double f2) {
  double r = 0.07895661799581076;
  r = fma(r, f2, 0.09088609072099012);
  r = fma(r, f2, 0.11111123067087354);
  r = fma(r, f2, 0.14285714257655663);
  r = fma(r, f2, 0.20000000000024065);
  r = fma(r, f2, 0.3333333333333333);
  return fma(r, f2, 1.0);
}

// R and Q on [0, kLongF2]
TAG_DEV double ln_series_R_long(double f2) {
  double r = -0.013669329626825622;
  r = fma(r, f2, -0.01045355622562932);
  r = fma(r, f2, -0.013573328231670736);
  r = fma(r, f2, -0.016783737201999518);
  r = fma(r, f2, -0.02179692429315078);
  r = fma(r, f2, -0.030194001406289393);
  r = fma(r, f2, -0.04656084657952881);
  r = fma(r, f2, -0.08888888888882568);
  r = fma(r, f2, -0.33333333333333337);
  return fma(r, f2, 1.0);
}
TAG_DEV double ln_series_Q_long(double f2) {
  double r = 0.07283496074780077;
  r = fma(r, f2, 0.047418568133941144);
  r = fma(r, f2, 0.05939688448611953);
  r = fma(r, f2, 0.06662915697122629);
  r = fma(r, f2, 0.07692458351815545);
  r = fma(r, f2, 0.09090905424531916);
  r = fma(r, f2, 0.11111111162196165);
  r = fma(r, f2, 0.14285714285353665);
  r = fma(r, f2, 0.20000000000000986);
  r = fma(r, f2, 0.3333333333333333);
  return fma(r, f2, 1.0);
}

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
// inv_sum_y (optional): 1/(ya + yb), a by-product of the shared reciprocal.
template <bool kNodeLogs, bool kShort = kNodeLogs>
TAG_DEV void ln_mean_pair(double xa, double xb, double ya, double yb, double Lxa, double Lxb,
                          double Lya, double Lyb, double& rho_mean, double& inv_beta_mean,
                          double* inv_sum_y = nullptr) {
  const double sx = xa + xb, dx = xb - xa;
  const double sy = ya + yb, dy = yb - ya;
  const double r = 1.0 / (sx * sy);
  const double isx = sy * r, isy = sx * r;
  if (inv_sum_y) *inv_sum_y = isy;
  const double tx = dx * isx, ty = dy * isy;
  const double f2x = tx * tx, f2y = ty * ty;
  const double fm = fmax(f2x, f2y);
  if (kShort && fm < kShortF2) {
    // nearly equal values (e.g. horizontal pairs of a smooth atmosphere)
    rho_mean = 0.5 * sx * ln_short_R(f2x);
    inv_beta_mean = 2.0 * isy * ln_short_Q(f2y);
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

// Out-of-line branch of ln_mean_pair_halved for a pair with f2 at or above
// the series range lim (kLongF2 or kSeriesF2) in either mean (elements
// flagged by needs_logs give per-node logarithms Lxa = log(xa/2) ...;
// kLogsInline takes log(y/x) here instead, for kernels whose elements rarely
// need them; differences of logarithms do not see the halving).  One
// reciprocal serves both means: rho_mean = nx/ex and inv_beta_mean = ny/ey.
template <bool kLong, bool kLogsInline>
static __device__ __noinline__ void ln_mean_pair_halved_log(double sx, double dx, double sy,
                                                            double dy, double f2x, double f2y,
                                                            double Lxa, double Lxb, double Lya,
                                                            double Lyb, double& rho_mean,
                                                            double& inv_beta_mean) {
  constexpr double lim = kLong ? kLongF2 : kSeriesF2;
  const bool lx = f2x >= lim, ly = f2y >= lim;
  const double Rx = kLong ? ln_series_R_long(f2x) : ln_series_R(f2x);
  const double Qy = kLong ? ln_series_Q_long(f2y) : ln_series_Q(f2y);
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
// reciprocal per pair.  Each mean takes the form its own f2 selects: the
// four-term series below kShortF2 (when kShort), else the polynomial on
// [0, kLongF2] (kLong) or [0, kSeriesF2]; logarithms for both once either f2
// is beyond that range.  So a pair's result does not depend on which pairs
// share its warp, and in a tall element's vertical lines, where the density
// varies and the temperature hardly does, inv_ln_mean keeps its short form.
// The branch tests compare the bit patterns of the non-negative f2 on the
// integer pipe.  kShort pays where a warp's pairs share one direction (both
// element kernels order their pairs so).
template <bool kShort = true, bool kLong = true, bool kLogsInline = false>
TAG_DEV void ln_mean_pair_halved(double hxa, double hxb, double hya, double hyb, double Lxa,
                                 double Lxb, double Lya, double Lyb, double& rho_mean,
                                 double& inv_beta_mean) {
  constexpr double lim = kLong ? kLongF2 : kSeriesF2;
  const double sx = hxa + hxb, dx = hxb - hxa;
  const double sy = hya + hyb, dy = hyb - hya;
  const double r = 1.0 / (sx * sy);
  const double isx = sy * r, isy = sx * r;
  const double tx = dx * isx, ty = dy * isy;
  const double f2x = tx * tx, f2y = ty * ty;
  const long long bx = __double_as_longlong(f2x), by = __double_as_longlong(f2y);
  if (max(bx, by) >= __double_as_longlong(lim)) {
    ln_mean_pair_halved_log<kLong, kLogsInline>(sx, dx, sy, dy, f2x, f2y, Lxa, Lxb, Lya, Lyb,
                                                rho_mean, inv_beta_mean);
    return;
  }
  double R, Q;
  if (kShort && bx < __double_as_longlong(kShortF2))
    R = ln_short_R(f2x);
  else
    R = kLong ? ln_series_R_long(f2x) : ln_series_R(f2x);
  if (kShort && by < __double_as_longlong(kShortF2))
    Q = ln_short_Q(f2y);
  else
    Q = kLong ? ln_series_Q_long(f2y) : ln_series_Q(f2y);
  rho_mean = sx * R;
  inv_beta_mean = isy * Q;
}

// One logarithmic mean (or its inverse) with its own reciprocal: the series of
// ln_mean_pair in the common range, the reference's (y-x)/log(y/x) outside.
TAG_DEV double ln_mean_single(double x, double y) {
  const double s = x + y, d = y - x;
  const double t = d / s, f2 = t * t;
  if (f2 < kSeriesF2) return 0.5 * s * ln_series_R(f2);
  return d / log(y / x);
}

TAG_DEV double inv_ln_mean_single(double x, double y) {
  const double s = x + y, d = y - x;
  const double t = d / s, f2 = t * t;
  if (f2 < kSeriesF2) return 2.0 * ln_series_Q(f2) / s;
  return log(y / x) / d;
}

// !(x > 0.0) and !isfinite(x) on the integer pipe (the FP64 pipe is the
// element kernels' bottleneck): IEEE bit patterns of positive doubles order
// like their values, and an exponent field of all ones is an infinity or NaN.
TAG_DEV bool not_positive(double x) {
  return (unsigned long long)__double_as_longlong(x) - 1ull >= 0x7ff0000000000000ull;
}
TAG_DEV bool not_finite(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) ==
         0x7ff0000000000000ull;
}

// Whether the values of one element can push a node pair out of the series
// range of ln_mean_pair.
TAG_DEV bool needs_logs(double vmin, double vmax, double range = kLogMeanRange) {
  const double t = (vmax - vmin) / (vmax + vmin);
  return t * t >= range;
}

// needs_logs for the two positive node fields q[node * stride + ka] and
// q[node * stride + kb] of one element, evaluated by one whole warp; the
// minima and maxima are taken on the integer pipe (the bit patterns of
// positive doubles order like their values).  Valid in every lane.
TAG_DEV bool element_needs_logs(const double* q, int nodes, int stride, int ka, int kb,
                                double range) {
  const int lane = threadIdx.x & 31;
  long long a0 = 0x7fefffffffffffffll, a1 = 0, b0 = 0x7fefffffffffffffll, b1 = 0;
  for (int node = lane; node < nodes; node += 32) {
    const long long x = __double_as_longlong(q[node * stride + ka]);
    const long long y = __double_as_longlong(q[node * stride + kb]);
    a0 = min(a0, x);
    a1 = max(a1, x);
    b0 = min(b0, y);
    b1 = max(b1, y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 = min(a0, __shfl_xor_sync(0xffffffffu, a0, o));
    a1 = max(a1, __shfl_xor_sync(0xffffffffu, a1, o));
    b0 = min(b0, __shfl_xor_sync(0xffffffffu, b0, o));
    b1 = max(b1, __shfl_xor_sync(0xffffffffu, b1, o));
  }
  return needs_logs(__longlong_as_double(a0), __longlong_as_double(a1), range) ||
         needs_logs(__longlong_as_double(b0), __longlong_as_double(b1), range);
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
