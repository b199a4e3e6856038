// dg_device.cuh -- equation modules, problem plugins and per-order tables
// for the sm_103a kernels.
//
// Equation modules follow the reference's compile-time plugin contract
// (src/2d/conservation/conserv_headers.cuh:5-34) as C++ traits: physical
// flux (eval_flux), numerical flux (riemann_solver), admissibility
// (is_physical), the CFL wave speed of a cell mean (eval_global_lambda) and
// the boundary ghost state (eval_boundary + the problem's U_* functions).
#pragma once
#include <cuda_runtime.h>

#include "dg_launch.h"
#include "dg_tables_data.h"

#define DG_HD __host__ __device__ __forceinline__

namespace dg {

constexpr int np_of(int p) { return (p + 1) * (p + 2) / 2; }
constexpr int nq_of(int p) { return p == 0 ? 1 : p == 1 ? 3 : p == 2 ? 6 : p == 3 ? 12 : p == 4 ? 16 : 25; }

// Per-order tabulation passed to every kernel as a __grid_constant__
// parameter: with the loops below fully unrolled every table entry is a
// constant-bank operand of the FP64 FMA that uses it.
template <int P>
struct Tab {
  static constexpr int NP = np_of(P), NQ = nq_of(P), N1 = P + 1;
  double B[NQ][NP];      // phi_i at volume point q
  double GR[NQ][NP];     // w_q dphi_i/dr
  double GS[NQ][NP];     // w_q dphi_i/ds
  double E[3][N1][NP];   // phi_i at edge point j of face f (face 2 reversed)
  double r[NQ], s[NQ], w[NQ];
  double t1[N1], w1[N1];
  double V[3][NP];       // phi_i at the vertices (0,0), (1,0), (0,1)
};


enum Problem {
  PB_NONE = 0, PB_ADV_SINE = 1, PB_ADV_LINEAR = 2, PB_EULER_VORTEX = 3, PB_EULER_RIEMANN4 = 4,
  PB_EULER_SUPERSONIC = 5, PB_SW_HUMP = 6, PB_SW_TEST = 7, PB_MAXWELL_PLANE = 8,
  PB_EULER_CYLINDER = 9, PB_EULER_LSHOCK = 10, PB_EULER_DOUBLEMACH = 11, PB_EULER_AIRFOIL = 12,
  PB_ADV_SQUAREHILL = 13, PB_ADV_ROTATINGHILL = 14, PB_ADV_SPIN = 15, PB_MAXWELL_CMIRROR = 16,
  PB_MAXWELL_WSCATTER = 17, PB_EULER_PULSE = 18
};

// double Mach reflection (euler/doublemach/doublemach.cu): the wall starts at
// x = 1/6; the post-shock state (rho 8, speed 8.25 at -30 degrees, p 116.5)
// and the quiescent gas (rho = gamma, p = 1)
constexpr double kDmX0 = 0.16666666666666666;
DG_HD void dm_shock(const EqP &q, double *U) {
  const double c = 0.86602540378443864676, s = 0.5;  // cos, sin of 30 degrees
  U[0] = 8.;
  U[1] = 8.25 * c * U[0];
  U[2] = -8.25 * s * U[0];
  U[3] = fma(0.5 * U[0], 8.25 * 8.25, 116.5 / (q.gamma - 1.0));
}
DG_HD void dm_rest(const EqP &q, double *U) {
  U[0] = q.gamma;
  U[1] = 0.;
  U[2] = 0.;
  U[3] = 1. / (q.gamma - 1.0);
}
// uniform flow along x at Mach M (cylinder.cu, lshock.cu: rho = gamma, p = 1)
DG_HD void uniform_mach(const EqP &q, double M, double *U) {
  U[0] = q.gamma;
  U[1] = U[0] * M;
  U[2] = 0.;
  U[3] = fma(0.5 * U[0], M * M, 1. / (q.gamma - 1.0));
}

constexpr double kPi = 3.141592653589793238462643383279502884;

// a Gaussian hill A exp(-|x - x0|^2 / (2 r^2)) carried by the solid rotation
// of angular speed w about the origin: the state at time t is the initial
// hill at the point rotated back by w t (rotatinghill.cu:58-67, whose
// inflow is this formula; spin.cu has the same form with its own hill)
DG_HD double rotated_hill(double A, double x0, double y0, double r, double w, double x, double y,
                          double t) {
  const double c = cos(w * t), s = sin(w * t);
  const double dx = fma(x, c, fma(y, s, -x0)), dy = fma(-x, s, fma(y, c, -y0));
  return A * exp(-fma(dx, dx, dy * dy) / (2 * r * r));
}
// rotation speeds of the two rotating problems: each file's velocity field
// (-2 PI y, 2 PI x) with its own PI (rotatinghill.cu:10, spin.cu:10)
constexpr double kRotHill = 2 * 3.14159265358979323, kRotSpin = 2 * 3.14159;

// the inflow pressure series of the tube and trumpet problems (tube.cu:52-97,
// trumpet.cu: U_inflow): p(t) = 1 + sum_k amp_k cos(omega_k (t + t0) +
// phase_k), rho = gamma p^(1/gamma), u = (p - 1) / gamma, v = 0
DG_HD void pulse_state(const EqP &q, double t, double *U) {
  double p = 1.0;
  const double tt = t + q.ser_t0;
  for (int k = 0; k < q.nser; k++) p += q.ser[k][0] * cos(fma(q.ser[k][1], tt, q.ser[k][2]));
  const double rho = q.gamma * pow(p, 1. / q.gamma), u = (p - 1) / q.gamma;
  U[0] = rho;
  U[1] = u * rho;
  U[2] = 0.;
  U[3] = fma(0.5 * rho, u * u, p / (q.gamma - 1.));
}

// a product that is not fused into an FMA with a later add (same rounding in
// every kernel instance that inlines the caller)
DG_HD double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

// 1/x for the flux evaluations, from the approximate reciprocal r of the PTX
// instruction rcp.approx.ftz.f64 (about 20 correct bits) by one third-order
// step of the Newton-Raphson family: with e = 1 - x r, 1/x = r / (1 - e) =
// r (1 + e + e^2 + ...), and r (1 + e + e^2) leaves a relative error of e^3,
// far below the 53 bits of a double.  The result is within 1 ulp of 1/x for
// normal x (checked against IEEE division by dg_probe_reciprocal).  Three
// FMAs where an IEEE division costs about three times that.
DG_HD double rcp(double x) {
#ifdef __CUDA_ARCH__
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
#else
  return 1.0 / x;
#endif
}

#ifdef __CUDACC__
// x to single precision from its high word alone, with integer instructions:
// sign, exponent rebiased, the top 20 of the 52 fraction bits (relative
// error below 2^-20); a zero or denormal x (exponent field 0) becomes a zero
// of its sign (off by less than 2^-1022: a denormal's square is far below
// any margin the filter below relies on); NaN when x is outside the normal
// float range otherwise
__device__ __forceinline__ float f32_of_hi(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned ex = (hi >> 20) & 0x7FFu;
  const unsigned b = (hi & 0x80000000u) | ((ex - 896u) << 23) | ((hi & 0xFFFFFu) << 3);
  return __uint_as_float(ex == 0u ? (hi & 0x80000000u) : ex - 897u < 253u ? b : 0x7FC00000u);
}

// true only if the Euler state U (rho, m_x, m_y, E) is physical (rho >= 0,
// 2 rho E >= |m|^2): with rho > 0 and a = 2 rho E in the normal range, a
// and b = |m|^2 formed in single precision from 20-bit copies are each
// within 2^-18.8 of the exact products, so a - b > 2^-16 (a + b) proves
// 2 rho E > |m|^2 with room for the FP64 test's own rounding (2^-51).
// False means "not settled here" (NaN, out of range, tiny, or close to the
// boundary), never "non-physical"
__device__ __forceinline__ bool physical_f32(const double *U) {
  const float r = f32_of_hi(U[0]), mx = f32_of_hi(U[1]), my = f32_of_hi(U[2]),
              E = f32_of_hi(U[3]);
  const float a = __fmul_rn(__fmul_rn(2.0f, r), E);
  const float b = __fmaf_rn(mx, mx, __fmul_rn(my, my));
  return r > 0.0f && a > 1e-30f &&
         __fsub_rn(a, b) > __fmul_rn(1.52587890625e-05f, __fadd_rn(a, b));
}
#endif

// sqrt(x) for the sound speeds, from the approximate reciprocal square root
// y of the PTX instruction rsqrt.approx.ftz.f64: with s = x y and e = 1 - s y
// (= 1 - x y^2), sqrt(x) = s (1 - e)^(-1/2) = s (1 + e/2 + 3 e^2 / 8 + ...),
// and the truncated series leaves a relative error of about e^3.  Five FP64
// operations; arguments outside the positive normal range (0, denormals,
// infinities, NaN, negatives) take the IEEE square root.  Checked against
// IEEE sqrt by dg_probe_sqrt (within 1 ulp).
DG_HD double sqrt_pos(double x) {
#ifdef __CUDA_ARCH__
  const unsigned hi = (unsigned)__double2hiint(x);
  if (hi - 0x00100000u < 0x7FE00000u) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double s = x * y;
    const double e = fma(-s, y, 1.0);
    return fma(s, e * fma(e, 0.375, 0.5), s);
  }
#endif
  return sqrt(x);
}

// --------------------------------------------------------------------------
// problem plugins: exact / initial / inflow state (U0, U_exact, U_inflow)
// --------------------------------------------------------------------------
DG_HD void exact_state(const EqP &q, double *U, double x, double y, double t) {
  const double *P = q.prm;
  switch (q.problem) {
    case PB_ADV_SINE: {
      double xs = x - q.ax * t, ys = y - q.ay * t;
      U[0] = sin(2 * kPi * xs) * sin(2 * kPi * ys);
      break;
    }
    case PB_ADV_LINEAR:  // advection/exact/exact.cu:25-27
      U[0] = x - y;
      break;
    case PB_EULER_VORTEX: {  // isentropic vortex, centre advected with (uinf, vinf)
      double gam = q.gamma, beta = P[0], L = P[5];
      double dx = x - (P[1] + P[3] * t), dy = y - (P[2] + P[4] * t);
      if (L > 0) {
        dx -= L * floor(dx / L + 0.5);
        dy -= L * floor(dy / L + 0.5);
      }
      double r2 = fma(dx, dx, dy * dy);
      double e = exp(0.5 * (1 - r2));
      double u = P[3] - beta / (2 * kPi) * e * dy;
      double v = P[4] + beta / (2 * kPi) * e * dx;
      double T = 1 - (gam - 1) * beta * beta / (8 * gam * kPi * kPi) * e * e;
      double rho = pow(T, 1 / (gam - 1));
      double p = pow(rho, gam);
      U[0] = rho;
      U[1] = rho * u;
      U[2] = rho * v;
      U[3] = fma(0.5 * rho, fma(u, u, v * v), p / (gam - 1));
      break;
    }
    case PB_EULER_RIEMANN4: {  // four-quadrant Riemann data split at (0.5, 0.5)
      double gam = q.gamma, rho, u, v, p;
      if (x >= 0.5 && y >= 0.5) { rho = 1.5; u = 0; v = 0; p = 1.5; }
      else if (x < 0.5 && y >= 0.5) { rho = 0.5323; u = 1.206; v = 0; p = 0.3; }
      else if (x < 0.5 && y < 0.5) { rho = 0.138; u = 1.206; v = 1.206; p = 0.029; }
      else { rho = 0.5323; u = 0; v = 1.206; p = 0.3; }
      U[0] = rho;
      U[1] = rho * u;
      U[2] = rho * v;
      U[3] = fma(0.5 * rho, fma(u, u, v * v), p / (gam - 1));
      break;
    }
    case PB_EULER_SUPERSONIC: {  // euler/supersonic/supersonic.cu:27-37
      const double GAM = 1.4, MACH = 2.25;
      double r = sqrt(fma(x, x, y * y));
      U[0] = pow(1 + 1.0125 * (1. - 1. / (r * r)), 2.5);
      U[1] = U[0] * sin(atan(y / x)) * MACH / r;
      U[2] = U[0] * -cos(atan(y / x)) * MACH / r;
      double p = (1.0 / GAM) * pow(U[0], GAM);
      U[3] = fma(0.5 * U[0], MACH * MACH / (r * r), p * (1. / (GAM - 1.)));
      break;
    }
    case PB_SW_HUMP: {  // still water with a Gaussian hump: h0, A, sigma, x0, y0
      double dx = x - P[3], dy = y - P[4], s = P[2];
      U[0] = fma(P[1], exp(-fma(dx, dx, dy * dy) / (s * s)), P[0]);
      U[1] = 0;
      U[2] = 0;
      break;
    }
    case PB_SW_TEST:  // shallowwater/test/test.cu:25-35
      U[0] = 10 + exp(-fma(x - 0.5, x - 0.5, (y - 0.5) * (y - 0.5)) / (2 * 0.1 * 0.1));
      U[1] = 0;
      U[2] = 0;
      break;
    case PB_EULER_CYLINDER:  // cylinder.cu:23-45: U0 = U_inflow = U_outflow, Mach 0.38
      uniform_mach(q, P[0] != 0 ? P[0] : 0.38, U);
      break;
    case PB_EULER_LSHOCK:  // lshock.cu:23-45, Mach 2
      uniform_mach(q, P[0] != 0 ? P[0] : 2.0, U);
      break;
    case PB_EULER_DOUBLEMACH:  // doublemach.cu:55-70: U_inflow = U_outflow
      if (x < kDmX0 + (1. + 20. * t) / sqrt(3.)) dm_shock(q, U);
      else dm_rest(q, U);
      break;
    case PB_EULER_AIRFOIL: {  // airfoil.cu:22-45: uniform flow at Mach P[0] (0: 0.98),
                              // P[1] degrees (0: 5)
      const double M = P[0] != 0 ? P[0] : 0.98, a = (P[1] != 0 ? P[1] : 5.) * (kPi / 180.);
      U[0] = q.gamma;
      U[1] = U[0] * M * cos(a);
      U[2] = U[0] * M * sin(a);
      U[3] = fma(0.5 * U[0], M * M, 1. / (q.gamma - 1.0));
      break;
    }
    case PB_EULER_PULSE:  // U_inflow = U_outflow
      pulse_state(q, t, U);
      break;
    case PB_ADV_SQUAREHILL: {  // squarehill.cu:22-30, translated by a t
      const double xs = x - q.ax * t, ys = y - q.ay * t;
      U[0] = (xs < -.2 && xs > -.8 && ys < .1 && ys > -.5) ? 1. : 0.;
      break;
    }
    case PB_ADV_ROTATINGHILL:
      U[0] = rotated_hill(5., 0.2, 0.0, 0.15, kRotHill, x, y, t);
      break;
    case PB_ADV_SPIN:  // spin.cu:22-30
      U[0] = rotated_hill(1., 0.5, 0.5, 0.1, kRotSpin, x, y, t);
      break;
    case PB_MAXWELL_PLANE: {  // plane TM wave along x
      double c = 1 / sqrt(q.mu * q.eps);
      double ez = sin(2 * kPi * (x - c * t));
      U[0] = 0;
      U[1] = sqrt(q.eps / q.mu) * ez;
      U[2] = ez;
      break;
    }
    default:
      U[0] = U[1] = U[2] = U[3] = 0;
  }
}

// the inflow state (U_inflow): the exact state, except where a problem's
// inflow differs from it
DG_HD void inflow_state(const EqP &q, double *U, double x, double y, double t) {
  switch (q.problem) {
    case PB_ADV_SQUAREHILL:  // squarehill.cu:43-45
    case PB_ADV_SPIN:        // spin.cu:43-46
      U[0] = 0.;
      return;
    case PB_MAXWELL_CMIRROR:  // cmirror.cu:38-47: a half-period pulse of E_z
      U[0] = U[1] = 0.;
      U[2] = t <= 1. / 20 ? 2 * sin(20. * kPi * t) : 0.;
      return;
    case PB_MAXWELL_WSCATTER:  // wscatter.cu:38-50: a pulse through a slit |y| < 0.15
      U[0] = U[1] = 0.;
      U[2] = (y < .15 && y > -.15 && t < 0.5) ? sin(2. * kPi * t) : 0.;
      return;
    default:
      exact_state(q, U, x, y, t);
  }
}

// the initial state (U0): the exact state at t = 0, except where a problem's
// initial data differ from its boundary data
DG_HD void init_state(const EqP &q, double *U, double x, double y) {
  if (q.problem == PB_EULER_DOUBLEMACH) {  // doublemach.cu:41-52: shock at 60 degrees
    const double angle = atan(y / (x - kDmX0));
    if (angle > 60. * kPi / 180 || x < kDmX0) dm_shock(q, U);
    else dm_rest(q, U);
    return;
  }
  if (q.problem == PB_EULER_PULSE) {  // tube.cu:25-45: gas at rest, rho = gamma, p = 1
    dm_rest(q, U);
    return;
  }
  exact_state(q, U, x, y, 0.0);
}

// --------------------------------------------------------------------------
// equation modules
// --------------------------------------------------------------------------
struct Advection {  // advection/advection.cu
  static constexpr int N = 1;
  static constexpr bool kBathymetry = false;
  // the velocity may vary in space (q.field): fluxes then take the position
  static constexpr bool kField = true;
  static constexpr bool kFolded = false;
  DG_HD static bool physical(const EqP &, const double *) { return true; }
  DG_HD static void flux(const EqP &q, const double *U, double *fx, double *fy) {
    fx[0] = q.ax * U[0];
    fy[0] = q.ay * U[0];
  }
  // get_velocity (advection.cu:12; rotatinghill.cu:37-40): the affine field
  // a(x, y) = (ax, ay) + agrad (x, y)
  DG_HD static void velocity(const EqP &q, double x, double y, double &vx, double &vy) {
    vx = fma(q.agrad[0], x, fma(q.agrad[1], y, q.ax));
    vy = fma(q.agrad[2], x, fma(q.agrad[3], y, q.ay));
  }
  // eval_flux with the velocity at the point (advection.cu:51-72)
  DG_HD static void flux_at(double vx, double vy, const double *U, double *fx, double *fy) {
    fx[0] = vx * U[0];
    fy[0] = vy * U[0];
  }
  // upwind flux with the velocity at the point (advection.cu:94-116)
  DG_HD static void riemann_at(double vx, double vy, const double *UL, const double *UR,
                               double nx, double ny, double *F) {
    double an = fma(nx, vx, ny * vy);
    F[0] = an > 0 ? an * UL[0] : an * UR[0];
  }
  // upwind flux (riemann_solver_upwind, advection.cu:94-116)
  // riemann_raw(..) * kRawScale is the numerical flux; face kernels fold the
  // (exact, power-of-two) scale into their own edge-length factor
  static constexpr double kRawScale = 1.0;
  DG_HD static void riemann_raw(const EqP &q, const double *UL, const double *UR, double nx,
                                double ny, double *F) {
    double an = fma(nx, q.ax, ny * q.ay);
    F[0] = an > 0 ? an * UL[0] : an * UR[0];
  }
  DG_HD static double mean_speed(const EqP &q, const double *) {
    // a field: the largest speed over the elements, each taken at its middle
    // quadrature point (eval_global_lambda, advection.cu:157-183), which
    // does not change in time and is found once on the host
    return q.field ? q.amax : sqrt(fma(q.ax, q.ax, q.ay * q.ay));
  }
  DG_HD static void reflect(const EqP &, const double *, double *UR, double, double, double,
                            double) {
    UR[0] = 0;  // the reference's advection problems have no reflecting walls
  }
  static constexpr bool outflow_uses_exact = false;
};

struct Euler {  // euler/euler.cu
  static constexpr int N = 4;
  static constexpr bool kBathymetry = false;
  static constexpr bool kField = false;
  // rho >= 0 and p >= 0 (is_physical, euler.cu:76-86); with rho > 0,
  // p < 0 <=> 2 rho E < |rho u|^2, which needs no FP64 division.  On the
  // device a single-precision test settles almost every state first
  // (physical_f32); only what it leaves open takes the FP64 test, so every
  // decision is the FP64 test's
  DG_HD static bool physical_fp64(const double *U) {
    if (U[0] < 0) return false;
    return !(2.0 * U[0] * U[3] < fma(U[1], U[1], U[2] * U[2]));
  }
  DG_HD static bool physical(const EqP &, const double *U) {
#ifdef __CUDA_ARCH__
    if (physical_f32(U)) return true;
#endif
    return physical_fp64(U);
  }
  DG_HD static void flux(const EqP &q, const double *U, double *fx, double *fy) {
    double ir = rcp(U[0]);
    double u = U[1] * ir, v = U[2] * ir;
    // p is reused as an addend: round it explicitly (never fused into an FMA)
    double p = mul_rn(q.gamma - 1., fma(-0.5, fma(U[1], u, U[2] * v), U[3]));
    double H = U[3] + p;
    fx[0] = U[1];
    fx[1] = fma(U[1], u, p);
    fx[2] = U[2] * u;
    fx[3] = H * u;
    fy[0] = U[2];
    fy[1] = U[1] * v;
    fy[2] = fma(U[2], v, p);
    fy[3] = H * v;
  }
  // the physical flux folded with the element metric, g = F . (ys, -xs) and
  // h = F . (-yr, xr), the two integrands of the volume term (eval_volume,
  // conserv_kernels.cu:1066-1074), formed from the momentum components
  // along those directions without F_x and F_y: 26 FP64 operations where
  // the flux and the fold take 33
  static constexpr bool kFolded = true;
  DG_HD static void flux_folded(const EqP &q, const double *U, double xr, double yr, double xs,
                                double ys, double *g, double *h) {
    const double ir = rcp(U[0]);
    const double ma = fma(U[1], ys, -U[2] * xs), mb = fma(U[2], xr, -U[1] * yr);
    const double ua = ma * ir, ub = mb * ir;
    const double m2 = fma(U[1], U[1], U[2] * U[2]);
    // p is reused as an addend: round it explicitly (never fused into an FMA)
    const double p = mul_rn(q.gamma - 1., fma(-0.5 * m2, ir, U[3]));
    const double H = U[3] + p;
    g[0] = ma;
    g[1] = fma(U[1], ua, p * ys);
    g[2] = fma(U[2], ua, -p * xs);
    g[3] = H * ua;
    h[0] = mb;
    h[1] = fma(U[1], ub, -p * yr);
    h[2] = fma(U[2], ub, p * xr);
    h[3] = H * ub;
  }
  // local Lax-Friedrichs (euler.cu:170-237)
  static constexpr double kRawScale = 0.5;  // LLF: F = 0.5 [ ... ]
  DG_HD static void riemann_raw(const EqP &q, const double *UL, const double *UR, double nx,
                                double ny, double *F) {
    // every multiply-add is an explicit fma so the rounding does not depend
    // on how the compiler contracts the expression in a given kernel; the
    // normal momenta m . n are the mass fluxes themselves
    const double irl = rcp(UL[0]), irr = rcp(UR[0]);
    const double mnl = fma(UL[1], nx, UL[2] * ny), mnr = fma(UR[1], nx, UR[2] * ny);
    const double snl = mnl * irl, snr = mnr * irr;
    const double m2l = fma(UL[1], UL[1], UL[2] * UL[2]), m2r = fma(UR[1], UR[1], UR[2] * UR[2]);
    const double pl = mul_rn(q.gamma - 1., fma(-0.5 * m2l, irl, UL[3]));
    const double pr = mul_rn(q.gamma - 1., fma(-0.5 * m2r, irr, UR[3]));
    const double cl = sqrt_pos(q.gamma * pl * irl), cr = sqrt_pos(q.gamma * pr * irr);
    const double lam = fmax(fabs(snl) + cl, fabs(snr) + cr);
    const double P = pl + pr;
    F[0] = fma(lam, UL[0] - UR[0], mnl + mnr);
    F[1] = fma(lam, UL[1] - UR[1], fma(UL[1], snl, fma(UR[1], snr, P * nx)));
    F[2] = fma(lam, UL[2] - UR[2], fma(UL[2], snl, fma(UR[2], snr, P * ny)));
    F[3] = fma(lam, UL[3] - UR[3], fma(UL[3] + pl, snl, (UR[3] + pr) * snr));
  }
  DG_HD static double mean_speed(const EqP &q, const double *U) {  // euler.cu:248-277
    // 1/rho and the square roots within 1 ulp of IEEE division and sqrt
    // (rcp, sqrt_pos): the wave speed is the CFL step's to 1e-15
    const double ir = rcp(U[0]);
    const double m2 = fma(U[1], U[1], U[2] * U[2]);
    const double p = (q.gamma - 1.) * fma(-0.5 * m2, ir, U[3]);
    const double c = sqrt_pos(q.gamma * p * ir);
    const double s = sqrt_pos(m2) * ir;
    return s > 0 ? s + c : -s + c;
  }
  DG_HD static void reflect(const EqP &q, const double *UL, double *UR, double x, double y,
                            double nx, double ny) {
    if (q.problem == PB_EULER_DOUBLEMACH && x < kDmX0) {  // doublemach.cu:75-93
      dm_shock(q, UR);
    } else if (q.problem == PB_EULER_SUPERSONIC || q.problem == PB_EULER_CYLINDER) {
      // curved wall around the origin (supersonic.cu:65-87, cylinder.cu:55-80)
      double d = sqrt(fma(x, x, y * y)), Nx = x / d, Ny = y / d;
      if (Nx * nx + Ny * ny < 0) {
        Nx = -Nx;
        Ny = -Ny;
      }
      UR[0] = UL[0];
      UR[3] = UL[3];
      const double tg = fma(UL[1], Ny, -UL[2] * Nx);
      UR[1] = tg * Ny;
      UR[2] = -tg * Nx;
    } else {  // slip wall: mirror the momentum
      double dot = fma(UL[1], nx, UL[2] * ny);
      UR[0] = UL[0];
      UR[1] = fma(-2 * dot, nx, UL[1]);
      UR[2] = fma(-2 * dot, ny, UL[2]);
      UR[3] = UL[3];
    }
  }
  static constexpr bool outflow_uses_exact = true;
};

struct ShallowWater {  // shallowwater/shallowwater.cu (g is a parameter here)
  static constexpr int N = 3;
  static constexpr bool kBathymetry = true;  // optional bed b(x, y): source -g h grad b
  static constexpr bool kField = false;
  static constexpr bool kFolded = false;
  DG_HD static bool physical(const EqP &, const double *U) { return U[0] >= 0.; }
  DG_HD static void flux(const EqP &q, const double *U, double *fx, double *fy) {
    double ih = rcp(U[0]);
    double u = U[1] * ih, v = U[2] * ih, hp = 0.5 * q.g * U[0] * U[0];
    fx[0] = U[1];
    fx[1] = fma(U[1], u, hp);
    fx[2] = U[2] * u;
    fy[0] = U[2];
    fy[1] = U[1] * v;
    fy[2] = fma(U[2], v, hp);
  }
  static constexpr double kRawScale = 0.5;  // LLF: F = 0.5 [ ... ]
  DG_HD static void riemann_raw(const EqP &q, const double *UL, const double *UR, double nx,
                                double ny, double *F) {  // shallowwater.cu:118-185
    // the normal momenta m . n are the mass fluxes themselves
    const double ihl = rcp(UL[0]), ihr = rcp(UR[0]);
    const double mnl = fma(nx, UL[1], ny * UL[2]), mnr = fma(nx, UR[1], ny * UR[2]);
    const double snl = mnl * ihl, snr = mnr * ihr;
    const double cl = sqrt_pos(UL[0] * q.g), cr = sqrt_pos(UR[0] * q.g);
    const double lam = fmax(fabs(snl) + cl, fabs(snr) + cr);
    const double P = 0.5 * q.g * fma(UL[0], UL[0], UR[0] * UR[0]);
    F[0] = fma(lam, UL[0] - UR[0], mnl + mnr);
    F[1] = fma(lam, UL[1] - UR[1], fma(UL[1], snl, fma(UR[1], snr, P * nx)));
    F[2] = fma(lam, UL[2] - UR[2], fma(UL[2], snl, fma(UR[2], snr, P * ny)));
  }
  DG_HD static double mean_speed(const EqP &q, const double *U) {  // shallowwater.cu:196-224
    // as Euler's: rcp and sqrt_pos within 1 ulp of IEEE division and sqrt
    const double c = sqrt_pos(U[0] * q.g);
    const double s = sqrt_pos(fma(U[1], U[1], U[2] * U[2])) * rcp(U[0]);
    return s > 0 ? s + c : -s + c;
  }
  DG_HD static void reflect(const EqP &, const double *UL, double *UR, double, double, double nx,
                            double ny) {  // shallowwater/test/test.cu:63-77
    double dot = fma(UL[1], nx, UL[2] * ny);
    UR[0] = UL[0];
    UR[1] = fma(-2 * dot, nx, UL[1]);
    UR[2] = fma(-2 * dot, ny, UL[2]);
  }
  static constexpr bool outflow_uses_exact = false;
};

struct Maxwell {  // maxwells/maxwells.cu, U = (Hx, Hy, Ez)
  static constexpr int N = 3;
  static constexpr bool kBathymetry = false;
  static constexpr bool kField = false;
  static constexpr bool kFolded = false;
  DG_HD static bool physical(const EqP &, const double *) { return true; }
  DG_HD static void flux(const EqP &q, const double *U, double *fx, double *fy) {
    double imu = 1. / q.mu, ieps = 1. / q.eps;
    fx[0] = 0.;
    fx[1] = imu * U[2];
    fx[2] = ieps * U[1];
    fy[0] = -imu * U[2];
    fy[1] = 0.;
    fy[2] = -ieps * U[0];
  }
  static constexpr double kRawScale = 0.5;  // LLF: F = 0.5 [ ... ]
  DG_HD static void riemann_raw(const EqP &q, const double *UL, const double *UR, double nx,
                                double ny, double *F) {  // maxwells.cu:93-163, LLF with lambda = 1/sqrt(eps mu)
    double imu = 1. / q.mu, ieps = 1. / q.eps, lam = fabs(1. / sqrt(q.eps * q.mu));
    double ez = UL[2] + UR[2], hx = UL[0] + UR[0], hy = UL[1] + UR[1];
    F[0] = fma(lam, UL[0] - UR[0], -imu * ez * ny);
    F[1] = fma(lam, UL[1] - UR[1], imu * ez * nx);
    F[2] = fma(lam, UL[2] - UR[2], ieps * fma(hy, nx, -hx * ny));
  }
  DG_HD static double mean_speed(const EqP &q, const double *) { return fabs(1. / sqrt(q.eps * q.mu)); }
  DG_HD static void reflect(const EqP &, const double *UL, double *UR, double, double, double nx,
                            double ny) {  // maxwells/cmirror/cmirror.cu:63-77
    // E_z kept; H: the normal component kept, the tangential one reversed
    double dot = fma(UL[0], nx, UL[1] * ny);
    UR[2] = UL[2];
    UR[0] = fma(2 * dot, nx, -UL[0]);
    UR[1] = fma(2 * dot, ny, -UL[1]);
  }
  static constexpr bool outflow_uses_exact = false;
};

// the volume integrands g = F . (ys, -xs), h = F . (-yr, xr) of a state U
// (eval_volume, conserv_kernels.cu:1066-1074): an equation's own folded
// flux where it has one, else the flux and the fold
template <class Eq>
DG_HD void folded_flux(const EqP &q, const double *U, double xr, double yr, double xs, double ys,
                       double *g, double *h) {
  if constexpr (Eq::kFolded) {
    Eq::flux_folded(q, U, xr, yr, xs, ys, g, h);
  } else {
    double fx[Eq::N], fy[Eq::N];
    Eq::flux(q, U, fx, fy);
    for (int n = 0; n < Eq::N; n++) {
      g[n] = fma(fx[n], ys, -fy[n] * xs);
      h[n] = fma(fy[n], xr, -fx[n] * yr);
    }
  }
}

// ghost state of a boundary side (eval_boundary, conserv_kernels.cu:820-843)
template <class Eq>
DG_HD void ghost_state(const EqP &q, int code, const double *UL, double *UR, double x, double y,
                       double t, double nx, double ny) {
  double G[4] = {0, 0, 0, 0};
  if (code == -4) {  // transmissive (new)
    for (int n = 0; n < Eq::N; n++) G[n] = UL[n];
  } else if (code == -3) {  // inflow
    inflow_state(q, G, x, y, t);
  } else if (code == -2) {  // outflow
    if (Eq::outflow_uses_exact) exact_state(q, G, x, y, t);
  } else {  // reflect
    Eq::reflect(q, UL, G, x, y, nx, ny);
  }
  for (int n = 0; n < Eq::N; n++) UR[n] = G[n];
}

}  // namespace dg
