// dg_kernels.cuh -- the RK-DG right-hand side on sm_103a, FP64.
//
// One RK stage is three kernels plus an optional limiter pass:
//
//   k_trace    one thread per element: the solution's values at the
//              3 x (p+1) Gauss points of its faces ("traces"), written
//              [elem][face][j][var]; an element with a non-physical trace is
//              flattened to its mean first (check_physical, euler.cu:92-116).
//   k_face     one thread per side: the numerical flux F*(u-, u+; n) at each
//              edge point, the right trace read at the mirrored point p-j
//              (eval_left_right, conserv_kernels.cu:850-892) or built from
//              the boundary code (eval_boundary, :820-843), scaled by
//              len/2 * w_j and stored [side][j][var].  Each flux is computed
//              once, where the reference's element-side formulation needs it
//              once per side too (eval_surface, :899-985).
//   k_element  one thread per element: the volume integral (eval_volume,
//              :992-1083) -- solution and flux at the area points projected
//              on the weighted basis gradients through the element metric --
//              plus a deterministic gather of the three faces' fluxes
//              projected on the edge basis (eval_rhs, time_integrator.cu:
//              26-101), times 1/J, and the RK stage update as epilogue:
//              out = ca*u^n + cb*u_s + cc*dt*du/dt.
//   k_limit    Barth-Jespersen limiter in place (limit_c, :640-720).
//
// SSP-RK3 steps skip k_trace after the first stage: k_element<TR=true>
// writes the traces of its output as it stores it, and k_limit_tr limits
// from those traces and rebuilds the ones it changes, so T always holds what
// k_trace would have computed from the next stage's input.
//
// FP64 is the binding resource on GB300 (the FP64 pipe runs at 1/62 of the
// FP32 rate), so the design minimises FP64 instructions: every basis value
// is a constant-bank operand (tables are __grid_constant__ parameters and
// all loops are unrolled), each Riemann flux is evaluated once per side,
// metric terms are folded into the flux before the projection (2 FMAs per
// mode and point instead of 6), and the limiter needs two divisions per
// variable instead of one per edge point.
#pragma once
#include "dg_device.cuh"
#include "dg_launch.h"

namespace dg {

constexpr int kBlock = 128;

template <int P>
__device__ __forceinline__ size_t trace_stride() {
  return 3 * (P + 1);
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_trace(const __grid_constant__ Tab<P> tab,
                                                  const __grid_constant__ EqP q, double *u,
                                                  double *__restrict__ T, int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[N][NP];
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) c[n][i] = u[(size_t)(n * NP + i) * Kp + e];
  double *Te = T + (size_t)e * (3 * N1 * N);
  bool bad = false;
#pragma unroll
  for (int f = 0; f < 3; f++)
#pragma unroll
    for (int j = 0; j < N1; j++) {
      double U[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        double a = c[n][0] * tab.E[f][j][0];
#pragma unroll
        for (int i = 1; i < NP; i++) a = fma(c[n][i], tab.E[f][j][i], a);
        U[n] = a;
      }
      bad |= !Eq::physical(q, U);
#pragma unroll
      for (int n = 0; n < N; n++) Te[(f * N1 + j) * N + n] = U[n];
    }
  if (bad) {  // flatten: higher modes to zero, traces to the mean
#pragma unroll
    for (int n = 0; n < N; n++) {
#pragma unroll
      for (int i = 1; i < NP; i++) u[(size_t)(n * NP + i) * Kp + e] = 0.0;
#pragma unroll
      for (int f = 0; f < 3; f++)
#pragma unroll
        for (int j = 0; j < N1; j++) Te[(f * N1 + j) * N + n] = c[n][0] * tab.E[f][j][0];
    }
  }
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_face(const __grid_constant__ Tab<P> tab,
                                                 const __grid_constant__ EqP q,
                                                 const double *__restrict__ T,
                                                 const int4 *__restrict__ side,
                                                 const double *__restrict__ sgeo,
                                                 const double *__restrict__ bxy,
                                                 double *__restrict__ Fh, const double *tptr,
                                                 const double *dtp, double tcoef, int S, int Sb) {
  constexpr int N = Eq::N, N1 = P + 1;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int4 sd = side[s];
  const double nx = sgeo[s], ny = sgeo[S + s], hl = sgeo[2 * (size_t)S + s];
  const double *TL = T + ((size_t)sd.x * 3 + sd.z) * (N1 * N);
  double *F = Fh + (size_t)s * (N1 * N);
  if (sd.y >= 0) {
    const double *TR = T + ((size_t)sd.y * 3 + sd.w) * (N1 * N);
#pragma unroll
    for (int j = 0; j < N1; j++) {
      double UL[N], UR[N], Fn[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        UL[n] = TL[j * N + n];
        UR[n] = TR[(N1 - 1 - j) * N + n];
      }
      Eq::riemann(q, UL, UR, nx, ny, Fn);
      const double sc = hl * tab.w1[j];
#pragma unroll
      for (int n = 0; n < N; n++) F[j * N + n] = Fn[n] * sc;
    }
  } else {
    const double t = *tptr + tcoef * *dtp;
    const double xa = bxy[s], ya = bxy[Sb + s], xb = bxy[2 * Sb + s], yb = bxy[3 * Sb + s];
#pragma unroll
    for (int j = 0; j < N1; j++) {
      double UL[N], UR[N], Fn[N];
#pragma unroll
      for (int n = 0; n < N; n++) UL[n] = TL[j * N + n];
      const double r = 0.5 + 0.5 * tab.t1[j];
      ghost_state<Eq>(q, sd.y, UL, UR, xa + r * (xb - xa), ya + r * (yb - ya), t, nx, ny);
      Eq::riemann(q, UL, UR, nx, ny, Fn);
      const double sc = hl * tab.w1[j];
#pragma unroll
      for (int n = 0; n < N; n++) F[j * N + n] = Fn[n] * sc;
    }
  }
}

// ---------------------------------------------------------------------------
// volume integral accumulated into acc; returns false if a point was
// non-physical (acc is then incomplete and must be recomputed)
template <class Eq, int P>
__device__ __forceinline__ bool volume(const Tab<P> &tab, const EqP &q,
                                       const double (&c)[Eq::N][Tab<P>::NP],
                                       double (&acc)[Eq::N][Tab<P>::NP], double xr, double yr,
                                       double xs, double ys) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, NQ = Tab<P>::NQ;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double U[N], fx[N], fy[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
      double a = c[n][0] * tab.B[k][0];
#pragma unroll
      for (int i = 1; i < NP; i++) a = fma(c[n][i], tab.B[k][i], a);
      U[n] = a;
    }
    ok &= Eq::physical(q, U);
    Eq::flux(q, U, fx, fy);
    // [fx fy] [y_s -y_r; -x_s x_r] folded once per point (eval_volume :1066-1074)
#pragma unroll
    for (int n = 0; n < N; n++) {
      const double gr = fma(fx[n], ys, -fy[n] * xs);
      const double gs = fma(fy[n], xr, -fx[n] * yr);
#pragma unroll
      for (int i = 1; i < NP; i++)  // grad phi_0 = 0
        acc[n][i] = fma(tab.GR[k][i], gr, fma(tab.GS[k][i], gs, acc[n][i]));
    }
  }
  return ok;
}

// TR: also write the edge traces of `out` into T (what k_trace would compute
// from it at the start of the next stage, bit for bit) and, when `check` is
// set, flatten an element whose new traces are non-physical
template <class Eq, int P, bool TR>
__global__ void __launch_bounds__(kBlock) k_element(
    const __grid_constant__ Tab<P> tab, const __grid_constant__ EqP q, double *us,
    const double *un, double *out, const double *__restrict__ Fh, const int *__restrict__ esd,
    const double *__restrict__ geo, const double *dtp, double ca, double cb, double cc, int K,
    int Kp, double *__restrict__ T, int check) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[N][NP], acc[N][NP];
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) {
      c[n][i] = us[(size_t)(n * NP + i) * Kp + e];
      acc[n][i] = 0.0;
    }
  const double xr = geo[e], yr = geo[(size_t)Kp + e], xs = geo[2 * (size_t)Kp + e],
               ys = geo[3 * (size_t)Kp + e], iJ = geo[4 * (size_t)Kp + e];
  if (!volume<Eq, P>(tab, q, c, acc, xr, yr, xs, ys)) {
    // non-physical volume value: the element's mean replaces it everywhere
#pragma unroll
    for (int n = 0; n < N; n++)
#pragma unroll
      for (int i = 0; i < NP; i++) {
        acc[n][i] = 0.0;
        if (i > 0) c[n][i] = 0.0;
      }
    volume<Eq, P>(tab, q, c, acc, xr, yr, xs, ys);
    if (us != out)
#pragma unroll
      for (int n = 0; n < N; n++)
#pragma unroll
        for (int i = 1; i < NP; i++) us[(size_t)(n * NP + i) * Kp + e] = 0.0;
  }
  // surface: -F on a left face, +F (mirrored points) on a right face
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const int sd = esd[(size_t)f * Kp + e];
    const bool right = sd & 1;
    const double *F = Fh + (size_t)(sd >> 1) * (N1 * N);
    const double sg = right ? 1.0 : -1.0;
#pragma unroll
    for (int j = 0; j < N1; j++) {
      const int jj = right ? (N1 - 1 - j) : j;
#pragma unroll
      for (int n = 0; n < N; n++) {
        const double fv = sg * F[jj * N + n];
#pragma unroll
        for (int i = 0; i < NP; i++) acc[n][i] = fma(fv, tab.E[f][j][i], acc[n][i]);
      }
    }
  }
  const double dt = *dtp;
  const double s = cc * dt * iJ;
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) {
      const size_t o = (size_t)(n * NP + i) * Kp + e;
      double v = fma(s, acc[n][i], cb * c[n][i]);
      if (ca != 0.0) v = fma(ca, un[o], v);
      out[o] = v;
      if (TR) acc[n][i] = v;
    }
  if (TR) {
    double *Te = T + (size_t)e * (3 * N1 * N);
    bool bad = false;
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < N1; j++) {
        double U[N];
#pragma unroll
        for (int n = 0; n < N; n++) {
          double a = acc[n][0] * tab.E[f][j][0];
#pragma unroll
          for (int i = 1; i < NP; i++) a = fma(acc[n][i], tab.E[f][j][i], a);
          U[n] = a;
        }
        bad |= !Eq::physical(q, U);
#pragma unroll
        for (int n = 0; n < N; n++) Te[(f * N1 + j) * N + n] = U[n];
      }
    if (check && bad) {
#pragma unroll
      for (int n = 0; n < N; n++) {
#pragma unroll
        for (int i = 1; i < NP; i++) out[(size_t)(n * NP + i) * Kp + e] = 0.0;
#pragma unroll
        for (int f = 0; f < 3; f++)
#pragma unroll
          for (int j = 0; j < N1; j++) Te[(f * N1 + j) * N + n] = acc[n][0] * tab.E[f][j][0];
      }
    }
  }
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_limit(const __grid_constant__ Tab<P> tab,
                                                  double *u, const int *__restrict__ nbr,
                                                  int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  const int nb0 = nbr[e], nb1 = nbr[(size_t)Kp + e], nb2 = nbr[2 * (size_t)Kp + e];
  const double phi0 = tab.B[0][0];
#pragma unroll
  for (int n = 0; n < N; n++) {
    const double *row = u + (size_t)(n * NP) * Kp;
    double c[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) c[i] = row[(size_t)i * Kp + e];
    const double Uc = c[0] * phi0;
    const double m0 = row[nb0] * phi0, m1 = row[nb1] * phi0, m2 = row[nb2] * phi0;
    const double Umin = fmin(Uc, fmin(m0, fmin(m1, m2)));
    const double Umax = fmax(Uc, fmax(m0, fmax(m1, m2)));
    // largest overshoot above / below the mean over the edge points; the
    // reference takes min_j over (Uc-Umin)/(U_j-Uc) resp. (Uc-Umax)/(U_j-Uc)
    // (conserv_kernels.cu:694-705), which is the same number: division
    // by the largest positive denominator gives the smallest quotient
    double up = 0.0, dn = 0.0;
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < N1; j++) {
        double a = c[0] * tab.E[f][j][0];
#pragma unroll
        for (int i = 1; i < NP; i++) a = fma(c[i], tab.E[f][j][i], a);
        const double d = a - Uc;
        up = fmax(up, d);
        dn = fmax(dn, -d);
      }
    double alpha = 1.0;
    if (up > 0.0) alpha = fmin(alpha, (Uc - Umin) / up);
    if (dn > 0.0) alpha = fmin(alpha, (Umax - Uc) / dn);
    if (alpha < 0.0) alpha = 0.0;
    if (alpha < 1.0) {
      double *w = u + (size_t)(n * NP) * Kp;
      w[(size_t)1 * Kp + e] = c[1] * alpha;
      w[(size_t)2 * Kp + e] = c[2] * alpha;
#pragma unroll
      for (int i = 3; i < NP; i++) w[(size_t)i * Kp + e] = 0.0;  // p > 1: drop higher modes
    }
  }
}

// ---------------------------------------------------------------------------
// The same limiter reading the edge traces k_element<TR> left in T instead of
// re-evaluating them; a limited variable's traces are rebuilt from its
// limited modes, then the positivity rule of k_trace is applied to the final
// traces.  T ends up holding exactly what k_trace would compute from the
// limited state.
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_limit_tr(const __grid_constant__ Tab<P> tab,
                                                     const __grid_constant__ EqP q, double *u,
                                                     double *__restrict__ T,
                                                     const int *__restrict__ nbr, int K,
                                                     int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  const int nb0 = nbr[e], nb1 = nbr[(size_t)Kp + e], nb2 = nbr[2 * (size_t)Kp + e];
  const double phi0 = tab.B[0][0];
  double *Te = T + (size_t)e * (3 * N1 * N);
  double c0[N];
  bool bad = false;
#pragma unroll
  for (int n = 0; n < N; n++) {
    double *row = u + (size_t)(n * NP) * Kp;
    c0[n] = row[e];
    const double Uc = c0[n] * phi0;
    const double m0 = row[nb0] * phi0, m1 = row[nb1] * phi0, m2 = row[nb2] * phi0;
    const double Umin = fmin(Uc, fmin(m0, fmin(m1, m2)));
    const double Umax = fmax(Uc, fmax(m0, fmax(m1, m2)));
    double up = 0.0, dn = 0.0;
#pragma unroll
    for (int k = 0; k < 3 * N1; k++) {
      const double d = Te[k * N + n] - Uc;
      up = fmax(up, d);
      dn = fmax(dn, -d);
    }
    double alpha = 1.0;
    if (up > 0.0) alpha = fmin(alpha, (Uc - Umin) / up);
    if (dn > 0.0) alpha = fmin(alpha, (Umax - Uc) / dn);
    if (alpha < 0.0) alpha = 0.0;
    if (alpha < 1.0) {
      const double c1 = row[(size_t)1 * Kp + e] * alpha, c2 = row[(size_t)2 * Kp + e] * alpha;
      row[(size_t)1 * Kp + e] = c1;
      row[(size_t)2 * Kp + e] = c2;
#pragma unroll
      for (int i = 3; i < NP; i++) row[(size_t)i * Kp + e] = 0.0;
#pragma unroll
      for (int f = 0; f < 3; f++)
#pragma unroll
        for (int j = 0; j < N1; j++) {
          double a = c0[n] * tab.E[f][j][0];
          a = fma(c1, tab.E[f][j][1], a);
          a = fma(c2, tab.E[f][j][2], a);
          Te[(f * N1 + j) * N + n] = a;
        }
    }
  }
#pragma unroll
  for (int k = 0; k < 3 * N1; k++) {
    double U[N];
#pragma unroll
    for (int n = 0; n < N; n++) U[n] = Te[k * N + n];
    bad |= !Eq::physical(q, U);
  }
  if (bad) {
#pragma unroll
    for (int n = 0; n < N; n++) {
#pragma unroll
      for (int i = 1; i < NP; i++) u[(size_t)(n * NP + i) * Kp + e] = 0.0;
#pragma unroll
      for (int f = 0; f < 3; f++)
#pragma unroll
        for (int j = 0; j < N1; j++) Te[(f * N1 + j) * N + n] = c0[n] * tab.E[f][j][0];
    }
  }
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_lambda(const __grid_constant__ Tab<P> tab,
                                                   const __grid_constant__ EqP q,
                                                   const double *__restrict__ u, DevScalars *ds,
                                                   int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double lam = 0.0;
  if (e < K) {
    double U[N];
#pragma unroll
    for (int n = 0; n < N; n++) U[n] = u[(size_t)(n * NP) * Kp + e] * tab.B[0][0];
    lam = Eq::mean_speed(q, U);
    if (!(lam == lam)) {
      atomicExch(&ds->status, 4);
      lam = 0.0;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lam = fmax(lam, __shfl_xor_sync(0xffffffffu, lam, o));
  __shared__ double sm[kBlock / 32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = lam;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = sm[0];
    for (int w = 1; w < kBlock / 32; w++) m = fmax(m, sm[w]);
    atomicMax(&ds->lam_bits, (unsigned long long)__double_as_longlong(m));
  }
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_init(const __grid_constant__ Tab<P> tab,
                                                 const __grid_constant__ EqP q, double *u,
                                                 const double *__restrict__ vtx, int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, NQ = Tab<P>::NQ;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double V[6];
#pragma unroll
  for (int k = 0; k < 6; k++) V[k] = vtx[(size_t)k * Kp + e];
  double acc[N][NP];
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) acc[n][i] = 0.0;
  // c_i = sum_q w_q U0(x_q) phi_i(q) (evalU0, euler.cu:31-55)
  for (int k = 0; k < NQ; k++) {
    const double r = tab.r[k], s = tab.s[k];
    const double x = V[2] * r + V[4] * s + V[0] * (1 - r - s);
    const double y = V[3] * r + V[5] * s + V[1] * (1 - r - s);
    double U0[4];
    exact_state(q, U0, x, y, 0.0);
#pragma unroll
    for (int i = 0; i < NP; i++)
#pragma unroll
      for (int n = 0; n < N; n++) acc[n][i] += tab.w[k] * U0[n] * tab.B[k][i];
  }
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) u[(size_t)(n * NP + i) * Kp + e] = acc[n][i];
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_l2err(const __grid_constant__ Tab<P> tab,
                                                  const __grid_constant__ EqP q,
                                                  const double *__restrict__ u,
                                                  const double *__restrict__ vtx,
                                                  const double *__restrict__ jac, double t,
                                                  double *partial, int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, NQ = Tab<P>::NQ;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double err[N];
#pragma unroll
  for (int n = 0; n < N; n++) err[n] = 0.0;
  if (e < K) {
    double V[6];
#pragma unroll
    for (int k = 0; k < 6; k++) V[k] = vtx[(size_t)k * Kp + e];
    const double J = jac[e];
    // sum_q w_q (u_exact - U)^2 J (eval_error_L2, conserv_kernels.cu:1432-1479)
    for (int k = 0; k < NQ; k++) {
      const double r = tab.r[k], s = tab.s[k];
      const double x = V[2] * r + V[4] * s + V[0] * (1 - r - s);
      const double y = V[3] * r + V[5] * s + V[1] * (1 - r - s);
      double ue[4];
      exact_state(q, ue, x, y, t);
#pragma unroll
      for (int n = 0; n < N; n++) {
        double U = 0.0;
#pragma unroll
        for (int i = 0; i < NP; i++) U += u[(size_t)(n * NP + i) * Kp + e] * tab.B[k][i];
        err[n] += tab.w[k] * (ue[n] - U) * (ue[n] - U) * J;
      }
    }
  }
  __shared__ double sm[kBlock][N];
#pragma unroll
  for (int n = 0; n < N; n++) sm[threadIdx.x][n] = err[n];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int n = 0; n < N; n++) {
      double a = 0.0;
      for (int k = 0; k < kBlock; k++) a += sm[k][n];
      partial[(size_t)blockIdx.x * N + n] = a;
    }
  }
}

// ---------------------------------------------------------------------------
// values of variable `var` at the three vertices (eval_u, conserv_kernels.cu:1284-1307)
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_vertex(const __grid_constant__ Tab<P> tab,
                                                   const double *__restrict__ u, int var,
                                                   double *__restrict__ out, int K, int Kp) {
  constexpr int NP = Tab<P>::NP;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[NP];
#pragma unroll
  for (int i = 0; i < NP; i++) c[i] = u[(size_t)(var * NP + i) * Kp + e];
#pragma unroll
  for (int v = 0; v < 3; v++) {
    double a = 0.0;
#pragma unroll
    for (int i = 0; i < NP; i++) a += c[i] * tab.V[v][i];
    out[(size_t)v * Kp + e] = a;
  }
}

// ---------------------------------------------------------------------------
// launchers: dispatch on p to the template instance
// ---------------------------------------------------------------------------
inline unsigned nblk(int n) { return (unsigned)((n + kBlock - 1) / kBlock); }

template <class Eq>
struct Launch {
  template <int P>
  static const Tab<P> &tab(const Ctx &c) {
    return *reinterpret_cast<const Tab<P> *>(c.tab);
  }

#define DG_DISPATCH_P(expr)         \
  switch (c.p) {                    \
    case 0: { constexpr int P = 0; expr; } break; \
    case 1: { constexpr int P = 1; expr; } break; \
    case 2: { constexpr int P = 2; expr; } break; \
    case 3: { constexpr int P = 3; expr; } break; \
    case 4: { constexpr int P = 4; expr; } break; \
    case 5: { constexpr int P = 5; expr; } break; \
  }

  static void trace(const Ctx &c, double *u) {
    if (!c.m.K) return;
    DG_DISPATCH_P((k_trace<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), *c.q, u, c.T,
                                                                     c.m.K, c.m.Kp)));
  }
  static void face(const Ctx &c, const double *t, double tcoef) {
    if (!c.m.S) return;
    DG_DISPATCH_P((k_face<Eq, P><<<nblk(c.m.S), kBlock, 0, c.st>>>(
        tab<P>(c), *c.q, c.T, c.m.side, c.m.sgeo, c.m.bxy, c.Fh, t, &c.ds->dt, tcoef, c.m.S,
        c.m.Sb)));
  }
  static void element(const Ctx &c, double *us, const double *un, double *out, double ca,
                      double cb, double cc, const double *dtp) {
    if (!c.m.K) return;
    DG_DISPATCH_P((k_element<Eq, P, false><<<nblk(c.m.K), kBlock, 0, c.st>>>(
        tab<P>(c), *c.q, us, un, out, c.Fh, c.m.esd, c.m.geo, dtp, ca, cb, cc, c.m.K,
        c.m.Kp, nullptr, 0)));
  }
  static void element_tr(const Ctx &c, double *us, const double *un, double *out, double ca,
                         double cb, double cc, const double *dtp, int check) {
    if (!c.m.K) return;
    DG_DISPATCH_P((k_element<Eq, P, true><<<nblk(c.m.K), kBlock, 0, c.st>>>(
        tab<P>(c), *c.q, us, un, out, c.Fh, c.m.esd, c.m.geo, dtp, ca, cb, cc, c.m.K,
        c.m.Kp, c.T, check)));
  }
  static void limit_tr(const Ctx &c, double *u) {
    if (!c.m.K || c.p < 1) return;
    DG_DISPATCH_P((k_limit_tr<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), *c.q, u, c.T,
                                                                        c.m.nbr, c.m.K,
                                                                        c.m.Kp)));
  }
  static void limit(const Ctx &c, double *u) {
    if (!c.m.K || c.p < 1) return;
    DG_DISPATCH_P((k_limit<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), u, c.m.nbr,
                                                                     c.m.K, c.m.Kp)));
  }
  static void lambda(const Ctx &c, const double *u) {
    DG_DISPATCH_P((k_lambda<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), *c.q, u, c.ds,
                                                                      c.m.K, c.m.Kp)));
  }
  static void init(const Ctx &c, double *u) {
    DG_DISPATCH_P((k_init<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), *c.q, u,
                                                                    c.m.vtx, c.m.K, c.m.Kp)));
  }
  static int l2err(const Ctx &c, const double *u, double t, double *partial) {
    DG_DISPATCH_P((k_l2err<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(
        tab<P>(c), *c.q, u, c.m.vtx, c.m.jac, t, partial, c.m.K, c.m.Kp)));
    return (int)nblk(c.m.K);
  }

  static void vertex(const Ctx &c, const double *u, int var, double *out) {
    DG_DISPATCH_P((k_vertex<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tab<P>(c), u, var, out,
                                                                      c.m.K, c.m.Kp)));
  }
#undef DG_DISPATCH_P

  static const Ops &ops() {
    static const Ops o = {trace, face, element, limit, lambda, init, l2err, element_tr,
                          limit_tr, vertex};
    return o;
  }
};

}  // namespace dg
