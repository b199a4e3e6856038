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
// writes the traces of its output as it stores it, so T always holds what
// k_trace would have computed from the next stage's input.  With the limiter
// on, the limiter runs on those traces: for Euler in the element kernel's own
// epilogue (k_element<TR, LIM>, or k_element_oz<LIM> on the tensor path),
// with the neighbours' new cell means found before the element stage by
// k_means from the per-side flux sums k_face<FS> leaves; for the other
// equations as the pass k_limit_tr.  Either way a limited element's traces
// are rebuilt from its limited modes.
//
// FP64 is the binding resource on GB300 (the FP64 pipe runs at 1/62 of the
// FP32 rate), so the design minimises FP64 instructions: every basis value
// is a constant-bank operand (tables are __grid_constant__ parameters and
// all loops are unrolled), each Riemann flux is evaluated once per side,
// metric terms are folded into the flux before the projection (2 FMAs per
// mode and point instead of 6), and the limiter needs two divisions per
// variable instead of one per edge point.
#pragma once
#include <algorithm>
#include "dg_device.cuh"
#include "dg_launch.h"

namespace dg {

constexpr int kBlock = 128;     // fixed block of the auxiliary kernels
constexpr int kMaxBlock = 256;  // largest autotuned block of the stage kernels

template <int P>
__device__ __forceinline__ size_t trace_stride() {
  return 3 * (P + 1);
}

// ---------------------------------------------------------------------------
template <class Eq, int P>
__device__ __forceinline__ void trace_body(const Tab<P> &tab, const EqP &q, double *u,
                                           double *__restrict__ T, int Kp, int e) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
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

template <class Eq, int P>
__global__ void __launch_bounds__(kMaxBlock) k_trace(const __grid_constant__ Tab<P> tab,
                                                     const __grid_constant__ EqP q, double *u,
                                                     double *__restrict__ T, int K, int Kp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < K) trace_body<Eq, P>(tab, q, u, T, Kp, e);
}

// ---------------------------------------------------------------------------
struct FaceArgs {
  const double *T;
  const int4 *side;
  const double *sgeo, *bxy;
  const double *vtx;  // element vertices (rows of Kp): edge-point positions of a velocity field
  double *Fh;
  double *Fs;         // per side the sum over its edge points of Fh, [side][var] (FS kernels)
  const double *tptr, *dtp;
  double tcoef;
  int S, Sb, Kp;
};

// N contiguous doubles at p (16-byte aligned when N is even): 128-bit loads
// and stores where N is even, scalar ones otherwise
template <int N>
__device__ __forceinline__ void load_vars(const double *p, double (&v)[N]) {
  if constexpr (N % 2 == 0) {
#pragma unroll
    for (int k = 0; k < N / 2; k++) {
      const double2 d = __ldg(reinterpret_cast<const double2 *>(p) + k);
      v[2 * k] = d.x;
      v[2 * k + 1] = d.y;
    }
  } else {
#pragma unroll
    for (int n = 0; n < N; n++) v[n] = p[n];
  }
}
template <int N>
__device__ __forceinline__ void store_vars(double *p, const double (&v)[N]) {
  if constexpr (N % 2 == 0) {
#pragma unroll
    for (int k = 0; k < N / 2; k++)
      reinterpret_cast<double2 *>(p)[k] = make_double2(v[2 * k], v[2 * k + 1]);
  } else {
#pragma unroll
    for (int n = 0; n < N; n++) p[n] = v[n];
  }
}

// FS: also store the per-side sums of the scaled fluxes in a.Fs
template <class Eq, int P, bool FS = false>
__device__ __forceinline__ void face_body(const Tab<P> &tab, const EqP &q, const FaceArgs &a,
                                          int s) {
  constexpr int N = Eq::N, N1 = P + 1;
  const int S = a.S, Sb = a.Sb;
  const int4 sd = a.side[s];
  const double nx = a.sgeo[s], ny = a.sgeo[S + s], hl = a.sgeo[2 * (size_t)S + s];
  const double *TL = a.T + ((size_t)sd.x * 3 + sd.z) * (N1 * N);
  double *F = a.Fh + (size_t)s * (N1 * N);
  double fs[N];
#pragma unroll
  for (int n = 0; n < N; n++) fs[n] = 0.0;
  if (sd.y >= 0) {
    const double *TR = a.T + ((size_t)sd.y * 3 + sd.w) * (N1 * N);
#pragma unroll
    for (int j = 0; j < N1; j++) {
      double UL[N], UR[N], Fn[N];
      load_vars<N>(TL + j * N, UL);
      load_vars<N>(TR + (N1 - 1 - j) * N, UR);
      if constexpr (Eq::kField) {
        if (q.field) {  // the velocity at the edge point, on the left face
          const int va = sd.z, vb = sd.z == 2 ? 0 : sd.z + 1;
          const size_t Kp = a.Kp;
          const double xa = a.vtx[2 * va * Kp + sd.x], ya = a.vtx[(2 * va + 1) * Kp + sd.x];
          const double xb = a.vtx[2 * vb * Kp + sd.x], yb = a.vtx[(2 * vb + 1) * Kp + sd.x];
          const double r = 0.5 + 0.5 * tab.t1[j];
          double vx, vy;
          Eq::velocity(q, fma(r, xb - xa, xa), fma(r, yb - ya, ya), vx, vy);
          Eq::riemann_at(vx, vy, UL, UR, nx, ny, Fn);
        } else {
          Eq::riemann_raw(q, UL, UR, nx, ny, Fn);
        }
      } else {
        Eq::riemann_raw(q, UL, UR, nx, ny, Fn);
      }
      const double sc = hl * tab.w1[j] * Eq::kRawScale;  // exact: a power of two
#pragma unroll
      for (int n = 0; n < N; n++) {
        Fn[n] *= sc;
        if (FS) fs[n] = j == 0 ? Fn[n] : fs[n] + Fn[n];
      }
      store_vars<N>(F + j * N, Fn);
    }
  } else {
    const double t = *a.tptr + a.tcoef * *a.dtp;
    const double *bxy = a.bxy;
    const double xa = bxy[s], ya = bxy[Sb + s], xb = bxy[2 * Sb + s], yb = bxy[3 * Sb + s];
#pragma unroll
    for (int j = 0; j < N1; j++) {
      double UL[N], UR[N], Fn[N];
      load_vars<N>(TL + j * N, UL);
      const double r = 0.5 + 0.5 * tab.t1[j];
      const double px = fma(r, xb - xa, xa), py = fma(r, yb - ya, ya);
      ghost_state<Eq>(q, sd.y, UL, UR, px, py, t, nx, ny);
      if constexpr (Eq::kField) {
        if (q.field) {
          double vx, vy;
          Eq::velocity(q, px, py, vx, vy);
          Eq::riemann_at(vx, vy, UL, UR, nx, ny, Fn);
        } else {
          Eq::riemann_raw(q, UL, UR, nx, ny, Fn);
        }
      } else {
        Eq::riemann_raw(q, UL, UR, nx, ny, Fn);
      }
      const double sc = hl * tab.w1[j] * Eq::kRawScale;  // exact: a power of two
#pragma unroll
      for (int n = 0; n < N; n++) {
        Fn[n] *= sc;
        if (FS) fs[n] = j == 0 ? Fn[n] : fs[n] + Fn[n];
      }
      store_vars<N>(F + j * N, Fn);
    }
  }
  if (FS) store_vars<N>(a.Fs + (size_t)s * N, fs);
}

template <class Eq, int P, bool FS = false>
__global__ void __launch_bounds__(kMaxBlock) k_face(const __grid_constant__ Tab<P> tab,
                                                    const __grid_constant__ EqP q,
                                                    const __grid_constant__ FaceArgs a) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < a.S) face_body<Eq, P, FS>(tab, q, a, s);
}

// ---------------------------------------------------------------------------
// volume integral accumulated into acc; returns false if a point was
// non-physical (acc is then incomplete and must be recomputed)
template <class Eq, int P>
__device__ __forceinline__ bool volume(const Tab<P> &tab, const EqP &q,
                                       const double (&c)[Eq::N][Tab<P>::NP],
                                       double (&acc)[Eq::N][Tab<P>::NP], double xr, double yr,
                                       double xs, double ys, const double *bz, double x1 = 0.0,
                                       double y1 = 0.0) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, NQ = Tab<P>::NQ;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double U[N], gr[N], gs[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
      double a = c[n][0] * tab.B[k][0];
#pragma unroll
      for (int i = 1; i < NP; i++) a = fma(c[n][i], tab.B[k][i], a);
      U[n] = a;
    }
    ok &= Eq::physical(q, U);
    // [fx fy] [y_s -y_r; -x_s x_r] once per point (eval_volume :1066-1074)
    if constexpr (Eq::kField) {
      // velocity at the point x = x1 + xr r + xs s (get_coordinates_2d, :231-235)
      double vx = q.ax, vy = q.ay, fx[N], fy[N];
      if (q.field)
        Eq::velocity(q, fma(xr, tab.r[k], fma(xs, tab.s[k], x1)),
                     fma(yr, tab.r[k], fma(ys, tab.s[k], y1)), vx, vy);
      Eq::flux_at(vx, vy, U, fx, fy);
#pragma unroll
      for (int n = 0; n < N; n++) {
        gr[n] = fma(fx[n], ys, -fy[n] * xs);
        gs[n] = fma(fy[n], xr, -fx[n] * yr);
      }
    } else {
      folded_flux<Eq>(q, U, xr, yr, xs, ys, gr, gs);
    }
#pragma unroll
    for (int n = 0; n < N; n++) {
#pragma unroll
      for (int i = 1; i < NP; i++)  // grad phi_0 = 0
        acc[n][i] = fma(tab.GR[k][i], gr[n], fma(tab.GS[k][i], gs[n], acc[n][i]));
    }
    if (Eq::kBathymetry && bz) {
      // bed slope source S = (0, -g h b_x, -g h b_y) (the reference's
      // source_term hook, eval_volume :1063-1079): w_q J S projected on
      // phi_i, with w_q J grad b from the weighted gradient tables
      double br = 0.0, bs = 0.0;
#pragma unroll
      for (int i = 1; i < NP; i++) {
        br = fma(bz[i], tab.GR[k][i], br);
        bs = fma(bz[i], tab.GS[k][i], bs);
      }
      const double gh = -q.g * U[0];
      const double sx = gh * fma(ys, br, -yr * bs), sy = gh * fma(xr, bs, -xs * br);
#pragma unroll
      for (int i = 0; i < NP; i++) {
        acc[1][i] = fma(sx, tab.B[k][i], acc[1][i]);
        acc[2][i] = fma(sy, tab.B[k][i], acc[2][i]);
      }
    }
  }
  return ok;
}

template <class Eq, int P>
__device__ __forceinline__ void limit_tr_body(const Tab<P> &tab, const EqP &q, double *u,
                                              double *__restrict__ T,
                                              const int *__restrict__ nbr, int Kp, int e,
                                              const double *mean, size_t mstride);

// arguments of one element-kernel launch on one problem
struct ElemArgs {
  double *us;               // stage input (flattened in place if needed)
  const double *un;         // u^n for the RK combination (ca != 0)
  double *out;              // stage output; may alias us or un
  const double *Fh;         // side fluxes
  const int *esd;           // sides of each element
  const double *geo;        // metric
  const double *dtp;        // time step
  const double *bathy;      // bed modes [mode][Kp] (shallow water) or null
  const double *vtx;        // element vertices (rows of Kp): positions for a velocity field
  double *T;                // traces of out (TR)
  const double *M;          // fused limiter: the means of out (k_means), rows of Kp
  const int *nbr;           // fused limiter: neighbours across faces 0..2, rows of Kp
  double ca, cb, cc;
  int K, Kp, check;
};

// TR: also write the edge traces of `out` into T (what k_trace would compute
// from it at the start of the next stage, bit for bit) and, when `check` is
// set, flatten an element whose new traces are non-physical
// LIM (with TR): the limiter in the epilogue -- mode 0 of the output is the
// stored mean a.M (k_means), and limit_tr_body runs on the new modes and
// traces with the neighbours' means from a.M
template <class Eq, int P, bool TR, bool LIM = false>
__device__ __forceinline__ void element_body(const Tab<P> &tab, const EqP &q, const ElemArgs &a,
                                             int e) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int Kp = a.Kp;
  double *us = a.us, *out = a.out;
  double c[N][NP], acc[N][NP];
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) {
      c[n][i] = us[(size_t)(n * NP + i) * Kp + e];
      acc[n][i] = 0.0;
    }
  const double *geo = a.geo;
  const double xr = geo[e], yr = geo[(size_t)Kp + e], xs = geo[2 * (size_t)Kp + e],
               ys = geo[3 * (size_t)Kp + e], iJ = geo[4 * (size_t)Kp + e];
  double bz[Eq::kBathymetry ? NP : 1];
  const bool has_b = Eq::kBathymetry && a.bathy;
  if (Eq::kBathymetry) {
#pragma unroll
    for (int i = 0; i < (Eq::kBathymetry ? NP : 1); i++)
      bz[i] = has_b ? a.bathy[(size_t)i * Kp + e] : 0.0;
  }
  const double *bzp = has_b ? bz : nullptr;
  double x1 = 0.0, y1 = 0.0;
  if constexpr (Eq::kField) {
    if (q.field) {
      x1 = a.vtx[e];
      y1 = a.vtx[(size_t)Kp + e];
    }
  }
  if (!volume<Eq, P>(tab, q, c, acc, xr, yr, xs, ys, bzp, x1, y1)) {
    // non-physical volume value: the element's mean replaces it everywhere
#pragma unroll
    for (int n = 0; n < N; n++)
#pragma unroll
      for (int i = 0; i < NP; i++) {
        acc[n][i] = 0.0;
        if (i > 0) c[n][i] = 0.0;
      }
    volume<Eq, P>(tab, q, c, acc, xr, yr, xs, ys, bzp, x1, y1);
    if (us != out)
#pragma unroll
      for (int n = 0; n < N; n++)
#pragma unroll
        for (int i = 1; i < NP; i++) us[(size_t)(n * NP + i) * Kp + e] = 0.0;
  }
  // surface: -F on a left face, +F (mirrored points) on a right face
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const int sd = a.esd[(size_t)f * Kp + e];
    const bool right = sd & 1;
    const double *F = a.Fh + (size_t)(sd >> 1) * (N1 * N);
    // the sign as a bit flip (exactly -F), off the FP64 pipe
    const long long sg = right ? 0ll : (long long)0x8000000000000000ull;
#pragma unroll
    for (int j = 0; j < N1; j++) {
      const int jj = right ? (N1 - 1 - j) : j;
#pragma unroll
      for (int n = 0; n < N; n++) {
        const double fv = __longlong_as_double(sg ^ __double_as_longlong(F[jj * N + n]));
#pragma unroll
        for (int i = 0; i < NP; i++) acc[n][i] = fma(fv, tab.E[f][j][i], acc[n][i]);
      }
    }
  }
  const double dt = *a.dtp;
  const double s = a.cc * dt * iJ;
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) {
      const size_t o = (size_t)(n * NP + i) * Kp + e;
      double v = fma(s, acc[n][i], a.cb * c[n][i]);
      if (a.ca != 0.0) v = fma(a.ca, a.un[o], v);
      if (LIM && i == 0) v = a.M[(size_t)n * Kp + e];
      out[o] = v;
      if (TR) acc[n][i] = v;
    }
  if (TR) {
    double *Te = a.T + (size_t)e * (3 * N1 * N);
    bool bad = false;
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < N1; j++) {
        double U[N];
#pragma unroll
        for (int n = 0; n < N; n++) {
          double v = acc[n][0] * tab.E[f][j][0];
#pragma unroll
          for (int i = 1; i < NP; i++) v = fma(acc[n][i], tab.E[f][j][i], v);
          U[n] = v;
        }
        bad |= !Eq::physical(q, U);
#pragma unroll
        for (int n = 0; n < N; n++) Te[(f * N1 + j) * N + n] = U[n];
      }
    if (!LIM && a.check && bad) {
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
    if constexpr (LIM) limit_tr_body<Eq, P>(tab, q, out, a.T, a.nbr, Kp, e, a.M, (size_t)Kp);
  }
}

template <class Eq, int P, bool TR, bool LIM = false>
__global__ void __launch_bounds__(kMaxBlock) k_element(const __grid_constant__ Tab<P> tab,
                                                       const __grid_constant__ EqP q,
                                                       const __grid_constant__ ElemArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < a.K) element_body<Eq, P, TR, LIM>(tab, q, a, e);
}

// ---------------------------------------------------------------------------
// The cell means of a stage's output before its element stage runs, so that
// the element stage can apply the limiter (which needs the new means of the
// three neighbours) in its own epilogue.  Basis function 0 is constant and
// has no gradient, so the mean's right-hand side is the surface term alone:
// phi_0's edge value times the sum of the element's side fluxes (-F on a
// left face, +F on a right face), from the per-side sums Fs of the face
// kernel.  M = ca * un_0 + cb * us_0 + cc * dt / J * that, with the element
// epilogue's roundings; the element stage writes these M as the output's
// mode 0, so the limiter's neighbour bounds see exactly the stored means.
template <class Eq, int P>
__device__ __forceinline__ void means_body(const Tab<P> &tab, const ElemArgs &a,
                                           const double *__restrict__ Fs, double *__restrict__ M,
                                           int e) {
  constexpr int N = Eq::N, NP = Tab<P>::NP;
  const size_t Kp = a.Kp;
  double sum[N];
#pragma unroll
  for (int n = 0; n < N; n++) sum[n] = 0.0;
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const int sd = a.esd[f * Kp + e];
    double F[N];
    load_vars<N>(Fs + (size_t)(sd >> 1) * N, F);
    // the sign as a bit flip (exactly -F), off the FP64 pipe
    const long long sg = (sd & 1) ? 0ll : (long long)0x8000000000000000ull;
#pragma unroll
    for (int n = 0; n < N; n++) sum[n] += __longlong_as_double(sg ^ __double_as_longlong(F[n]));
  }
  const double sc = a.cc * *a.dtp * a.geo[4 * Kp + e];
  const double e0 = tab.E[0][0][0];
#pragma unroll
  for (int n = 0; n < N; n++) {
    const size_t o = (size_t)(n * NP) * Kp + e;
    double v = fma(sc, sum[n] * e0, a.cb == 1.0 ? a.us[o] : a.cb * a.us[o]);
    if (a.ca != 0.0) v = fma(a.ca, a.un[o], v);
    M[(size_t)n * Kp + e] = v;
  }
}

template <class Eq, int P>
__global__ void __launch_bounds__(kMaxBlock) k_means(const __grid_constant__ Tab<P> tab,
                                                     const __grid_constant__ ElemArgs a,
                                                     const double *__restrict__ Fs,
                                                     double *__restrict__ M) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < a.K) means_body<Eq, P>(tab, a, Fs, M, e);
}

// ---------------------------------------------------------------------------
// Order-preserving integer view of a double: for non-NaN x, y,
// x < y  <=>  order_key(x) < order_key(y) (with -0 just below +0).  Negative
// values get their 63 low bits flipped, so signed 64-bit comparison follows
// the real line.  The map is its own inverse.
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ (long long)((unsigned long long)(b >> 63) >> 1);
}
__device__ __forceinline__ double from_order_key(long long k) {
  return __longlong_as_double(k ^ (long long)((unsigned long long)(k >> 63) >> 1));
}

// bounds of the cell means over an element (c) and its three neighbours
// (a, b, d), each mean the product c phi0: with phi0 > 0 the rounded product
// is monotonic in c, so min_k (c_k phi0) = (min_k c_k) phi0 exactly, and the
// extremes are found on the integer pipe
__device__ __forceinline__ void mean_bounds(double c, double a, double b, double d, double phi0,
                                            double &lo, double &hi) {
  const long long kc = order_key(c), ka = order_key(a), kb = order_key(b), kd = order_key(d);
  lo = __dmul_rn(from_order_key(min(min(kc, ka), min(kb, kd))), phi0);
  hi = __dmul_rn(from_order_key(max(max(kc, ka), max(kb, kd))), phi0);
}

template <class Eq, int P>
__global__ void __launch_bounds__(kMaxBlock) k_limit(const __grid_constant__ Tab<P> tab,
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
    // products reused as addends are rounded explicitly (__dmul_rn is never
    // fused into an FMA), so every kernel instance rounds them the same way
    const double Uc = __dmul_rn(c[0], phi0);
    double Umin, Umax;
    mean_bounds(c[0], row[nb0], row[nb1], row[nb2], phi0, Umin, Umax);
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
    // a quotient >= 1 leaves alpha as it is, and a / b >= 1 exactly when
    // a >= b > 0 (IEEE division is monotonic): divide only when it limits
    double alpha = 1.0;
    const double lo = Uc - Umin, hi = Umax - Uc;
    // lo, hi >= +0; where a bound has collapsed (a uniform neighbourhood:
    // lo or hi is +0, tested on its bits) the quotient is +0 without dividing
    if (up > lo) alpha = fmin(alpha, __double_as_longlong(lo) ? lo / up : 0.0);
    if (dn > hi) alpha = fmin(alpha, __double_as_longlong(hi) ? hi / dn : 0.0);
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
// mean: the cell means (mode-0 coefficients) of variable n of element x are
// mean[n * mstride + x]: the state's own rows (mean = u, mstride = NP Kp), or
// the means k_means stored before the element stage wrote u (mean = M,
// mstride = Kp), when the neighbours' rows may not be written yet
template <class Eq, int P>
__device__ __forceinline__ void limit_tr_body(const Tab<P> &tab, const EqP &q, double *u,
                                              double *__restrict__ T,
                                              const int *__restrict__ nbr, int Kp, int e,
                                              const double *mean, size_t mstride) {
  constexpr int N = Eq::N, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int nb0 = nbr[e], nb1 = nbr[(size_t)Kp + e], nb2 = nbr[2 * (size_t)Kp + e];
  const double phi0 = tab.B[0][0];
  double *Te = T + (size_t)e * (3 * N1 * N);
  double c0[N];
  bool bad = false;
#pragma unroll
  for (int n = 0; n < N; n++) {
    double *row = u + (size_t)(n * NP) * Kp;
    const double *mn = mean + (size_t)n * mstride;
    c0[n] = mn[e];
    // products reused as addends are rounded explicitly (__dmul_rn is never
    // fused into an FMA), so every kernel instance rounds them the same way
    const double Uc = __dmul_rn(c0[n], phi0);
    double Umin, Umax;
    mean_bounds(c0[n], mn[nb0], mn[nb1], mn[nb2], phi0, Umin, Umax);
    // max_k (T_k - Uc) = max_k T_k - Uc exactly (rounding is monotonic), so
    // the extremes of the edge values are found first, on the integer pipe
    // (order_key), and each is subtracted once
    long long kmax = order_key(Te[n]), kmin = kmax;
#pragma unroll
    for (int k = 1; k < 3 * N1; k++) {
      const long long kk = order_key(Te[k * N + n]);
      kmax = max(kmax, kk);
      kmin = min(kmin, kk);
    }
    const double up = fmax(0.0, from_order_key(kmax) - Uc);
    const double dn = fmax(0.0, Uc - from_order_key(kmin));
    // a quotient >= 1 leaves alpha as it is, and a / b >= 1 exactly when
    // a >= b > 0 (IEEE division is monotonic): divide only when it limits
    double alpha = 1.0;
    const double lo = Uc - Umin, hi = Umax - Uc;
    // lo, hi >= +0; where a bound has collapsed (a uniform neighbourhood:
    // lo or hi is +0, tested on its bits) the quotient is +0 without dividing
    if (up > lo) alpha = fmin(alpha, __double_as_longlong(lo) ? lo / up : 0.0);
    if (dn > hi) alpha = fmin(alpha, __double_as_longlong(hi) ? hi / dn : 0.0);
    if (alpha < 0.0) alpha = 0.0;
    if (alpha < 1.0) {
      const double c1 = row[(size_t)1 * Kp + e] * alpha, c2 = row[(size_t)2 * Kp + e] * alpha;
      row[(size_t)1 * Kp + e] = c1;
      row[(size_t)2 * Kp + e] = c2;
#pragma unroll
      for (int i = 3; i < NP; i++) row[(size_t)i * Kp + e] = 0.0;
      // basis function 0 is constant: c0 phi_0 is one product for every point
      const double a0 = c0[n] * tab.E[0][0][0];
      if (alpha == 0.0 && a0 != 0.0) {
        // c1 = c2 = +-0 add nothing to a nonzero a0: the traces are a0 (the
        // common case: a uniform region, where the limiter removes
        // rounding-sized higher modes)
#pragma unroll
        for (int k = 0; k < 3 * N1; k++) Te[k * N + n] = a0;
      } else {
#pragma unroll
        for (int f = 0; f < 3; f++)
#pragma unroll
          for (int j = 0; j < N1; j++) {
            double a = a0;
            a = fma(c1, tab.E[f][j][1], a);
            a = fma(c2, tab.E[f][j][2], a);
            Te[(f * N1 + j) * N + n] = a;
          }
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
      const double a0 = c0[n] * tab.E[0][0][0];
#pragma unroll
      for (int f = 0; f < 3; f++)
#pragma unroll
        for (int j = 0; j < N1; j++) Te[(f * N1 + j) * N + n] = a0;
    }
  }
}

template <class Eq, int P>
__global__ void __launch_bounds__(kMaxBlock) k_limit_tr(const __grid_constant__ Tab<P> tab,
                                                        const __grid_constant__ EqP q,
                                                        double *u, double *__restrict__ T,
                                                        const int *__restrict__ nbr, int K,
                                                        int Kp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < K) limit_tr_body<Eq, P>(tab, q, u, T, nbr, Kp, e, u, (size_t)Tab<P>::NP * Kp);
}

// ---------------------------------------------------------------------------
// block max of the cell-mean wave speed of elements [e0, e0 + blockDim) into
// ds->lam_bits (the block's elements belong to one problem)
template <class Eq, int P>
__device__ __forceinline__ void lambda_body(const Tab<P> &tab, const EqP &q,
                                            const double *__restrict__ u, DevScalars *ds, int K,
                                            int Kp, int e) {
  constexpr int N = Eq::N, NP = Tab<P>::NP;
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

// the same maximum over a single problem, grid-stride: a few blocks per SM
// each take the max over many elements, so one atomic per block stays cheap
// (one per 128 elements serialises on the one word)
constexpr int kLambdaBlocks = 1024;
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_lambda(const __grid_constant__ Tab<P> tab,
                                                   const __grid_constant__ EqP q,
                                                   const double *__restrict__ u, DevScalars *ds,
                                                   int K, int Kp) {
  constexpr int N = Eq::N, NP = Tab<P>::NP;
  double lam = 0.0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K; e += gridDim.x * blockDim.x) {
    double U[N];
#pragma unroll
    for (int n = 0; n < N; n++) U[n] = u[(size_t)(n * NP) * Kp + e] * tab.B[0][0];
    double l = Eq::mean_speed(q, U);
    if (!(l == l)) {
      atomicExch(&ds->status, 4);
      l = 0.0;
    }
    lam = fmax(lam, l);
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
    init_state(q, U0, x, y);
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
// values of variable `var` at the three vertices: mode 0 the solution
// (eval_u, conserv_kernels.cu:1284-1307), 1 the exact solution at time t
// (plot_exact, :1310-1331), 2 solution minus exact (plot_error, :1334-1369;
// the reference reads basis_vertex with stride 6 there, past the [n_p][3]
// table, which here is read as the table it is)
template <class Eq, int P>
__global__ void __launch_bounds__(kBlock) k_vertex(const __grid_constant__ Tab<P> tab,
                                                   const __grid_constant__ EqP q,
                                                   const double *__restrict__ u, int var,
                                                   int mode, double t,
                                                   const double *__restrict__ vtx,
                                                   double *__restrict__ out, int K, int Kp) {
  constexpr int NP = Tab<P>::NP;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[NP];
#pragma unroll
  for (int i = 0; i < NP; i++) c[i] = mode == 1 ? 0.0 : u[(size_t)(var * NP + i) * Kp + e];
#pragma unroll
  for (int v = 0; v < 3; v++) {
    double a = 0.0;
#pragma unroll
    for (int i = 0; i < NP; i++) a += c[i] * tab.V[v][i];
    if (mode != 0) {
      double U[4];
      exact_state(q, U, vtx[(size_t)(2 * v) * Kp + e], vtx[(size_t)(2 * v + 1) * Kp + e], t);
      a = mode == 1 ? U[var] : a - U[var];
    }
    out[(size_t)v * Kp + e] = a;
  }
}

// ---------------------------------------------------------------------------
// batched kernels: one launch covers every problem of an ensemble.  Block b
// belongs to problem blk2prob[b] (each problem's elements, or sides, start a
// fresh block), and runs the same per-element body as the single-problem
// kernel, with that problem's arrays, parameters and order p in {1, 2, 3}.
// SSP-RK3 stage st: 0: W = U + dt L(U); 1: W = 3/4 U + 1/4 (W + dt L(W));
// 2: U = 1/3 U + 2/3 (W + dt L(W)).
// ---------------------------------------------------------------------------
struct BatchTabs {
  Tab<1> t1;
  Tab<2> t2;
  Tab<3> t3;
};

__device__ __forceinline__ ElemArgs batch_elem_args(const BatchProb &pr, int stage, int check) {
  ElemArgs a;
  a.us = stage == 0 ? pr.U : pr.W;
  a.un = pr.U;
  a.out = stage == 2 ? pr.U : pr.W;
  a.Fh = pr.Fh;
  a.esd = pr.esd;
  a.geo = pr.geo;
  a.dtp = &pr.ds->dt;
  a.bathy = pr.bathy;
  a.vtx = pr.vtx;
  a.T = pr.T;
  a.M = pr.M;
  a.nbr = pr.nbr;
  a.ca = stage == 0 ? 0.0 : stage == 1 ? 0.75 : 1.0 / 3.0;
  a.cb = stage == 0 ? 1.0 : stage == 1 ? 0.25 : 2.0 / 3.0;
  a.cc = stage == 0 ? 1.0 : stage == 1 ? 0.25 : 2.0 / 3.0;
  a.K = pr.K;
  a.Kp = pr.Kp;
  a.check = check;
  return a;
}

// the fused element stage of a batch, over the blocks [b_lo, b_lo +
// gridDim.x) of the problems of one order P and one mesh-size group (the
// block map lists the problems by group): one launch per group, each at its
// own register count and block size
template <class Eq, int P, bool LIM = false>
__global__ void __launch_bounds__(kMaxBlock)
    k_element_batch_p(const __grid_constant__ Tab<P> tab, const BatchProb *__restrict__ probs,
                      const int *__restrict__ blk2prob, const int *__restrict__ blk0, int b_lo,
                      int stage, int check) {
  const int b = b_lo + (int)blockIdx.x;
  const int pi = blk2prob[b];
  const BatchProb &pr = probs[pi];
  const int e = (b - blk0[pi]) * blockDim.x + threadIdx.x;
  if (e >= pr.K) return;
  const ElemArgs a = batch_elem_args(pr, stage, check);
  element_body<Eq, P, true, LIM>(tab, pr.q, a, e);
}

// the next stage output's cell means of every member (k_means), over the
// element blocks of the shared block size
template <class Eq>
__global__ void __launch_bounds__(kMaxBlock)
    k_means_batch(const __grid_constant__ BatchTabs tb, const BatchProb *__restrict__ probs,
                  const int *__restrict__ blk2prob, const int *__restrict__ blk0, int stage) {
  const int pi = blk2prob[blockIdx.x];
  const BatchProb &pr = probs[pi];
  const int e = (blockIdx.x - blk0[pi]) * blockDim.x + threadIdx.x;
  if (e >= pr.K) return;
  const ElemArgs a = batch_elem_args(pr, stage, 0);
  switch (pr.p) {
    case 1: means_body<Eq, 1>(tb.t1, a, pr.Fs, pr.M, e); break;
    case 2: means_body<Eq, 2>(tb.t2, a, pr.Fs, pr.M, e); break;
    case 3: means_body<Eq, 3>(tb.t3, a, pr.Fs, pr.M, e); break;
  }
}

template <class Eq, bool FS = false>
__global__ void __launch_bounds__(kMaxBlock)
    k_face_batch(const __grid_constant__ BatchTabs tb, const BatchProb *__restrict__ probs,
                 const int *__restrict__ blk2prob, const int *__restrict__ blk0, double tcoef) {
  const int pi = blk2prob[blockIdx.x];
  const BatchProb &pr = probs[pi];
  const int s = (blockIdx.x - blk0[pi]) * blockDim.x + threadIdx.x;
  if (s >= pr.S) return;
  FaceArgs a;
  a.T = pr.T;
  a.side = pr.side;
  a.sgeo = pr.sgeo;
  a.bxy = pr.bxy;
  a.vtx = pr.vtx;
  a.Fh = pr.Fh;
  a.Fs = pr.Fs;
  a.tptr = &pr.ds->t;
  a.dtp = &pr.ds->dt;
  a.tcoef = tcoef;
  a.S = pr.S;
  a.Sb = pr.Sb;
  a.Kp = pr.Kp;
  switch (pr.p) {
    case 1: face_body<Eq, 1, FS>(tb.t1, pr.q, a, s); break;
    case 2: face_body<Eq, 2, FS>(tb.t2, pr.q, a, s); break;
    case 3: face_body<Eq, 3, FS>(tb.t3, pr.q, a, s); break;
  }
}

template <class Eq>
__global__ void __launch_bounds__(kMaxBlock)
    k_limit_tr_batch(const __grid_constant__ BatchTabs tb, const BatchProb *__restrict__ probs,
                     const int *__restrict__ blk2prob, const int *__restrict__ blk0, int stage) {
  const int pi = blk2prob[blockIdx.x];
  const BatchProb &pr = probs[pi];
  const int e = (blockIdx.x - blk0[pi]) * blockDim.x + threadIdx.x;
  if (e >= pr.K) return;
  double *u = stage == 2 ? pr.U : pr.W;
  switch (pr.p) {
    case 1: limit_tr_body<Eq, 1>(tb.t1, pr.q, u, pr.T, pr.nbr, pr.Kp, e, u, (size_t)Tab<1>::NP * pr.Kp); break;
    case 2: limit_tr_body<Eq, 2>(tb.t2, pr.q, u, pr.T, pr.nbr, pr.Kp, e, u, (size_t)Tab<2>::NP * pr.Kp); break;
    case 3: limit_tr_body<Eq, 3>(tb.t3, pr.q, u, pr.T, pr.nbr, pr.Kp, e, u, (size_t)Tab<3>::NP * pr.Kp); break;
  }
}

template <class Eq>
__global__ void __launch_bounds__(kMaxBlock)
    k_trace_batch(const __grid_constant__ BatchTabs tb, const BatchProb *__restrict__ probs,
                  const int *__restrict__ blk2prob, const int *__restrict__ blk0) {
  const int pi = blk2prob[blockIdx.x];
  const BatchProb &pr = probs[pi];
  const int e = (blockIdx.x - blk0[pi]) * blockDim.x + threadIdx.x;
  if (e >= pr.K) return;
  switch (pr.p) {
    case 1: trace_body<Eq, 1>(tb.t1, pr.q, pr.U, pr.T, pr.Kp, e); break;
    case 2: trace_body<Eq, 2>(tb.t2, pr.q, pr.U, pr.T, pr.Kp, e); break;
    case 3: trace_body<Eq, 3>(tb.t3, pr.q, pr.U, pr.T, pr.Kp, e); break;
  }
}

template <class Eq>
__global__ void __launch_bounds__(kBlock)
    k_lambda_batch(const __grid_constant__ BatchTabs tb, const BatchProb *__restrict__ probs,
                   const int *__restrict__ blk2prob, const int *__restrict__ blk0) {
  const int pi = blk2prob[blockIdx.x];
  const BatchProb &pr = probs[pi];
  const int e = (blockIdx.x - blk0[pi]) * blockDim.x + threadIdx.x;
  switch (pr.p) {
    case 1: lambda_body<Eq, 1>(tb.t1, pr.q, pr.U, pr.ds, pr.K, pr.Kp, e); break;
    case 2: lambda_body<Eq, 2>(tb.t2, pr.q, pr.U, pr.ds, pr.K, pr.Kp, e); break;
    case 3: lambda_body<Eq, 3>(tb.t3, pr.q, pr.U, pr.ds, pr.K, pr.Kp, e); break;
  }
}

// ---------------------------------------------------------------------------
// launchers: dispatch on p to the template instance
// ---------------------------------------------------------------------------
inline unsigned nblk(int n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

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

  static ElemArgs eargs(const Ctx &c, double *us, const double *un, double *out, double ca,
                        double cb, double cc, const double *dtp, double *T, int check) {
    ElemArgs a;
    a.us = us;
    a.un = un;
    a.out = out;
    a.Fh = c.Fh;
    a.esd = c.m.esd;
    a.geo = c.m.geo;
    a.dtp = dtp;
    a.bathy = c.m.bathy;
    a.vtx = c.m.vtx;
    a.T = T;
    a.M = c.M;
    a.nbr = c.m.nbr;
    a.ca = ca;
    a.cb = cb;
    a.cc = cc;
    a.K = c.m.K;
    a.Kp = c.m.Kp;
    a.check = check;
    return a;
  }

  static void trace(const Ctx &c, double *u) {
    if (!c.m.K) return;
    DG_DISPATCH_P((k_trace<Eq, P><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(tab<P>(c), *c.q, u,
                                                                          c.T, c.m.K, c.m.Kp)));
  }
  template <bool FS>
  static void face_args(const Ctx &c, const double *t, double tcoef, double *Fs) {
    if (!c.m.S) return;
    FaceArgs a;
    a.T = c.T;
    a.side = c.m.side;
    a.sgeo = c.m.sgeo;
    a.bxy = c.m.bxy;
    a.vtx = c.m.vtx;
    a.Fh = c.Fh;
    a.Fs = Fs;
    a.tptr = t;
    a.dtp = &c.ds->dt;
    a.tcoef = tcoef;
    a.S = c.m.S;
    a.Sb = c.m.Sb;
    a.Kp = c.m.Kp;
    DG_DISPATCH_P((k_face<Eq, P, FS><<<nblk(c.m.S, c.blk), c.blk, 0, c.st>>>(tab<P>(c), *c.q,
                                                                             a)));
  }
  static void face(const Ctx &c, const double *t, double tcoef) {
    face_args<false>(c, t, tcoef, nullptr);
  }
  // face() that also leaves the per-side flux sums in c.Fs (instantiated only
  // where an equation's fused-limiter stage uses it)
  static void face_fs(const Ctx &c, const double *t, double tcoef) {
    face_args<true>(c, t, tcoef, c.Fs);
  }
  // the means of a stage's output into c.M (k_means)
  static void means(const Ctx &c, double *us, const double *un, double ca, double cb, double cc,
                    const double *dtp) {
    if (!c.m.K) return;
    const ElemArgs a = eargs(c, us, un, nullptr, ca, cb, cc, dtp, nullptr, 0);
    DG_DISPATCH_P((k_means<Eq, P><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(tab<P>(c), a, c.Fs,
                                                                          c.M)));
  }
  static void element(const Ctx &c, double *us, const double *un, double *out, double ca,
                      double cb, double cc, const double *dtp) {
    if (!c.m.K) return;
    const ElemArgs a = eargs(c, us, un, out, ca, cb, cc, dtp, nullptr, 0);
    DG_DISPATCH_P((k_element<Eq, P, false><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(tab<P>(c),
                                                                                   *c.q, a)));
  }
  // element_tr() with the limiter in the epilogue (c.M holds the output's
  // means from k_means)
  static void element_lim(const Ctx &c, double *us, const double *un, double *out, double ca,
                          double cb, double cc, const double *dtp) {
    if (!c.m.K) return;
    const ElemArgs a = eargs(c, us, un, out, ca, cb, cc, dtp, c.T, 0);
    DG_DISPATCH_P((k_element<Eq, P, true, true><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(
        tab<P>(c), *c.q, a)));
  }
  static void element_tr(const Ctx &c, double *us, const double *un, double *out, double ca,
                         double cb, double cc, const double *dtp, int check) {
    if (!c.m.K) return;
    const ElemArgs a = eargs(c, us, un, out, ca, cb, cc, dtp, c.T, check);
    DG_DISPATCH_P((k_element<Eq, P, true><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(tab<P>(c),
                                                                                  *c.q, a)));
  }
  static void limit_tr(const Ctx &c, double *u) {
    if (!c.m.K || c.p < 1) return;
    DG_DISPATCH_P((k_limit_tr<Eq, P><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(
        tab<P>(c), *c.q, u, c.T, c.m.nbr, c.m.K, c.m.Kp)));
  }
  static void limit(const Ctx &c, double *u) {
    if (!c.m.K || c.p < 1) return;
    DG_DISPATCH_P((k_limit<Eq, P><<<nblk(c.m.K, c.blk), c.blk, 0, c.st>>>(tab<P>(c), u, c.m.nbr,
                                                                          c.m.K, c.m.Kp)));
  }
  static void lambda(const Ctx &c, const double *u) {
    const unsigned g = std::min(nblk(c.m.K), (unsigned)kLambdaBlocks);
    DG_DISPATCH_P((k_lambda<Eq, P><<<g, kBlock, 0, c.st>>>(tab<P>(c), *c.q, u, c.ds, c.m.K,
                                                            c.m.Kp)));
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

  static void vertex(const Ctx &c, const double *u, int var, int mode, double t, double *out) {
    DG_DISPATCH_P((k_vertex<Eq, P><<<nblk(c.m.K), kBlock, 0, c.st>>>(
        tab<P>(c), *c.q, u, var, mode, t, c.m.vtx, out, c.m.K, c.m.Kp)));
  }
#undef DG_DISPATCH_P

  static const Ops &ops() {
    static const Ops o = {trace,  face,       element,  limit,  lambda,  init,    l2err,
                          element_tr, limit_tr, vertex, nullptr, nullptr, nullptr};
    return o;
  }

  // ---- batched launches ----
  static const BatchTabs &btabs(const BatchLaunch &b) {
    return *reinterpret_cast<const BatchTabs *>(b.tabs);
  }
  static void b_trace(const BatchLaunch &b) {
    k_trace_batch<Eq><<<b.nublk, b.blk, 0, b.st>>>(btabs(b), b.probs, b.ublk2prob, b.ublk0);
  }
  static void b_face(const BatchLaunch &b, double tcoef) {
    k_face_batch<Eq><<<b.nsblk, b.blk, 0, b.st>>>(btabs(b), b.probs, b.sblk2prob, b.sblk0,
                                                   tcoef);
  }
  template <bool LIM>
  static void b_element_v(const BatchLaunch &b, int stage) {
    const BatchTabs &tb = btabs(b);
    const int check = b.limiter ? 0 : 1;
    // one launch per (order, mesh-size) group, each with its own block size;
    // the groups after the first on their own streams, concurrent with it
    bool first = true;
    if (b.fork) cudaEventRecord(b.fork, b.st);
    for (int g = 0; g < BatchLaunch::kGroups; g++) {
      const int lo = b.eblk_g[g], n = b.eblk_g[g + 1] - lo, p = 1 + g / 2, blk = b.blk_g[g];
      if (n <= 0) continue;
      const bool side = b.fork && !first;
      const cudaStream_t st = side ? b.gst[g] : b.st;
      first = false;
      if (side) cudaStreamWaitEvent(st, b.fork, 0);
      if (p == 1)
        k_element_batch_p<Eq, 1, LIM><<<n, blk, 0, st>>>(tb.t1, b.probs, b.eblk2prob, b.eblk0,
                                                           lo, stage, check);
      else if (p == 2)
        k_element_batch_p<Eq, 2, LIM><<<n, blk, 0, st>>>(tb.t2, b.probs, b.eblk2prob, b.eblk0,
                                                           lo, stage, check);
      else
        k_element_batch_p<Eq, 3, LIM><<<n, blk, 0, st>>>(tb.t3, b.probs, b.eblk2prob, b.eblk0,
                                                           lo, stage, check);
      if (side) {
        cudaEventRecord(b.join[g], st);
        cudaStreamWaitEvent(b.st, b.join[g], 0);
      }
    }
  }
  static void b_element(const BatchLaunch &b, int stage) { b_element_v<false>(b, stage); }
  // the fused-limiter stage (instantiated only where an equation uses it)
  static void b_element_lim(const BatchLaunch &b, int stage) { b_element_v<true>(b, stage); }
  static void b_face_fs(const BatchLaunch &b, double tcoef) {
    k_face_batch<Eq, true><<<b.nsblk, b.blk, 0, b.st>>>(btabs(b), b.probs, b.sblk2prob, b.sblk0,
                                                         tcoef);
  }
  static void b_means(const BatchLaunch &b, int stage) {
    k_means_batch<Eq><<<b.nublk, b.blk, 0, b.st>>>(btabs(b), b.probs, b.ublk2prob, b.ublk0,
                                                    stage);
  }
  static void b_limit_tr(const BatchLaunch &b, int stage) {
    k_limit_tr_batch<Eq><<<b.nublk, b.blk, 0, b.st>>>(btabs(b), b.probs, b.ublk2prob, b.ublk0,
                                                       stage);
  }
  static void b_lambda(const BatchLaunch &b) {
    k_lambda_batch<Eq><<<b.nlblk, kBlock, 0, b.st>>>(btabs(b), b.probs, b.lblk2prob, b.lblk0);
  }
  static const BatchOps &batch_ops() {
    static const BatchOps o = {b_trace, b_face,   b_element, b_limit_tr,
                               b_lambda, nullptr, nullptr,   nullptr};
    return o;
  }
};

}  // namespace dg
