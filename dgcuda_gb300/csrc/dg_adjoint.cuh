// dg_adjoint.cuh -- tangent-linear and adjoint kernels of the shallow-water
// RK-DG right-hand side (no reference counterpart: DGCUDA has no
// derivatives).
//
// L(u, b) = (1/J) [ V(u, b) + S(u) ] with, per element and mode i,
//   V_i = sum_q GR_qi Gr_q + GS_qi Gs_q  + sum_q B_qi w_q J src_q
//   S_i = -/+ sum_j (len/2) w_j F*(U_L(j), U_R(j); n) E_i(j)     (left / right)
// Gr = fx ys - fy xs, Gs = fy xr - fx yr, src = (0, -g h b_x, -g h b_y).
// Both derivative codes use the same hand-derived 3x3 Jacobians, applied to
// vectors without forming them (sw_jac_mul, sw_jac_tmul):
//   A(U; n) = d(F(U).n)/dU, the physical normal flux of shallow water;
//   Rusanov F* = 1/2 (F(U_L).n + F(U_R).n + lam (U_L - U_R)),
//   lam = max(lam_L, lam_R), lam_X = |q_X / h_X| + sqrt(g h_X), q = m.n:
//     dF*/dU_L = 1/2 (A_L + lam I + (U_L - U_R) dlam/dU_L)
//     dF*/dU_R = 1/2 (A_R - lam I + (U_L - U_R) dlam/dU_R)
//   with the branch of the max (and the sign of q) taken from the state.
// Tangent-linear: dL = (dL/du) du + (dL/db) db (matrix-vector with A);
// adjoint: (dL/du)^T Lbar and (dL/db)^T Lbar (with A^T).  The dot-product
// test <Lbar, dL> = <ubar, du> + <bbar, db> holds to rounding.
#pragma once
#include "dg_kernels.cuh"

namespace dg {

// A(U; n) = d(F(U).n)/dU for shallow water, U = (h, hu, hv), applied to a
// vector without forming the matrix.  With u = hu/h, v = hv/h, qh = (hu,hv).n/h
// and gh = g h the rows are
//   [0, nx, ny],  [gh nx - u qh, u nx + qh, u ny],  [gh ny - v qh, v nx, v ny + qh].
// y = A x
__device__ __forceinline__ void sw_jac_mul(double u, double v, double qh, double gh, double nx,
                                           double ny, const double *x, double *y) {
  const double xn = fma(nx, x[1], ny * x[2]);
  const double t = fma(-qh, x[0], xn);
  const double g0 = gh * x[0];
  y[0] = xn;
  y[1] = fma(u, t, fma(qh, x[1], g0 * nx));
  y[2] = fma(v, t, fma(qh, x[2], g0 * ny));
}
// z = A^T f
__device__ __forceinline__ void sw_jac_tmul(double u, double v, double qh, double gh, double nx,
                                            double ny, const double *f, double *z) {
  const double wf = fma(u, f[1], v * f[2]);
  const double fn = fma(nx, f[1], ny * f[2]);
  const double fw = f[0] + wf;
  z[0] = fma(-qh, wf, gh * fn);
  z[1] = fma(nx, fw, qh * f[1]);
  z[2] = fma(ny, fw, qh * f[2]);
}

// one trace of a side: the pieces of A(U; n), c = sqrt(g h) and
// lam = |qh| + c
struct SwTrace {
  double ih, u, v, qh, gh, c, lam;
};
__device__ __forceinline__ SwTrace sw_trace(double g, const double *U, double nx, double ny) {
  SwTrace w;
  w.ih = rcp(U[0]);
  w.u = U[1] * w.ih;
  w.v = U[2] * w.ih;
  w.qh = fma(U[1], nx, U[2] * ny) * w.ih;
  w.gh = g * U[0];
  w.c = sqrt_pos(w.gh);
  w.lam = fabs(w.qh) + w.c;
  return w;
}
// d lam / dU = (-sg qh / h + c / (2 h), sg nx / h, sg ny / h), sg = sign(qh)
// (d sqrt(g h)/dh = g / (2 c) = c / (2 h))
__device__ __forceinline__ void sw_dlam(const SwTrace &w, double nx, double ny, double dl[3]) {
  const double sih = w.qh >= 0.0 ? w.ih : -w.ih;
  dl[0] = fma(-w.qh, sih, 0.5 * w.c * w.ih);
  dl[1] = sih * nx;
  dl[2] = sih * ny;
}

// d(ghost)/d(U_L) of a boundary code (reflect mirrors the momentum,
// transmissive copies, inflow / outflow ghosts do not depend on U_L)
__device__ __forceinline__ void sw_ghost_jac(int code, double nx, double ny, double M[3][3]) {
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) M[a][b] = 0.0;
  if (code == -4) {
    M[0][0] = M[1][1] = M[2][2] = 1.0;
  } else if (code == -1) {
    M[0][0] = 1.0;
    M[1][1] = 1.0 - 2 * nx * nx;
    M[1][2] = -2 * nx * ny;
    M[2][1] = -2 * ny * nx;
    M[2][2] = 1.0 - 2 * ny * ny;
  }
}

// ---------------------------------------------------------------------------
// linear traces of a field (no admissibility check): Tv[e][f][j][n]
template <int P>
__global__ void __launch_bounds__(kBlock) k_lin_trace(const __grid_constant__ Tab<P> tab,
                                                      const double *__restrict__ u,
                                                      const double *__restrict__ scale,
                                                      double sc, double *__restrict__ Tv, int K,
                                                      int Kp) {
  constexpr int N = 3, NP = Tab<P>::NP, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  const double f0 = scale ? sc * scale[e] : sc;
  double *Te = Tv + (size_t)e * (3 * N1 * N);
#pragma unroll
  for (int n = 0; n < N; n++) {
    double c[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) c[i] = f0 * u[(size_t)(n * NP + i) * Kp + e];
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < N1; j++) {
        double a = c[0] * tab.E[f][j][0];
#pragma unroll
        for (int i = 1; i < NP; i++) a = fma(c[i], tab.E[f][j][i], a);
        Te[(f * N1 + j) * N + n] = a;
      }
  }
}

// ---------------------------------------------------------------------------
// TL face: dF*(j) = (dF*/dU_L dU_L + dF*/dU_R dU_R) len/2 w_j into dFh.
// ADJ face: Fbar(j) = len/2 w_j (-Tbar_L(j) + Tbar_R(p-j)) from the
// adjoint traces, then Ubar_L = A_L^T Fbar -> UbL[s][j], Ubar_R = A_R^T
// Fbar -> UbR[s][j] (for a boundary side Ubar_R goes back to U_L).
template <int P, bool ADJ>
__global__ void __launch_bounds__(kBlock)
    k_sw_face_lin(const __grid_constant__ Tab<P> tab, const __grid_constant__ EqP q,
                  const double *__restrict__ T, const double *__restrict__ Tv,
                  const int4 *__restrict__ side, const double *__restrict__ sgeo,
                  double *__restrict__ out0, double *__restrict__ out1, int S) {
  constexpr int N = 3, N1 = P + 1;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int4 sd = side[s];
  const double nx = sgeo[s], ny = sgeo[S + s], hl = sgeo[2 * (size_t)S + s];
  const double *TL = T + ((size_t)sd.x * 3 + sd.z) * (N1 * N);
  const double *VL = Tv + ((size_t)sd.x * 3 + sd.z) * (N1 * N);
  const bool inner = sd.y >= 0;
  const double *TR = inner ? T + ((size_t)sd.y * 3 + sd.w) * (N1 * N) : nullptr;
  const double *VR = inner ? Tv + ((size_t)sd.y * 3 + sd.w) * (N1 * N) : nullptr;
#pragma unroll
  for (int j = 0; j < N1; j++) {
    double UL[N], UR[N], M[3][3];
#pragma unroll
    for (int n = 0; n < N; n++) UL[n] = TL[j * N + n];
    if (inner) {
#pragma unroll
      for (int n = 0; n < N; n++) UR[n] = TR[(N1 - 1 - j) * N + n];
    } else {
      ghost_state<ShallowWater>(q, sd.y, UL, UR, 0.0, 0.0, 0.0, nx, ny);
      sw_ghost_jac(sd.y, nx, ny, M);
    }
    // Rusanov: dF*/dU_L = 1/2 (A_L + lam I + d dlam_L^T), dF*/dU_R = 1/2 (A_R
    // - lam I + d dlam_R^T), d = U_L - U_R, the dlam term on the side of the
    // max only; the 1/2 goes into the edge scale
    const SwTrace wL = sw_trace(q.g, UL, nx, ny), wR = sw_trace(q.g, UR, nx, ny);
    const bool left = wL.lam >= wR.lam;
    const double lam = left ? wL.lam : wR.lam;
    double dl[3];
    sw_dlam(left ? wL : wR, nx, ny, dl);
    const double sc = 0.5 * hl * tab.w1[j];
    if (!ADJ) {
      double dUL[N], dUR[N], aL[N], aR[N];
#pragma unroll
      for (int n = 0; n < N; n++) dUL[n] = VL[j * N + n];
      if (inner) {
#pragma unroll
        for (int n = 0; n < N; n++) dUR[n] = VR[(N1 - 1 - j) * N + n];
      } else {
#pragma unroll
        for (int a = 0; a < N; a++)
          dUR[a] = fma(M[a][0], dUL[0], fma(M[a][1], dUL[1], M[a][2] * dUL[2]));
      }
      sw_jac_mul(wL.u, wL.v, wL.qh, wL.gh, nx, ny, dUL, aL);
      sw_jac_mul(wR.u, wR.v, wR.qh, wR.gh, nx, ny, dUR, aR);
      const double *dX = left ? dUL : dUR;
      const double dlam = fma(dl[0], dX[0], fma(dl[1], dX[1], dl[2] * dX[2]));
#pragma unroll
      for (int a = 0; a < N; a++) {
        const double v = fma(UL[a] - UR[a], dlam, fma(lam, dUL[a] - dUR[a], aL[a] + aR[a]));
        out0[(size_t)s * (N1 * N) + j * N + a] = v * sc;
      }
    } else {
      double Fb[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        const double r = inner ? VR[(N1 - 1 - j) * N + n] : 0.0;
        Fb[n] = sc * (r - VL[j * N + n]);
      }
      double bL[N], bR[N];
      sw_jac_tmul(wL.u, wL.v, wL.qh, wL.gh, nx, ny, Fb, bL);
      sw_jac_tmul(wR.u, wR.v, wR.qh, wR.gh, nx, ny, Fb, bR);
      const double dF = fma(UL[0] - UR[0], Fb[0], fma(UL[1] - UR[1], Fb[1], (UL[2] - UR[2]) * Fb[2]));
#pragma unroll
      for (int b = 0; b < N; b++) {
        bL[b] = fma(lam, Fb[b], bL[b]);
        bR[b] = fma(-lam, Fb[b], bR[b]);
        if (left) bL[b] = fma(dl[b], dF, bL[b]);
        else bR[b] = fma(dl[b], dF, bR[b]);
      }
      if (!inner) {  // U_R = ghost(U_L): its adjoint returns to U_L
#pragma unroll
        for (int b = 0; b < N; b++)
          bL[b] = fma(M[0][b], bR[0], fma(M[1][b], bR[1], fma(M[2][b], bR[2], bL[b])));
      }
#pragma unroll
      for (int n = 0; n < N; n++) {
        out0[(size_t)s * (N1 * N) + j * N + n] = bL[n];
        out1[(size_t)s * (N1 * N) + j * N + n] = inner ? bR[n] : 0.0;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// TL element: dout = ca du^n + cb du_s + cc dt (1/J) [dV + dS], dS gathered
// from dFh like the forward surface term.
// ADJ element: with Rbar = cc dt (1/J) obar, writes
//   ubar_s = cb obar + (dV/du)^T Rbar + (surface, gathered from UbL/UbR)
// and adds (dV/db)^T Rbar to bbar.  The ca u^n term is applied by the caller.
template <int P, bool ADJ>
__global__ void __launch_bounds__(kBlock)
    k_sw_element_lin(const __grid_constant__ Tab<P> tab, const __grid_constant__ EqP q,
                     const double *__restrict__ us, const double *__restrict__ bz_all,
                     const double *__restrict__ vin, const double *__restrict__ dbz_all,
                     const double *__restrict__ vn, double *__restrict__ vout,
                     double *__restrict__ bbar, const double *__restrict__ F0,
                     const double *__restrict__ F1, const int *__restrict__ esd,
                     const double *__restrict__ geo, double ca, double cb, double ccdt, int K,
                     int Kp) {
  constexpr int N = 3, NP = Tab<P>::NP, NQ = Tab<P>::NQ, N1 = Tab<P>::N1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[N][NP], v[N][NP], acc[N][NP], bz[NP], dbz[NP], bb[NP];
#pragma unroll
  for (int n = 0; n < N; n++)
#pragma unroll
    for (int i = 0; i < NP; i++) {
      c[n][i] = us[(size_t)(n * NP + i) * Kp + e];
      v[n][i] = vin[(size_t)(n * NP + i) * Kp + e];
      acc[n][i] = 0.0;
    }
#pragma unroll
  for (int i = 0; i < NP; i++) {
    bz[i] = bz_all ? bz_all[(size_t)i * Kp + e] : 0.0;
    dbz[i] = (!ADJ && dbz_all) ? dbz_all[(size_t)i * Kp + e] : 0.0;
    bb[i] = 0.0;
  }
  const double xr = geo[e], yr = geo[(size_t)Kp + e], xs = geo[2 * (size_t)Kp + e],
               ys = geo[3 * (size_t)Kp + e], iJ = geo[4 * (size_t)Kp + e];
  const double g = q.g;
  if (ADJ) {  // Rbar = cc dt (1/J) obar
    const double f = ccdt * iJ;
#pragma unroll
    for (int n = 0; n < N; n++)
#pragma unroll
      for (int i = 0; i < NP; i++) v[n][i] *= f;
  }
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double U[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
      double a = c[n][0] * tab.B[k][0];
#pragma unroll
      for (int i = 1; i < NP; i++) a = fma(c[n][i], tab.B[k][i], a);
      U[n] = a;
    }
    // A_x = A(U; (1, 0)) and A_y = A(U; (0, 1)): qh is u resp. v
    const double ih = rcp(U[0]);
    const double uu = U[1] * ih, vv = U[2] * ih, gh = g * U[0];
    double br = 0.0, bs = 0.0;
#pragma unroll
    for (int i = 1; i < NP; i++) {
      br = fma(bz[i], tab.GR[k][i], br);
      bs = fma(bz[i], tab.GS[k][i], bs);
    }
    const double bx = fma(ys, br, -yr * bs), by = fma(xr, bs, -xs * br);
    if (!ADJ) {
      double dU[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        double a = v[n][0] * tab.B[k][0];
#pragma unroll
        for (int i = 1; i < NP; i++) a = fma(v[n][i], tab.B[k][i], a);
        dU[n] = a;
      }
      double dfx[N], dfy[N];
      sw_jac_mul(uu, vv, uu, gh, 1.0, 0.0, dU, dfx);
      sw_jac_mul(uu, vv, vv, gh, 0.0, 1.0, dU, dfy);
#pragma unroll
      for (int n = 0; n < N; n++) {
        const double gr = fma(dfx[n], ys, -dfy[n] * xs), gs = fma(dfy[n], xr, -dfx[n] * yr);
#pragma unroll
        for (int i = 1; i < NP; i++)
          acc[n][i] = fma(tab.GR[k][i], gr, fma(tab.GS[k][i], gs, acc[n][i]));
      }
      if (bz_all || dbz_all) {
        double dbr = 0.0, dbs = 0.0;
#pragma unroll
        for (int i = 1; i < NP; i++) {
          dbr = fma(dbz[i], tab.GR[k][i], dbr);
          dbs = fma(dbz[i], tab.GS[k][i], dbs);
        }
        const double dbx = fma(ys, dbr, -yr * dbs), dby = fma(xr, dbs, -xs * dbr);
        const double sx = -g * fma(dU[0], bx, U[0] * dbx), sy = -g * fma(dU[0], by, U[0] * dby);
#pragma unroll
        for (int i = 0; i < NP; i++) {
          acc[1][i] = fma(sx, tab.B[k][i], acc[1][i]);
          acc[2][i] = fma(sy, tab.B[k][i], acc[2][i]);
        }
      }
    } else {
      double Ub[N], Gr[N], Gs[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        double a = 0.0, b = 0.0;
#pragma unroll
        for (int i = 1; i < NP; i++) {
          a = fma(tab.GR[k][i], v[n][i], a);
          b = fma(tab.GS[k][i], v[n][i], b);
        }
        Gr[n] = a;
        Gs[n] = b;
      }
      double fxb[N], fyb[N], zx[N], zy[N];
#pragma unroll
      for (int n = 0; n < N; n++) {
        fxb[n] = fma(ys, Gr[n], -yr * Gs[n]);
        fyb[n] = fma(xr, Gs[n], -xs * Gr[n]);
      }
      sw_jac_tmul(uu, vv, uu, gh, 1.0, 0.0, fxb, zx);
      sw_jac_tmul(uu, vv, vv, gh, 0.0, 1.0, fyb, zy);
#pragma unroll
      for (int m = 0; m < N; m++) Ub[m] = zx[m] + zy[m];
      if (bbar) {
        double Sx = 0.0, Sy = 0.0;
#pragma unroll
        for (int i = 0; i < NP; i++) {
          Sx = fma(tab.B[k][i], v[1][i], Sx);
          Sy = fma(tab.B[k][i], v[2][i], Sy);
        }
        Ub[0] = fma(-g, fma(bx, Sx, by * Sy), Ub[0]);
        const double hb = -g * U[0];
        const double bxb = hb * Sx, byb = hb * Sy;  // adjoints of bx, by
        const double brb = fma(ys, bxb, -xs * byb), bsb = fma(xr, byb, -yr * bxb);
#pragma unroll
        for (int i = 1; i < NP; i++) bb[i] = fma(tab.GR[k][i], brb, fma(tab.GS[k][i], bsb, bb[i]));
      }
#pragma unroll
      for (int n = 0; n < N; n++)
#pragma unroll
        for (int i = 0; i < NP; i++) acc[n][i] = fma(tab.B[k][i], Ub[n], acc[n][i]);
    }
  }
  // surface
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const int sd = esd[(size_t)f * Kp + e];
    const bool right = sd & 1;
    const size_t so = (size_t)(sd >> 1) * (N1 * N);
#pragma unroll
    for (int j = 0; j < N1; j++) {
      const int jj = right ? (N1 - 1 - j) : j;
#pragma unroll
      for (int n = 0; n < N; n++) {
        double fv;
        if (!ADJ) fv = (right ? 1.0 : -1.0) * F0[so + jj * N + n];
        else fv = right ? F1[so + jj * N + n] : F0[so + jj * N + n];
#pragma unroll
        for (int i = 0; i < NP; i++) acc[n][i] = fma(fv, tab.E[f][j][i], acc[n][i]);
      }
    }
  }
  if (!ADJ) {
    const double s = ccdt * iJ;
#pragma unroll
    for (int n = 0; n < N; n++)
#pragma unroll
      for (int i = 0; i < NP; i++) {
        const size_t o = (size_t)(n * NP + i) * Kp + e;
        double r = fma(s, acc[n][i], cb * v[n][i]);
        if (ca != 0.0) r = fma(ca, vn[o], r);
        vout[o] = r;
      }
  } else {
#pragma unroll
    for (int n = 0; n < N; n++)
#pragma unroll
      for (int i = 0; i < NP; i++) {
        const size_t o = (size_t)(n * NP + i) * Kp + e;
        vout[o] = fma(cb, vn[o], acc[n][i]);
      }
    if (bbar)
#pragma unroll
      for (int i = 0; i < NP; i++) bbar[(size_t)i * Kp + e] += bb[i];
  }
}

}  // namespace dg
