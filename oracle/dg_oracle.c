/* dg_oracle.c -- CPU restatement of the reference RK-DG method (TEST ORACLE).
 *
 * This file is test infrastructure: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it, as the reference for results and the timed CPU
 * baseline.  The product never links it.
 *
 * It restates, as plain C loops over sides and elements in the reference's
 * data layout C[var][mode][elem], the algorithm of DGCUDA's GPU solver
 * (src/2d/conservation):
 *   geometry ........ preval_* kernels, conserv_kernels.cu:412-585 (FP64:
 *                     the reference takes sqrtf of doubles there)
 *   surface ......... eval_surface / eval_left_right / eval_boundary,
 *                     conserv_kernels.cu:820-985
 *   volume .......... eval_volume, conserv_kernels.cu:992-1083
 *   assembly ........ eval_rhs, time_integrator.cu:26-101
 *   limiter ......... limit_c, conserv_kernels.cu:640-720
 *   equations ....... euler/euler.cu, shallowwater/shallowwater.cu,
 *                     advection/advection.cu (upwind), maxwells/maxwells.cu
 *   RK4 / RK2 ....... time_integrator.cu:139-433, :511-717
 *   CFL ............. eval_global_lambda + host max + dt formula,
 *                     time_integrator.cu:200-217
 *   projection ...... init_conditions / evalU0, conserv_kernels.cu:201-228
 *   L2 error ........ eval_error_L2, conserv_kernels.cu:1432-1479
 * plus the pieces the reference lacks (marked "extension"): SSP-RK3, the
 * transmissive boundary code -4, the limiter for p > 1, the gravity
 * parameter.
 *
 * Parity pinning: tests/test_oracle_golden.py checks every function here
 * against golden vectors produced by the reference's own kernels
 * (tests/golden/make_golden.py), with the reference's basis tabulation
 * loaded through or_set_tables.
 *
 * Positivity: where the reference flattens an element whose trace or
 * volume value is non-physical it does so racily from several GPU threads
 * (euler.cu:92-116).  The oracle uses the order-free rule the GPU solver
 * implements: an element whose edge traces contain a non-physical value is
 * flattened to its mean before any face uses it; an element with a
 * non-physical volume value is flattened too and its mean is used for the
 * whole volume integral (and by the RK update that follows).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../dgcuda_gb300/csrc/dg_tables_data.h"

#define NMAX 4
#define NPM DG_NP_MAX
#define NQM DG_NQ_MAX
#define N1M DG_N1_MAX

enum { EQ_ADV = 0, EQ_EULER = 1, EQ_SW = 2, EQ_MAXWELL = 3 };
enum {
  PB_NONE = 0, PB_ADV_SINE = 1, PB_ADV_LINEAR = 2, PB_EULER_VORTEX = 3, PB_EULER_RIEMANN4 = 4,
  PB_EULER_SUPERSONIC = 5, PB_SW_HUMP = 6, PB_SW_TEST = 7, PB_MAXWELL_PLANE = 8,
  PB_EULER_CYLINDER = 9, PB_EULER_LSHOCK = 10, PB_EULER_DOUBLEMACH = 11, PB_EULER_AIRFOIL = 12,
  PB_ADV_SQUAREHILL = 13, PB_ADV_ROTATINGHILL = 14, PB_ADV_SPIN = 15, PB_MAXWELL_CMIRROR = 16,
  PB_MAXWELL_WSCATTER = 17, PB_EULER_PULSE = 18
};
#define NSER 16

typedef struct or_solver {
  int eq, p, N, np, nq, n1, K, S, problem;
  double gamma, g, ax, ay, mu, eps, prm[8];
  /* advection velocity a = (ax, ay) + agrad (x, y) (extension of a constant
   * get_velocity to affine fields); inflow pressure series (tube.cu:52-97) */
  double agrad[4];
  int nser;
  double ser_t0, ser[NSER][3];
  /* tables */
  double r[NQM], s[NQM], w[NQM], t1[N1M], w1[N1M];
  double B[NQM][NPM], GR[NQM][NPM], GS[NQM][NPM], E[3][N1M][NPM], VT[3][NPM];
  /* mesh, reference layout */
  double *V; /* 6*K */
  int *es;   /* 3*K */
  double *sxy;
  int *left, *right, *lsn, *rsn;
  /* geometry */
  double *J, *xr, *yr, *xs, *ys, *slen, *nx, *ny;
  double min_r;
  /* work */
  double *vol, *sl, *sr;
  int flattened;
  double *bathy; /* shallow-water bed modes [mode][elem] or NULL (extension) */
} or_solver;

static double dmin2(double a, double b) { return a < b ? a : b; }

/* ---------------- tables ---------------- */
static long double poly(int k, long double r, long double s, int dr, int ds) {
  /* phi_k and its derivatives from the monomial coefficients */
  long double acc = 0;
  for (int m = 0; m <= k; m++) {
    int a = DG_MONO[m][0], b = DG_MONO[m][1];
    long double c = DG_COEF[k][m];
    if (c == 0) continue;
    long double term = c;
    if (dr) {
      if (a == 0) continue;
      term *= a;
      a -= 1;
    }
    if (ds) {
      if (b == 0) continue;
      term *= b;
      b -= 1;
    }
    for (int i = 0; i < a; i++) term *= r;
    for (int i = 0; i < b; i++) term *= s;
    acc += term;
  }
  return acc;
}

static void exact_tables(or_solver *o) {
  const dg_order_tables *T = &DG_TABLES[o->p];
  o->nq = T->n_q;
  o->n1 = T->n_1;
  for (int q = 0; q < o->nq; q++) {
    o->r[q] = T->r[q];
    o->s[q] = T->s[q];
    o->w[q] = T->w[q];
  }
  for (int j = 0; j < o->n1; j++) {
    o->t1[j] = T->t1[j];
    o->w1[j] = T->w1[j];
  }
  /* tabulate from the monomial coefficients (basis.cu:196-214) */
  for (int i = 0; i < o->np; i++) {
    for (int q = 0; q < o->nq; q++) {
      o->B[q][i] = (double)poly(i, o->r[q], o->s[q], 0, 0);
      o->GR[q][i] = (double)(o->w[q] * poly(i, o->r[q], o->s[q], 1, 0));
      o->GS[q][i] = (double)(o->w[q] * poly(i, o->r[q], o->s[q], 0, 1));
    }
    for (int j = 0; j < o->n1; j++) {
      long double t = o->t1[j], tr = o->t1[o->n1 - 1 - j];
      o->E[0][j][i] = (double)poly(i, 0.5L + 0.5L * t, 0, 0, 0);
      o->E[1][j][i] = (double)poly(i, (1 - t) / 2, (1 + t) / 2, 0, 0);
      o->E[2][j][i] = (double)poly(i, 0, 0.5L + 0.5L * tr, 0, 0);
    }
    o->VT[0][i] = (double)poly(i, 0, 0, 0, 0);
    o->VT[1][i] = (double)poly(i, 1, 0, 0, 0);
    o->VT[2][i] = (double)poly(i, 0, 1, 0, 0);
  }
}

int or_set_tables(or_solver *o, int nq, int n1, const double *basis, const double *gx,
                  const double *gy, const double *side, const double *vertex, const double *w,
                  const double *r1, const double *r2, const double *r_oned,
                  const double *w_oned) {
  if (nq != o->nq || n1 != o->n1) return 1;
  int np = o->np;
  for (int q = 0; q < nq; q++) {
    o->w[q] = w[q];
    o->r[q] = r1[q];
    o->s[q] = r2[q];
    for (int i = 0; i < np; i++) {
      o->B[q][i] = basis[i * nq + q];
      o->GR[q][i] = gx[i * nq + q];
      o->GS[q][i] = gy[i * nq + q];
    }
  }
  for (int j = 0; j < n1; j++) {
    o->t1[j] = r_oned[j];
    o->w1[j] = w_oned[j];
    for (int f = 0; f < 3; f++)
      for (int i = 0; i < np; i++) o->E[f][j][i] = side[f * np * n1 + i * n1 + j];
  }
  for (int v = 0; v < 3; v++)
    for (int i = 0; i < np; i++) o->VT[v][i] = vertex[i * 3 + v];
  return 0;
}

/* the tabulation in the reference's flat layout (basis, grad_x, grad_y,
 * side, vertex, w, r1, r2, r_oned, w_oned; see or_set_tables) */
int or_get_tables(const or_solver *o, double *out) {
  int np = o->np, nq = o->nq, n1 = o->n1;
  double *p = out;
  for (int i = 0; i < np; i++) for (int q = 0; q < nq; q++) *p++ = o->B[q][i];
  for (int i = 0; i < np; i++) for (int q = 0; q < nq; q++) *p++ = o->GR[q][i];
  for (int i = 0; i < np; i++) for (int q = 0; q < nq; q++) *p++ = o->GS[q][i];
  for (int f = 0; f < 3; f++)
    for (int i = 0; i < np; i++) for (int j = 0; j < n1; j++) *p++ = o->E[f][j][i];
  for (int i = 0; i < np; i++) for (int v = 0; v < 3; v++) *p++ = o->VT[v][i];
  for (int q = 0; q < nq; q++) *p++ = o->w[q];
  for (int q = 0; q < nq; q++) *p++ = o->r[q];
  for (int q = 0; q < nq; q++) *p++ = o->s[q];
  for (int j = 0; j < n1; j++) *p++ = o->t1[j];
  for (int j = 0; j < n1; j++) *p++ = o->w1[j];
  return (int)(p - out);
}

/* ---------------- problems (initial / boundary / exact states) ---------------- */
/* double Mach reflection (euler/doublemach/doublemach.cu:20-93) */
#define DM_X0 0.16666666666666666
static void dm_shock(const or_solver *o, double *U) {
  U[0] = 8.;
  U[1] = 8.25 * 0.86602540378443864676 * U[0];
  U[2] = -8.25 * 0.5 * U[0];
  U[3] = 0.5 * U[0] * 8.25 * 8.25 + 116.5 / (o->gamma - 1.0);
}
static void dm_rest(const or_solver *o, double *U) {
  U[0] = o->gamma;
  U[1] = 0.;
  U[2] = 0.;
  U[3] = 1. / (o->gamma - 1.0);
}
/* uniform flow along x at Mach M (cylinder.cu:23-45, lshock.cu:23-45) */
static void uniform_mach(const or_solver *o, double M, double *U) {
  U[0] = o->gamma;
  U[1] = U[0] * M;
  U[2] = 0.;
  U[3] = 0.5 * U[0] * M * M + 1. / (o->gamma - 1.0);
}

/* Gaussian hill carried by the rotation of speed w about the origin: the
 * initial hill at the point rotated back by w t (rotatinghill.cu:58-67) */
#define ROT_HILL (2 * 3.14159265358979323) /* rotatinghill.cu:10 */
#define ROT_SPIN (2 * 3.14159)             /* spin.cu:10 */
static double rotated_hill(double A, double x0, double y0, double r, double w, double x, double y,
                           double t) {
  double c = cos(w * t), s = sin(w * t);
  double dx = x * c + y * s - x0, dy = -x * s + y * c - y0;
  return A * exp(-(dx * dx + dy * dy) / (2 * r * r));
}

/* inflow of the tube / trumpet problems (tube.cu:52-97) */
static void pulse_state(const or_solver *o, double t, double *U) {
  double p = 1.0, tt = t + o->ser_t0;
  for (int k = 0; k < o->nser; k++) p += o->ser[k][0] * cos(o->ser[k][1] * tt + o->ser[k][2]);
  double rho = o->gamma * pow(p, 1. / o->gamma), u = (p - 1) / o->gamma;
  U[0] = rho;
  U[1] = u * rho;
  U[2] = 0.;
  U[3] = 0.5 * rho * u * u + p / (o->gamma - 1.);
}

static void exact_state(const or_solver *o, double *U, double x, double y, double t) {
  const double *P = o->prm;
  switch (o->problem) {
    case PB_ADV_SINE: {
      double xs = x - o->ax * t, ys = y - o->ay * t;
      U[0] = sin(2 * M_PI * xs) * sin(2 * M_PI * ys);
      break;
    }
    case PB_ADV_LINEAR: /* advection/exact/exact.cu:25-27 */
      U[0] = x - y;
      break;
    case PB_EULER_VORTEX: {
      double gam = o->gamma, beta = P[0], L = P[5];
      double xc = P[1] + P[3] * t, yc = P[2] + P[4] * t;
      double dx = x - xc, dy = y - yc;
      if (L > 0) {
        dx -= L * floor(dx / L + 0.5);
        dy -= L * floor(dy / L + 0.5);
      }
      double r2 = dx * dx + dy * dy;
      double e = exp(0.5 * (1 - r2));
      double u = P[3] - beta / (2 * M_PI) * e * dy;
      double v = P[4] + beta / (2 * M_PI) * e * dx;
      double T = 1 - (gam - 1) * beta * beta / (8 * gam * M_PI * M_PI) * e * e;
      double rho = pow(T, 1 / (gam - 1));
      double p = pow(rho, gam);
      U[0] = rho;
      U[1] = rho * u;
      U[2] = rho * v;
      U[3] = p / (gam - 1) + 0.5 * rho * (u * u + v * v);
      break;
    }
    case PB_EULER_RIEMANN4: {
      double gam = o->gamma, rho, u, v, p;
      if (x >= 0.5 && y >= 0.5) { rho = 1.5; u = 0; v = 0; p = 1.5; }
      else if (x < 0.5 && y >= 0.5) { rho = 0.5323; u = 1.206; v = 0; p = 0.3; }
      else if (x < 0.5 && y < 0.5) { rho = 0.138; u = 1.206; v = 1.206; p = 0.029; }
      else { rho = 0.5323; u = 0; v = 1.206; p = 0.3; }
      U[0] = rho;
      U[1] = rho * u;
      U[2] = rho * v;
      U[3] = p / (gam - 1) + 0.5 * rho * (u * u + v * v);
      break;
    }
    case PB_EULER_SUPERSONIC: { /* euler/supersonic/supersonic.cu:27-37 */
      const double GAM = 1.4, MACH = 2.25;
      double r = sqrt(x * x + y * y);
      U[0] = pow(1 + 1.0125 * (1. - 1. / (r * r)), 2.5);
      U[1] = U[0] * sin(atan(y / x)) * MACH / r;
      U[2] = U[0] * -cos(atan(y / x)) * MACH / r;
      double p = (1.0 / GAM) * pow(U[0], GAM);
      U[3] = 0.5 * U[0] * (MACH * MACH / (r * r)) + p * (1. / (GAM - 1.));
      break;
    }
    case PB_SW_HUMP: {
      double dx = x - P[3], dy = y - P[4], s = P[2];
      U[0] = P[0] + P[1] * exp(-(dx * dx + dy * dy) / (s * s));
      U[1] = 0;
      U[2] = 0;
      break;
    }
    case PB_SW_TEST: /* shallowwater/test/test.cu:25-35 */
      U[0] = 10 + exp(-(pow(x - 0.5, 2) + pow(y - 0.5, 2)) / (2 * 0.1 * 0.1));
      U[1] = 0;
      U[2] = 0;
      break;
    case PB_EULER_CYLINDER:
      uniform_mach(o, P[0] != 0 ? P[0] : 0.38, U);
      break;
    case PB_EULER_LSHOCK:
      uniform_mach(o, P[0] != 0 ? P[0] : 2.0, U);
      break;
    case PB_EULER_DOUBLEMACH: /* U_inflow = U_outflow (doublemach.cu:55-70) */
      if (x < DM_X0 + (1. + 20. * t) / sqrt(3.)) dm_shock(o, U);
      else dm_rest(o, U);
      break;
    case PB_EULER_AIRFOIL: { /* airfoil.cu:22-45 */
      double M = P[0] != 0 ? P[0] : 0.98, a = (P[1] != 0 ? P[1] : 5.) * (M_PI / 180.);
      U[0] = o->gamma;
      U[1] = U[0] * M * cos(a);
      U[2] = U[0] * M * sin(a);
      U[3] = 0.5 * U[0] * M * M + 1. / (o->gamma - 1.0);
      break;
    }
    case PB_EULER_PULSE: /* tube.cu:52-97: U_inflow = U_outflow */
      pulse_state(o, t, U);
      break;
    case PB_ADV_SQUAREHILL: { /* squarehill.cu:22-30, translated */
      double xs = x - o->ax * t, ys = y - o->ay * t;
      U[0] = (xs < -.2 && xs > -.8 && ys < .1 && ys > -.5) ? 1. : 0.;
      break;
    }
    case PB_ADV_ROTATINGHILL: /* rotatinghill.cu:22-30, 58-67 */
      U[0] = rotated_hill(5., 0.2, 0.0, 0.15, ROT_HILL, x, y, t);
      break;
    case PB_ADV_SPIN: /* spin.cu:22-30 */
      U[0] = rotated_hill(1., 0.5, 0.5, 0.1, ROT_SPIN, x, y, t);
      break;
    case PB_MAXWELL_PLANE: {
      double c = 1 / sqrt(o->mu * o->eps);
      double ez = sin(2 * M_PI * (x - c * t));
      U[0] = 0;
      U[1] = sqrt(o->eps / o->mu) * ez;
      U[2] = ez;
      break;
    }
    default:
      for (int n = 0; n < NMAX; n++) U[n] = 0;
  }
}

/* the initial state U0: the exact state at t = 0 except where a problem's
 * initial data differ from its boundary data */
static void init_state(const or_solver *o, double *U, double x, double y) {
  if (o->problem == PB_EULER_DOUBLEMACH) { /* doublemach.cu:41-52 */
    double angle = atan(y / (x - DM_X0));
    if (angle > 60. * M_PI / 180 || x < DM_X0) dm_shock(o, U);
    else dm_rest(o, U);
    return;
  }
  if (o->problem == PB_EULER_PULSE) { /* tube.cu:25-45: at rest */
    dm_rest(o, U);
    return;
  }
  exact_state(o, U, x, y, 0.0);
}

/* U_inflow: the exact state except where a problem's inflow differs */
static void inflow_state(const or_solver *o, double *U, double x, double y, double t) {
  switch (o->problem) {
    case PB_ADV_SQUAREHILL: /* squarehill.cu:43-45 */
    case PB_ADV_SPIN:       /* spin.cu:43-46 */
      U[0] = 0.;
      return;
    case PB_MAXWELL_CMIRROR: /* cmirror.cu:38-47 */
      U[0] = U[1] = 0.;
      U[2] = t <= 1. / 20 ? 2 * sin(20. * M_PI * t) : 0.;
      return;
    case PB_MAXWELL_WSCATTER: /* wscatter.cu:38-50 */
      U[0] = U[1] = 0.;
      U[2] = (y < .15 && y > -.15 && t < 0.5) ? sin(2. * M_PI * t) : 0.;
      return;
    default:
      exact_state(o, U, x, y, t);
  }
}

/* ghost state of a boundary side (eval_boundary, conserv_kernels.cu:820-843) */
static void ghost(const or_solver *o, int code, const double *UL, double *UR, double x, double y,
                  double t, double nx, double ny) {
  for (int n = 0; n < NMAX; n++) UR[n] = 0;
  if (code == -4) { /* extension: transmissive */
    for (int n = 0; n < o->N; n++) UR[n] = UL[n];
    return;
  }
  if (code == -3) { /* inflow: U_inflow */
    inflow_state(o, UR, x, y, t);
    return;
  }
  if (code == -2) { /* outflow: Euler problems use the exact state; others leave zero */
    if (o->eq == EQ_EULER) exact_state(o, UR, x, y, t);
    return;
  }
  /* reflect */
  if (o->eq == EQ_EULER) {
    if (o->problem == PB_EULER_DOUBLEMACH && x < DM_X0) { /* doublemach.cu:75-93 */
      dm_shock(o, UR);
    } else if (o->problem == PB_EULER_SUPERSONIC || o->problem == PB_EULER_CYLINDER) {
      /* curved wall around the origin (supersonic.cu:65-87, cylinder.cu:55-80) */
      double d = sqrt(x * x + y * y), Nx = x / d, Ny = y / d;
      if (Nx * nx + Ny * ny < 0) {
        Nx = -Nx;
        Ny = -Ny;
      }
      UR[0] = UL[0];
      UR[3] = UL[3];
      UR[1] = (UL[1] * Ny - UL[2] * Nx) * Ny;
      UR[2] = -(UL[1] * Ny - UL[2] * Nx) * Nx;
    } else {
      double dot = UL[1] * nx + UL[2] * ny;
      UR[0] = UL[0];
      UR[1] = UL[1] - 2 * dot * nx;
      UR[2] = UL[2] - 2 * dot * ny;
      UR[3] = UL[3];
    }
  } else if (o->eq == EQ_SW) { /* shallowwater/test/test.cu:63-77 */
    double dot = UL[1] * nx + UL[2] * ny;
    UR[0] = UL[0];
    UR[1] = UL[1] - 2 * dot * nx;
    UR[2] = UL[2] - 2 * dot * ny;
  } else if (o->eq == EQ_MAXWELL) { /* maxwells/cmirror/cmirror.cu:63-77 */
    double dot = UL[0] * nx + UL[1] * ny;
    UR[2] = UL[2];
    UR[0] = -UL[0] + 2 * dot * nx;
    UR[1] = -UL[1] + 2 * dot * ny;
  }
}

/* ---------------- equations ---------------- */
static int physical(const or_solver *o, const double *U) {
  if (o->eq == EQ_EULER) { /* euler.cu:76-86 */
    if (U[0] < 0) return 0;
    double p = (o->gamma - 1.) * (U[3] - (U[1] * U[1] + U[2] * U[2]) / 2. / U[0]);
    return !(p < 0);
  }
  if (o->eq == EQ_SW) return U[0] >= 0.; /* shallowwater.cu:48-50 */
  return 1;
}

static void flux(const or_solver *o, const double *U, double *fx, double *fy) {
  switch (o->eq) {
    case EQ_ADV: /* advection.cu:51-71 */
      fx[0] = o->ax * U[0];
      fy[0] = o->ay * U[0];
      break;
    case EQ_EULER: { /* euler.cu:138-160 */
      double rho = U[0], ru = U[1], rv = U[2], E = U[3];
      double p = (o->gamma - 1.) * (E - (ru * ru + rv * rv) / 2. / rho);
      fx[0] = ru;
      fx[1] = ru * ru / rho + p;
      fx[2] = ru * rv / rho;
      fx[3] = ru * (E + p) / rho;
      fy[0] = rv;
      fy[1] = ru * rv / rho;
      fy[2] = rv * rv / rho + p;
      fy[3] = rv * (E + p) / rho;
      break;
    }
    case EQ_SW: { /* shallowwater.cu:91-109 */
      double h = U[0], uh = U[1], vh = U[2], G = o->g;
      fx[0] = uh;
      fx[1] = uh * uh / h + 0.5 * G * h * h;
      fx[2] = uh * vh / h;
      fy[0] = vh;
      fy[1] = uh * vh / h;
      fy[2] = vh * vh / h + 0.5 * G * h * h;
      break;
    }
    case EQ_MAXWELL: /* maxwells.cu:67-84 */
      fx[0] = 0.;
      fx[1] = 1. / o->mu * U[2];
      fx[2] = 1. / o->eps * U[1];
      fy[0] = -1. / o->mu * U[2];
      fy[1] = 0.;
      fy[2] = -1. / o->eps * U[0];
      break;
  }
}

/* speed |s| + c with the reference's sign logic (euler.cu:170-213) */
static double side_speed(const or_solver *o, const double *U, double nx, double ny) {
  double c, s;
  if (o->eq == EQ_EULER) {
    double p = (o->gamma - 1.) * (U[3] - (U[1] * U[1] + U[2] * U[2]) / 2. / U[0]);
    c = sqrt(o->gamma * p / U[0]);
  } else {
    c = sqrt(U[0] * o->g);
  }
  s = nx * (U[1] / U[0]) + ny * (U[2] / U[0]);
  return s > 0. ? s + c : -s + c;
}

/* get_velocity (advection.cu:12) for an affine field */
static void velocity(const or_solver *o, double x, double y, double *vx, double *vy) {
  *vx = o->ax + o->agrad[0] * x + o->agrad[1] * y;
  *vy = o->ay + o->agrad[2] * x + o->agrad[3] * y;
}

/* numerical flux at a point (x, y) of the side (advection needs it) */
static void riemann(const or_solver *o, const double *UL, const double *UR, double nx, double ny,
                    double x, double y, double *F) {
  int N = o->N;
  if (o->eq == EQ_ADV) { /* upwind, advection.cu:94-116 */
    double vx, vy;
    velocity(o, x, y, &vx, &vy);
    if (nx * vx + ny * vy > 0)
      F[0] = vx * UL[0] * nx + vy * UL[0] * ny;
    else
      F[0] = vx * UR[0] * nx + vy * UR[0] * ny;
    return;
  }
  double fxl[NMAX], fyl[NMAX], fxr[NMAX], fyr[NMAX], lam;
  flux(o, UL, fxl, fyl);
  flux(o, UR, fxr, fyr);
  if (o->eq == EQ_MAXWELL) {
    lam = fabs(1. / sqrt(o->eps * o->mu)); /* maxwells.cu:93-105 */
  } else {
    double a = fabs(side_speed(o, UL, nx, ny)), b = fabs(side_speed(o, UR, nx, ny));
    lam = a > b ? a : b;
  }
  for (int n = 0; n < N; n++) /* local Lax-Friedrichs, euler.cu:233-236 */
    F[n] = 0.5 * ((fxl[n] + fxr[n]) * nx + (fyl[n] + fyr[n]) * ny + lam * (UL[n] - UR[n]));
}

/* ---------------- set-up ---------------- */
static void *xmalloc(size_t n) { return calloc(n ? n : 1, 1); }

or_solver *or_create(int eq, int p, int K, int S, const double *V, const int *es,
                     const double *sxy, const int *se, const double *prm16, int problem) {
  if (eq < 0 || eq > 3 || p < 0 || p > DG_PMAX || K <= 0 || S <= 0) return 0;
  or_solver *o = (or_solver *)xmalloc(sizeof *o);
  static const int NV[4] = {1, 4, 3, 3};
  o->eq = eq;
  o->p = p;
  o->N = NV[eq];
  o->np = (p + 1) * (p + 2) / 2;
  o->K = K;
  o->S = S;
  o->problem = problem;
  o->gamma = prm16[1];
  o->ax = prm16[2];
  o->ay = prm16[3];
  o->mu = prm16[4];
  o->eps = prm16[5];
  o->g = prm16[6];
  for (int i = 0; i < 8; i++) o->prm[i] = prm16[8 + i];
  if (problem == PB_ADV_ROTATINGHILL || problem == PB_ADV_SPIN) {
    /* the problem's rotation (-w y, w x) (rotatinghill.cu:37-40, spin.cu:37-40) */
    double w = problem == PB_ADV_SPIN ? ROT_SPIN : ROT_HILL;
    o->ax = o->ay = 0.;
    o->agrad[1] = -w;
    o->agrad[2] = w;
  }
  exact_tables(o);
  o->V = (double *)xmalloc(sizeof(double) * 6 * K);
  memcpy(o->V, V, sizeof(double) * 6 * K);
  o->es = (int *)xmalloc(sizeof(int) * 3 * K);
  memcpy(o->es, es, sizeof(int) * 3 * K);
  o->sxy = (double *)xmalloc(sizeof(double) * 4 * S);
  memcpy(o->sxy, sxy, sizeof(double) * 4 * S);
  o->left = (int *)xmalloc(sizeof(int) * 4 * S);
  memcpy(o->left, se, sizeof(int) * 4 * S);
  o->right = o->left + S;
  o->lsn = o->left + 2 * S;
  o->rsn = o->left + 3 * S;
  o->J = (double *)xmalloc(sizeof(double) * 5 * K);
  o->xr = o->J + K;
  o->yr = o->J + 2 * K;
  o->xs = o->J + 3 * K;
  o->ys = o->J + 4 * K;
  o->slen = (double *)xmalloc(sizeof(double) * 3 * S);
  o->nx = o->slen + S;
  o->ny = o->slen + 2 * S;
  size_t nd = (size_t)o->N * o->np;
  o->vol = (double *)xmalloc(sizeof(double) * nd * K);
  o->sl = (double *)xmalloc(sizeof(double) * nd * S);
  o->sr = (double *)xmalloc(sizeof(double) * nd * S);
  const double *V1x = V, *V1y = V + K, *V2x = V + 2 * K, *V2y = V + 3 * K, *V3x = V + 4 * K,
               *V3y = V + 5 * K;
  /* preval_inscribed_circles (diameter) -> min, preval_jacobian, preval_partials */
  o->min_r = 1e300;
  for (int e = 0; e < K; e++) {
    double a = sqrt(pow(V1x[e] - V2x[e], 2) + pow(V1y[e] - V2y[e], 2));
    double b = sqrt(pow(V2x[e] - V3x[e], 2) + pow(V2y[e] - V3y[e], 2));
    double c = sqrt(pow(V1x[e] - V3x[e], 2) + pow(V1y[e] - V3y[e], 2));
    double k = 0.5 * (a + b + c);
    double d = 2 * sqrt(k * (k - a) * (k - b) * (k - c)) / k;
    if (e == 0 || d < o->min_r) o->min_r = d;
    o->J[e] = (V2x[e] - V1x[e]) * (V3y[e] - V1y[e]) - (V3x[e] - V1x[e]) * (V2y[e] - V1y[e]);
    o->xr[e] = V2x[e] - V1x[e];
    o->yr[e] = V2y[e] - V1y[e];
    o->xs[e] = V3x[e] - V1x[e];
    o->ys[e] = V3y[e] - V1y[e];
  }
  /* preval_side_length, preval_normals, preval_normals_direction */
  for (int s = 0; s < S; s++) {
    double x = sxy[2 * S + s] - sxy[s], y = sxy[3 * S + s] - sxy[S + s];
    double len = sqrt(pow(x, 2) + pow(y, 2));
    o->slen[s] = len;
    double nx = -y / len, ny = x / len;
    int L = o->left[s], f = o->lsn[s];
    double tx, ty, ix, iy;
    if (f == 0) {
      tx = V3x[L]; ty = V3y[L];
      ix = (V1x[L] + V2x[L]) / 2.; iy = (V1y[L] + V2y[L]) / 2.;
    } else if (f == 1) {
      tx = V1x[L]; ty = V1y[L];
      ix = (V2x[L] + V3x[L]) / 2.; iy = (V2y[L] + V3y[L]) / 2.;
    } else {
      tx = V2x[L]; ty = V2y[L];
      ix = (V1x[L] + V3x[L]) / 2.; iy = (V1y[L] + V3y[L]) / 2.;
    }
    if (nx * (tx - ix) + ny * (ty - iy) > 0) {
      nx = -nx;
      ny = -ny;
    }
    o->nx[s] = nx;
    o->ny[s] = ny;
  }
  return o;
}

/* shallow-water bed modes [mode][elem] (copied), or NULL for a flat bed */
/* advection velocity field a = (ax, ay) + grad (x, y) */
int or_set_field(or_solver *o, double ax, double ay, const double *grad) {
  o->ax = ax;
  o->ay = ay;
  for (int i = 0; i < 4; i++) o->agrad[i] = grad ? grad[i] : 0.;
  return 0;
}

/* inflow pressure series of the pulse problem */
int or_set_series(or_solver *o, int n, const double *amp, const double *omega,
                  const double *phase, double t0) {
  if (n < 0 || n > NSER) return 1;
  o->nser = n;
  o->ser_t0 = t0;
  for (int k = 0; k < n; k++) {
    o->ser[k][0] = amp[k];
    o->ser[k][1] = omega[k];
    o->ser[k][2] = phase[k];
  }
  return 0;
}

int or_set_bathymetry(or_solver *o, const double *b) {
  free(o->bathy);
  o->bathy = 0;
  if (b) {
    size_t n = (size_t)o->np * o->K;
    o->bathy = (double *)xmalloc(sizeof(double) * n);
    memcpy(o->bathy, b, sizeof(double) * n);
  }
  return 0;
}

void or_destroy(or_solver *o) {
  if (!o) return;
  free(o->bathy);
  free(o->V);
  free(o->es);
  free(o->sxy);
  free(o->left);
  free(o->J);
  free(o->slen);
  free(o->vol);
  free(o->sl);
  free(o->sr);
  free(o);
}

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

double or_min_diameter(const or_solver *o) { return o->min_r; }
/* elements flattened by the positivity rule since the last or_rhs / or_step */
int or_flattened(const or_solver *o) { return o->flattened; }

/* ---------------- the DG operator ---------------- */
#define CI(n, i, e) ((size_t)K * np * (n) + (size_t)(i) * K + (e))

/* face point (j) coordinates on face f of element e (get_coordinates_1d) */
static void face_xy(const or_solver *o, int e, int f, int j, double *x, double *y) {
  int K = o->K;
  const double *V = o->V;
  double r, s, t = o->t1[j];
  if (f == 0) { r = 0.5 + 0.5 * t; s = 0.; }
  else if (f == 1) { r = (1. - t) / 2.; s = (1. + t) / 2.; }
  else { r = 0.; s = 0.5 + 0.5 * o->t1[o->n1 - 1 - j]; }
  *x = V[2 * K + e] * r + V[4 * K + e] * s + V[e] * (1 - r - s);
  *y = V[3 * K + e] * r + V[5 * K + e] * s + V[K + e] * (1 - r - s);
}

static void vol_xy(const or_solver *o, int e, int q, double *x, double *y) {
  int K = o->K;
  const double *V = o->V;
  double r = o->r[q], s = o->s[q];
  *x = V[2 * K + e] * r + V[4 * K + e] * s + V[e] * (1 - r - s);
  *y = V[3 * K + e] * r + V[5 * K + e] * s + V[K + e] * (1 - r - s);
}

/* flatten elements whose edge traces are non-physical (order-free rule) */
static int flatten_pass(or_solver *o, double *C) {
  int K = o->K, np = o->np, N = o->N, n1 = o->n1, cnt = 0;
  if (o->eq != EQ_EULER && o->eq != EQ_SW) return 0;
#pragma omp parallel for reduction(+ : cnt) schedule(static)
  for (int e = 0; e < K; e++) {
    int bad = 0;
    for (int f = 0; f < 3 && !bad; f++)
      for (int j = 0; j < n1 && !bad; j++) {
        double U[NMAX] = {0, 0, 0, 0};
        for (int i = 0; i < np; i++)
          for (int n = 0; n < N; n++) U[n] += C[CI(n, i, e)] * o->E[f][j][i];
        if (!physical(o, U)) bad = 1;
      }
    if (bad) {
      cnt++;
      for (int n = 0; n < N; n++)
        for (int i = 1; i < np; i++) C[CI(n, i, e)] = 0.;
    }
  }
  return cnt;
}

/* k = dt/J (vol + surf) for state C at time t; C may be flattened in place */
static void dg_operator(or_solver *o, double *C, double t, double dt, double *out) {
  int K = o->K, S = o->S, np = o->np, N = o->N, n1 = o->n1, nq = o->nq;
  o->flattened += flatten_pass(o, C);
  double *sl = o->sl, *sr = o->sr, *vol = o->vol;
  /* surface, per side (eval_surface) */
#pragma omp parallel for schedule(static)
  for (int s = 0; s < S; s++) {
    int L = o->left[s], R = o->right[s], lf = o->lsn[s], rf = o->rsn[s];
    double len = o->slen[s], nx = o->nx[s], ny = o->ny[s];
    double acc_l[NMAX * NPM], acc_r[NMAX * NPM];
    memset(acc_l, 0, sizeof acc_l);
    memset(acc_r, 0, sizeof acc_r);
    for (int j = 0; j < n1; j++) {
      double UL[NMAX] = {0, 0, 0, 0}, UR[NMAX] = {0, 0, 0, 0}, F[NMAX];
      double x = 0, y = 0;
      for (int i = 0; i < np; i++)
        for (int n = 0; n < N; n++) UL[n] += C[CI(n, i, L)] * o->E[lf][j][i];
      if (R < 0 || o->eq == EQ_ADV) face_xy(o, L, lf, j, &x, &y);
      if (R < 0) {
        ghost(o, R, UL, UR, x, y, t, nx, ny);
      } else {
        for (int i = 0; i < np; i++)
          for (int n = 0; n < N; n++) UR[n] += C[CI(n, i, R)] * o->E[rf][n1 - 1 - j][i];
      }
      riemann(o, UL, UR, nx, ny, x, y, F);
      for (int i = 0; i < np; i++)
        for (int n = 0; n < N; n++) {
          acc_l[n * NPM + i] += -len / 2 * (o->w1[j] * F[n] * o->E[lf][j][i]);
          acc_r[n * NPM + i] += len / 2 * (o->w1[j] * F[n] * o->E[rf][n1 - 1 - j][i]);
        }
    }
    for (int n = 0; n < N; n++)
      for (int i = 0; i < np; i++) {
        sl[(size_t)S * np * n + (size_t)i * S + s] = acc_l[n * NPM + i];
        sr[(size_t)S * np * n + (size_t)i * S + s] = acc_r[n * NPM + i];
      }
  }
  /* volume, per element (eval_volume) */
#pragma omp parallel for schedule(static)
  for (int e = 0; e < K; e++) {
    double acc[NMAX * NPM];
    double xr = o->xr[e], yr = o->yr[e], xs = o->xs[e], ys = o->ys[e];
    int flat = 0;
    for (int q = 0; q < nq && !flat; q++) {
      double U[NMAX] = {0, 0, 0, 0};
      for (int i = 0; i < np; i++)
        for (int n = 0; n < N; n++) U[n] += C[CI(n, i, e)] * o->B[q][i];
      if (!physical(o, U)) flat = 1;
    }
    if (flat) { /* the element's state becomes its mean (C_global write, euler.cu:98-108) */
#pragma omp atomic
      o->flattened++;
      for (int n = 0; n < N; n++)
        for (int i = 1; i < np; i++) C[CI(n, i, e)] = 0.;
    }
    memset(acc, 0, sizeof acc);
    for (int q = 0; q < nq; q++) {
      double U[NMAX] = {0, 0, 0, 0}, fx[NMAX], fy[NMAX];
      if (flat) {
        for (int n = 0; n < N; n++) U[n] = C[CI(n, 0, e)] * o->B[0][0];
      } else {
        for (int i = 0; i < np; i++)
          for (int n = 0; n < N; n++) U[n] += C[CI(n, i, e)] * o->B[q][i];
      }
      if (o->eq == EQ_ADV) { /* eval_flux with the velocity at the point */
        double x, y, vx, vy;
        vol_xy(o, e, q, &x, &y);
        velocity(o, x, y, &vx, &vy);
        fx[0] = vx * U[0];
        fy[0] = vy * U[0];
      } else {
        flux(o, U, fx, fy);
      }
      for (int i = 0; i < np; i++)
        for (int n = 0; n < N; n++)
          acc[n * NPM + i] += fx[n] * (o->GR[q][i] * ys - o->GS[q][i] * yr) +
                              fy[n] * (-o->GR[q][i] * xs + o->GS[q][i] * xr);
      /* source term (euler.cu:282-287 defines it zero); extension: the
       * shallow-water bed slope -g h grad b, with w_q J grad b from the
       * weighted gradient tables, projected on phi_i */
      if (o->bathy && o->eq == EQ_SW) {
        double br = 0, bs = 0;
        for (int i = 1; i < np; i++) {
          br += o->bathy[(size_t)i * K + e] * o->GR[q][i];
          bs += o->bathy[(size_t)i * K + e] * o->GS[q][i];
        }
        double gh = -o->g * U[0];
        double sx = gh * (ys * br - yr * bs), sy = gh * (xr * bs - xs * br);
        for (int i = 0; i < np; i++) {
          acc[1 * NPM + i] += sx * o->B[q][i];
          acc[2 * NPM + i] += sy * o->B[q][i];
        }
      }
    }
    for (int n = 0; n < N; n++)
      for (int i = 0; i < np; i++) vol[CI(n, i, e)] = acc[n * NPM + i];
  }
  /* assembly (eval_rhs) */
#pragma omp parallel for schedule(static)
  for (int e = 0; e < K; e++) {
    double jj = o->J[e];
    for (int n = 0; n < N; n++)
      for (int i = 0; i < np; i++) {
        double a = dt / jj * vol[CI(n, i, e)];
        for (int f = 0; f < 3; f++) {
          int s = o->es[f * K + e];
          size_t so = (size_t)S * np * n + (size_t)i * S + s;
          a += dt / jj * ((e == o->left[s]) ? sl[so] : sr[so]);
        }
        out[CI(n, i, e)] = a;
      }
  }
}

int or_rhs(or_solver *o, const double *C, double t, double *out) {
  size_t nd = (size_t)o->N * o->np * o->K;
  double *tmp = (double *)xmalloc(sizeof(double) * nd);
  memcpy(tmp, C, sizeof(double) * nd);
  o->flattened = 0;
  dg_operator(o, tmp, t, 1.0, out);
  free(tmp);
  return 0;
}

/* ---------------- limiter (limit_c, conserv_kernels.cu:640-720) ---------------- */
int or_limit(or_solver *o, double *C) {
  int K = o->K, np = o->np, N = o->N, n1 = o->n1, S = o->S;
  if (np < 3) return 0;
  double *mean = (double *)xmalloc(sizeof(double) * N * K);
  for (int n = 0; n < N; n++)
    for (int e = 0; e < K; e++) mean[n * K + e] = C[CI(n, 0, e)] * o->B[0][0];
  (void)S;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < K; e++) {
    int nb[3];
    for (int f = 0; f < 3; f++) {
      int s = o->es[f * K + e];
      nb[f] = (o->left[s] == e) ? o->right[s] : o->left[s];
      if (nb[f] < 0) nb[f] = e;
    }
    for (int n = 0; n < N; n++) {
      double Uc = mean[n * K + e], Umin = Uc, Umax = Uc;
      for (int f = 0; f < 3; f++) {
        double Ui = mean[n * K + nb[f]];
        Umin = (Ui < Umin) ? Ui : Umin;
        Umax = (Ui > Umax) ? Ui : Umax;
      }
      double amin = 1.;
      for (int j = 0; j < n1; j++)
        for (int f = 0; f < 3; f++) {
          double Ui = 0., a;
          for (int i = 0; i < np; i++) Ui += C[CI(n, i, e)] * o->E[f][j][i];
          /* the reference pairs the overshoot above the mean with the
           * distance to the minimum, and vice versa (conserv_kernels.cu:694-700) */
          if (Ui > Uc) a = dmin2(1., (Uc - Umin) / (Ui - Uc));
          else if (Ui < Uc) a = dmin2(1., (Uc - Umax) / (Ui - Uc));
          else a = 1;
          if (a < amin) amin = a;
        }
      if (amin < 0) amin = 0.;
      C[CI(n, 1, e)] *= amin;
      C[CI(n, 2, e)] *= amin;
      if (amin < 1.) /* extension for p > 1: drop the higher modes */
        for (int i = 3; i < np; i++) C[CI(n, i, e)] = 0.;
    }
  }
  free(mean);
  return 0;
}

/* ---------------- CFL (eval_global_lambda) ---------------- */
static double elem_lambda(const or_solver *o, const double *C, int e, double t) {
  int K = o->K, np = o->np;
  double U[NMAX];
  for (int n = 0; n < o->N; n++) U[n] = C[CI(n, 0, e)] * o->B[0][0];
  switch (o->eq) {
    case EQ_ADV: { /* advection.cu:157-183: the velocity at point n_q / 2 */
      double x, y, vx, vy;
      vol_xy(o, e, o->nq / 2, &x, &y);
      velocity(o, x, y, &vx, &vy);
      return sqrt(vx * vx + vy * vy);
    }
    case EQ_EULER: { /* euler.cu:248-277 */
      double p = (o->gamma - 1.) * (U[3] - (U[1] * U[1] + U[2] * U[2]) / 2. / U[0]);
      double c = sqrt(o->gamma * p / U[0]);
      double s = sqrt(U[1] * U[1] + U[2] * U[2]) / U[0];
      return s > 0 ? s + c : -s + c;
    }
    case EQ_SW: { /* shallowwater.cu:196-224 */
      double c = sqrt(U[0] * o->g);
      double s = sqrt(U[1] * U[1] + U[2] * U[2]) / U[0];
      return s > 0 ? s + c : -s + c;
    }
    default: /* maxwells.cu:174-185 */
      return fabs(1. / sqrt(o->eps * o->mu));
  }
  (void)t;
}

int or_lambda(or_solver *o, const double *C, double t, double *lam, double *min_r) {
  for (int e = 0; e < o->K; e++) lam[e] = elem_lambda(o, C, e, t);
  if (min_r) *min_r = o->min_r;
  return 0;
}

static double max_lambda(or_solver *o, const double *C, double t) {
  double ml = elem_lambda(o, C, 0, t);
  for (int e = 0; e < o->K; e++) {
    double l = elem_lambda(o, C, e, t);
    ml = (l > ml) ? l : ml;
  }
  return ml;
}

/* ---------------- time stepping ---------------- */
/* scheme 0: SSP-RK3 (extension); 1: RK4 and 2: midpoint RK2 as the
 * reference drives them, including its order of operations (t advanced
 * before the stages, limiter applied to each increment). endtime > 0 stops
 * at endtime (last step shortened). Returns the number of steps taken. */
int or_step(or_solver *o, double *C, int nsteps, int scheme, int limiter, double cfl,
            double fixed_dt, double endtime, double *tio) {
  size_t nd = (size_t)o->N * o->np * o->K;
  double *k1 = (double *)xmalloc(sizeof(double) * nd), *k2 = (double *)xmalloc(sizeof(double) * nd),
         *k3 = (double *)xmalloc(sizeof(double) * nd), *k4 = (double *)xmalloc(sizeof(double) * nd);
  double t = *tio;
  int step = 0;
  o->flattened = 0;
  if (limiter) or_limit(o, C);
  while (endtime > 0 ? (t < endtime) : (step < nsteps)) {
    double dt = fixed_dt > 0 ? fixed_dt : cfl * o->min_r / max_lambda(o, C, t) / (2. * o->p + 1.);
    if (!(dt == dt)) break;
    if (endtime > 0 && t + dt > endtime) dt = endtime - t;
    step++;
    if (scheme == 0) {
      /* u1 = u + dt L(u); u2 = 3/4 u + 1/4 (u1 + dt L(u1));
       * u = 1/3 u + 2/3 (u2 + dt L(u2)); stage times t, t + dt, t + dt/2.
       * Each stage output is limited, then flattened where its traces are
       * non-physical (the GPU's fused stage does both before the next stage
       * reads the output, so the state after a step is the flattened one) */
      dg_operator(o, C, t, dt, k1);
      for (size_t i = 0; i < nd; i++) k2[i] = C[i] + k1[i];
      if (limiter) or_limit(o, k2);
      o->flattened += flatten_pass(o, k2);
      dg_operator(o, k2, t + dt, dt, k1);
      for (size_t i = 0; i < nd; i++) k3[i] = 0.75 * C[i] + 0.25 * (k2[i] + k1[i]);
      if (limiter) or_limit(o, k3);
      o->flattened += flatten_pass(o, k3);
      dg_operator(o, k3, t + 0.5 * dt, dt, k1);
      for (size_t i = 0; i < nd; i++) C[i] = C[i] / 3. + 2. / 3. * (k3[i] + k1[i]);
      if (limiter) or_limit(o, C);
      o->flattened += flatten_pass(o, C);
      t += dt;
    } else if (scheme == 1) {
      t += dt;
      dg_operator(o, C, t, dt, k1);
      if (limiter) or_limit(o, k1);
      for (size_t i = 0; i < nd; i++) k2[i] = C[i] + 0.5 * k1[i];
      dg_operator(o, k2, t + 0.5 * dt, dt, k2);
      if (limiter) or_limit(o, k2);
      for (size_t i = 0; i < nd; i++) k3[i] = C[i] + 0.5 * k2[i];
      dg_operator(o, k3, t + 0.5 * dt, dt, k3);
      if (limiter) or_limit(o, k3);
      for (size_t i = 0; i < nd; i++) k4[i] = C[i] + k3[i];
      dg_operator(o, k4, t + dt, dt, k4);
      if (limiter) or_limit(o, k4);
      for (size_t i = 0; i < nd; i++) C[i] += k1[i] / 6. + k2[i] / 3. + k3[i] / 3. + k4[i] / 6.;
      if (limiter) or_limit(o, C);
    } else {
      t += dt;
      dg_operator(o, C, t, dt, k1);
      if (limiter) or_limit(o, k1);
      for (size_t i = 0; i < nd; i++) k1[i] = C[i] + 0.5 * k1[i];
      dg_operator(o, k1, t + 0.5 * dt, dt, k1);
      if (limiter) or_limit(o, k1);
      for (size_t i = 0; i < nd; i++) C[i] += k1[i];
      if (limiter) or_limit(o, C);
    }
  }
  *tio = t;
  free(k1);
  free(k2);
  free(k3);
  free(k4);
  return step;
}

/* ---------------- projection and error ---------------- */
int or_init(or_solver *o, double *C) {
  int K = o->K, np = o->np, N = o->N;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < K; e++)
    for (int i = 0; i < np; i++) {
      double U[NMAX] = {0, 0, 0, 0};
      for (int q = 0; q < o->nq; q++) {
        double x, y, u0[NMAX];
        vol_xy(o, e, q, &x, &y);
        init_state(o, u0, x, y);
        for (int n = 0; n < N; n++) U[n] += o->w[q] * u0[n] * o->B[q][i];
      }
      for (int n = 0; n < N; n++) C[CI(n, i, e)] = U[n];
    }
  return 0;
}

int or_l2err(or_solver *o, const double *C, double t, double *err2) {
  int K = o->K, np = o->np, N = o->N;
  for (int n = 0; n < N; n++) {
    double tot = 0;
    for (int e = 0; e < K; e++) {
      double ee = 0;
      for (int q = 0; q < o->nq; q++) {
        double x, y, u[NMAX], U = 0;
        vol_xy(o, e, q, &x, &y);
        for (int i = 0; i < np; i++) U += C[CI(n, i, e)] * o->B[q][i];
        exact_state(o, u, x, y, t);
        ee += o->w[q] * (u[n] - U) * (u[n] - U) * o->J[e];
      }
      tot += ee;
    }
    err2[n] = tot;
  }
  return 0;
}

/* ---------------- synthetic square meshes ----------------
 * The jittered square-split meshes of the benchmark configurations, built
 * without the product library (bench.py's reference arm times the oracle on
 * the same mesh the GPU runs).  Same construction, numbering and rounding as
 * the library's dg_mesh_square: nx x ny squares on [x0,x1]x[y0,y1], each cut
 * along its (0,0)-(1,1) diagonal into two CCW triangles; interior vertices
 * jittered by (2u - 1) jitter h with u from splitmix64(seed), x then y, row by
 * row; sides in first-visit order (element by element, faces 0, 1, 2; face k
 * joins vertices k and k+1, the .pmsh convention of genmesh.py), left = the
 * first element to visit a side; then boundary sides first by code -1..-4
 * (stable), interior sides after them.  bc = {left, right, bottom, top}: 0 is
 * periodic (paired), else a boundary code.  Arrays in .pmsh column order:
 * V[6][K], es[3][K], sxy[4][S], se[4][S].  tests/test_oracle_mesh.py checks
 * that the arrays equal the library's bit for bit. */
static unsigned long long sm64(unsigned long long *s) {
  unsigned long long z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double unif01(unsigned long long *s) { return (double)(sm64(s) >> 11) * 0x1.0p-53; }

int or_mesh_square_sizes(int nx, int ny, const int *bc, int *K, int *S) {
  const int px = bc[0] == 0, py = bc[2] == 0;
  if (nx < 1 || ny < 1) return 1;
  *K = 2 * nx * ny;
  *S = 3 * nx * ny + (px ? 0 : ny) + (py ? 0 : nx);
  return 0;
}

typedef struct {
  double x1, y1, x2, y2;
  int left, right, lsn, rsn, box;
} or_tmp_side;

int or_mesh_square(int nx, int ny, double x0, double x1, double y0, double y1, double jitter,
                   unsigned long long seed, const int *bc, double *V, int *es, double *sxy,
                   int *se) {
  const int px = bc[0] == 0 || bc[1] == 0, py = bc[2] == 0 || bc[3] == 0;
  int K, Sx;
  if ((bc[0] == 0) != (bc[1] == 0) || (bc[2] == 0) != (bc[3] == 0)) return 1;
  if (or_mesh_square_sizes(nx, ny, bc, &K, &Sx)) return 1;
  const double hx = (x1 - x0) / nx, hy = (y1 - y0) / ny;
  const int vx = nx + 1, vy = ny + 1;
  const unsigned long long nv = (unsigned long long)vx * vy;
  double *X = (double *)xmalloc(sizeof(double) * nv), *Y = (double *)xmalloc(sizeof(double) * nv);
  unsigned long long st = seed;
  for (int j = 0; j < vy; j++)
    for (int i = 0; i < vx; i++) {
      double x = x0 + i * hx, y = y0 + j * hy;
      if (i > 0 && i < nx && j > 0 && j < ny) {
        double ux = unif01(&st), uy = unif01(&st);
        x += (2 * ux - 1) * jitter * hx;
        y += (2 * uy - 1) * jitter * hy;
      }
      X[(size_t)j * vx + i] = x;
      Y[(size_t)j * vx + i] = y;
    }
  /* open-addressing table: side key -> side index */
  size_t cap = 1;
  while (cap < (size_t)2 * Sx + 16) cap <<= 1;
  unsigned long long *keys = (unsigned long long *)xmalloc(sizeof(unsigned long long) * cap);
  int *vals = (int *)xmalloc(sizeof(int) * cap);
  or_tmp_side *sd = (or_tmp_side *)xmalloc(sizeof(or_tmp_side) * (size_t)Sx);
  int ns = 0, e = 0, rc = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const int tri[2][3][2] = {{{i, j}, {i + 1, j}, {i + 1, j + 1}},
                                {{i, j}, {i + 1, j + 1}, {i, j + 1}}};
      for (int t = 0; t < 2; t++, e++) {
        for (int k = 0; k < 3; k++) {
          size_t gv = (size_t)tri[t][k][1] * vx + tri[t][k][0];
          V[(size_t)(2 * k) * K + e] = X[gv];
          V[(size_t)(2 * k + 1) * K + e] = Y[gv];
        }
        for (int k = 0; k < 3; k++) {
          const int a = k, b = (k + 1) % 3;
          const int ia = tri[t][a][0], ja = tri[t][a][1], ib = tri[t][b][0], jb = tri[t][b][1];
          long long ka = (long long)(py ? ja % ny : ja) * vx + (px ? ia % nx : ia);
          long long kb = (long long)(py ? jb % ny : jb) * vx + (px ? ib % nx : ib);
          const unsigned long long key =
              (unsigned long long)(ka < kb ? ka : kb) * nv + (unsigned long long)(ka < kb ? kb : ka) + 1;
          size_t h = (size_t)((key * 0x9E3779B97F4A7C15ull) >> 17) & (cap - 1);
          while (keys[h] && keys[h] != key) h = (h + 1) & (cap - 1);
          if (!keys[h]) {
            if (ns >= Sx) { rc = 2; goto done; }
            or_tmp_side *s = &sd[ns];
            s->x1 = V[(size_t)(2 * a) * K + e];
            s->y1 = V[(size_t)(2 * a + 1) * K + e];
            s->x2 = V[(size_t)(2 * b) * K + e];
            s->y2 = V[(size_t)(2 * b + 1) * K + e];
            s->left = e;
            s->lsn = k;
            s->right = -1;
            s->rsn = 0;
            s->box = -1;
            if (ia == 0 && ib == 0) s->box = 0;
            else if (ia == nx && ib == nx) s->box = 1;
            else if (ja == 0 && jb == 0) s->box = 2;
            else if (ja == ny && jb == ny) s->box = 3;
            if (s->box >= 0 && bc[s->box] == 0) s->box = -1;
            keys[h] = key;
            vals[h] = ns;
            es[(size_t)k * K + e] = ns++;
          } else {
            or_tmp_side *s = &sd[vals[h]];
            s->right = e;
            s->rsn = k;
            es[(size_t)k * K + e] = vals[h];
          }
        }
      }
    }
  if (ns != Sx) { rc = 2; goto done; }
  for (int n = 0; n < ns; n++)
    if (sd[n].right < 0) {
      if (sd[n].box < 0) { rc = 3; goto done; }
      sd[n].right = bc[sd[n].box];
    }
  {
    /* stable order: codes -1, -2, -3, -4, then interior sides */
    int *newidx = (int *)xmalloc(sizeof(int) * (size_t)ns);
    int pos = 0;
    for (int rank = 1; rank <= 5; rank++)
      for (int n = 0; n < ns; n++) {
        const int r = sd[n].right < 0 ? -sd[n].right : 5;
        if (r != rank) continue;
        newidx[n] = pos;
        sxy[pos] = sd[n].x1;
        sxy[(size_t)ns + pos] = sd[n].y1;
        sxy[2 * (size_t)ns + pos] = sd[n].x2;
        sxy[3 * (size_t)ns + pos] = sd[n].y2;
        se[pos] = sd[n].left;
        se[(size_t)ns + pos] = sd[n].right;
        se[2 * (size_t)ns + pos] = sd[n].lsn;
        se[3 * (size_t)ns + pos] = sd[n].rsn;
        pos++;
      }
    for (size_t q = 0; q < (size_t)3 * K; q++) es[q] = newidx[es[q]];
    free(newidx);
  }
done:
  free(X);
  free(Y);
  free(keys);
  free(vals);
  free(sd);
  return rc;
}
