/* ref_driver.cpp -- runs the reference's own DG kernels on the host.
 *
 * Test infrastructure only: it produces golden vectors for the oracle and the
 * GPU parity tests.  It is compiled once per equation with the reference's
 * equation module included unmodified (REF_EQ_FILE, e.g. "euler/euler.cu"),
 * which pulls in the reference's conserv_kernels.cu, quadrature.cu and
 * basis.cu through ../main.cu (see main.cu beside this directory).
 *
 * What is the reference's code here: every kernel body (eval_surface,
 * eval_volume, limit_c, init_conditions, eval_error_L2, eval_global_lambda,
 * the preval_* geometry kernels), the equation modules, the quadrature
 * tables, basis tabulation (preval_basis) and the basis coefficients.
 * What this file restates: the per-problem plugin functions (U0, U_inflow,
 * U_outflow, U_reflection, U_exact, get_GAMMA, get_velocity, get_mu,
 * get_eps -- each a short formula, cited below), the quadrature selection of
 * main.cu:124-194, the eval_rhs gather of time_integrator.cu:26-101 and the
 * RK4 / RK2 step loops of time_integrator.cu:139-433 and :511-717, and a
 * zero source_term for the modules that do not define one (the GPU build of
 * those modules fails to link without it).
 *
 * I/O: argv[1] = input file, argv[2] = output file, both raw little-endian.
 * Input: int32 hdr[16], double prm[16], then mesh arrays in the .pmsh order,
 * then the state C in the reference layout [var][mode][elem].
 */
#include "shim.h"
#include REF_EQ_FILE

#include <vector>
#include <string>

shim_dim3 threadIdx, blockIdx, blockDim;

/* ------------------------------------------------------------------ */
/* problem plugin (runtime-selected)                                   */
/* ------------------------------------------------------------------ */
enum {
  PB_NONE = 0,
  PB_ADV_SINE = 1,
  PB_ADV_LINEAR = 2,
  PB_EULER_VORTEX = 3,
  PB_EULER_RIEMANN4 = 4,
  PB_EULER_SUPERSONIC = 5,
  PB_SW_HUMP = 6,
  PB_SW_TEST = 7,
  PB_MAXWELL_PLANE = 8,
  PB_EULER_AIRFOIL = 12,
  PB_ADV_SQUAREHILL = 13,
  PB_ADV_ROTATINGHILL = 14,
  PB_ADV_SPIN = 15,
  PB_MAXWELL_CMIRROR = 16,
  PB_MAXWELL_WSCATTER = 17,
  PB_EULER_PULSE = 18
};
static int g_problem = PB_NONE;
static double g_prm[16];
/* prm layout: 0 t, 1 gamma, 2 ax, 3 ay, 4 mu, 5 eps, 6 (unused), 7 cfl,
 * 8..15 problem parameters */

/* rotatinghill.cu:58-67 (its U_inflow): the hill at the point rotated back */
static double rotated_hill(double A, double x0, double y0, double r, double x, double y,
                           double t) {
  double c = cos(2 * M_PI * t), s = sin(2 * M_PI * t);
  return A * exp(-(pow(x * c + y * s - x0, 2) + pow(-x * s + y * c - y0, 2)) / (2 * r * r));
}

/* tube.cu:52-97 with a short series in prm 8 t0, then (amp, omega, phase) x 2 */
static void pulse_state(double *U, double t) {
  double GAM = g_prm[1], p = 1.0;
  t += g_prm[8];
  for (int k = 0; k < 2; k++) p += g_prm[9 + 3 * k] * cos(g_prm[10 + 3 * k] * t + g_prm[11 + 3 * k]);
  double rho = GAM * pow(p, (1. / GAM)), u = ((p - 1) / GAM), v = 0.0;
  U[0] = rho;
  U[1] = u * rho;
  U[2] = v * rho;
  U[3] = 0.5 * rho * (u * u + v * v) + (p / (GAM - 1.));
}

static void exact_state(double *U, double x, double y, double t) {
  switch (g_problem) {
    case PB_EULER_AIRFOIL: {
      /* airfoil.cu:22-27 (MACH .98, ALPHA 5) */
      double GAM = g_prm[1], MACH = 0.98, ALPHA = 5.;
      U[0] = GAM;
      U[1] = U[0] * MACH * cos(M_PI * (ALPHA / 180.));
      U[2] = U[0] * MACH * sin(M_PI * (ALPHA / 180.));
      U[3] = 0.5 * U[0] * MACH * MACH + 1. / (GAM - 1.0);
      break;
    }
    case PB_EULER_PULSE:
      pulse_state(U, t);
      break;
    case PB_ADV_SQUAREHILL: {
      /* squarehill.cu:22-30, translated by the velocity */
      double xs = x - g_prm[2] * t, ys = y - g_prm[3] * t;
      U[0] = (xs < -.2 && xs > -.8 && ys < .1 && ys > -.5) ? 1. : 0.;
      break;
    }
    case PB_ADV_ROTATINGHILL:
      U[0] = rotated_hill(5., 0.2, 0.0, 0.15, x, y, t);
      break;
    case PB_ADV_SPIN:
      /* spin.cu:22-30 */
      U[0] = exp(-((x - .5) * (x - .5) + (y - .5) * (y - .5)) / (2 * .1 * .1));
      break;
    case PB_ADV_SINE: {
      /* u0 = sin(2 pi x) sin(2 pi y) translated by a t on the unit square */
      double xs = x - g_prm[2] * t, ys = y - g_prm[3] * t;
      U[0] = sin(2 * M_PI * xs) * sin(2 * M_PI * ys);
      break;
    }
    case PB_ADV_LINEAR:
      /* advection/exact/exact.cu:25-27: u = x - y, steady under a = (1, 1) */
      U[0] = x - y;
      break;
    case PB_EULER_VORTEX: {
      /* isentropic vortex, prm 8 beta, 9 x0, 10 y0, 11 uinf, 12 vinf,
       * 13 period L (centre advected and wrapped into the periodic box) */
      double gam = g_prm[1], beta = g_prm[8], L = g_prm[13];
      double xc = g_prm[9] + g_prm[11] * t, yc = g_prm[10] + g_prm[12] * t;
      double dx = x - xc, dy = y - yc;
      if (L > 0) {
        dx -= L * floor(dx / L + 0.5);
        dy -= L * floor(dy / L + 0.5);
      }
      double r2 = dx * dx + dy * dy;
      double e = exp(0.5 * (1 - r2));
      double u = g_prm[11] - beta / (2 * M_PI) * e * dy;
      double v = g_prm[12] + beta / (2 * M_PI) * e * dx;
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
      double gam = g_prm[1];
      double rho, u, v, p;
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
    case PB_EULER_SUPERSONIC: {
      /* euler/supersonic/supersonic.cu:27-37 (GAMMA 1.4, MACH 2.25) */
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
      /* still water hump: prm 8 h0, 9 A, 10 sigma, 11 x0, 12 y0 */
      double dx = x - g_prm[11], dy = y - g_prm[12], s = g_prm[10];
      U[0] = g_prm[8] + g_prm[9] * exp(-(dx * dx + dy * dy) / (s * s));
      U[1] = 0;
      U[2] = 0;
      break;
    }
    case PB_SW_TEST: {
      /* shallowwater/test/test.cu:25-35 */
      double x0 = 0.5, y0 = 0.5, r = 0.1;
      U[0] = 10 + exp(-(pow(x - x0, 2) + pow(y - y0, 2)) / (2 * r * r));
      U[1] = 0.;
      U[2] = 0.;
      break;
    }
    case PB_MAXWELL_PLANE: {
      /* plane wave along x: Ez = sin(2 pi (x - c t)), Hy = sqrt(eps/mu) Ez */
      double mu = g_prm[4], eps = g_prm[5], c = 1 / sqrt(mu * eps);
      double ez = sin(2 * M_PI * (x - c * t));
      U[0] = 0;
      U[1] = sqrt(eps / mu) * ez;
      U[2] = ez;
      break;
    }
    default:
      for (int n = 0; n < N; n++) U[n] = 0; /* the module's variable count */
  }
}

/* the problem plugin entry points the reference modules call */
void U0(double *U, double x, double y) {
  if (g_problem == PB_EULER_PULSE) { /* tube.cu:25-45: at rest */
    double GAM = g_prm[1];
    U[0] = GAM;
    U[1] = U[2] = 0.;
    U[3] = 1. / (GAM - 1.0);
    return;
  }
  exact_state(U, x, y, 0.0);
}
void U_exact(double *U, double x, double y, double t) { exact_state(U, x, y, t); }
void U_inflow(double *U, double x, double y, double t) {
  switch (g_problem) {
    case PB_ADV_SQUAREHILL: /* squarehill.cu:43-45 */
    case PB_ADV_SPIN:       /* spin.cu:43-46 */
      U[0] = 0;
      return;
    case PB_MAXWELL_CMIRROR: /* cmirror.cu:38-47 */
      U[0] = 0.;
      U[1] = 0.;
      U[2] = t <= 1. / 20 ? 2 * sin(M_PI * 20 * t) : 0.;
      return;
    case PB_MAXWELL_WSCATTER: /* wscatter.cu:38-50 (f = 1) */
      U[0] = 0.;
      U[1] = 0.;
      U[2] = (y < .15 && y > -.15 && t < 1. / 2.) ? sin(M_PI * 2 * t) : 0.;
      return;
    default:
      exact_state(U, x, y, t);
  }
}
void U_outflow(double *U, double x, double y, double t) {
  /* exact.cu:50-52 and test.cu:53-55 leave the ghost state untouched;
   * supersonic.cu:55-57 uses U0; Euler problems here use the exact state */
  switch (g_problem) {
    case PB_EULER_VORTEX:
    case PB_EULER_RIEMANN4:
    case PB_EULER_SUPERSONIC:
    case PB_EULER_AIRFOIL: /* airfoil.cu:55-57: U0 */
    case PB_EULER_PULSE:   /* tube.cu:107-109: U_inflow */
      exact_state(U, x, y, t);
      break;
    case PB_MAXWELL_PLANE:
    case PB_MAXWELL_CMIRROR:  /* cmirror.cu:55-59 */
    case PB_MAXWELL_WSCATTER: /* wscatter.cu:58-63 */
      U[0] = U[1] = U[2] = 0;
      break;
    default:
      break;
  }
}
void U_reflection(double *U_left, double *U_right, double x, double y, double t, double nx,
                  double ny) {
  switch (g_problem) {
    case PB_EULER_SUPERSONIC: {
      /* supersonic.cu:65-87: curved-wall normal from the position, ghost
       * momentum = tangential projection of the interior momentum */
      double Nx, Ny, dot;
      U_right[0] = U_left[0];
      U_right[3] = U_left[3];
      dot = sqrt(x * x + y * y);
      Nx = x / dot;
      Ny = y / dot;
      if (Nx * nx + Ny * ny < 0) {
        Nx *= -1;
        Ny *= -1;
      }
      U_right[1] = (U_left[1] * Ny - U_left[2] * Nx) * Ny;
      U_right[2] = -(U_left[1] * Ny - U_left[2] * Nx) * Nx;
      break;
    }
    case PB_EULER_AIRFOIL: {
      /* airfoil.cu:63-100: normal part reversed, tangential part kept */
      double u_N, u_T;
      U_right[0] = U_left[0];
      U_right[3] = U_left[3];
      u_N = -(nx * U_left[1] + ny * U_left[2]);
      u_T = ny * U_left[1] - nx * U_left[2];
      U_right[1] = u_N * nx + u_T * ny;
      U_right[2] = u_N * ny - u_T * nx;
      break;
    }
    case PB_EULER_PULSE: /* tube.cu:121-135: normal reflection */
    case PB_EULER_VORTEX:
    case PB_EULER_RIEMANN4: {
      /* slip wall: mirror the momentum about the face */
      double dot = U_left[1] * nx + U_left[2] * ny;
      U_right[0] = U_left[0];
      U_right[1] = U_left[1] - 2 * dot * nx;
      U_right[2] = U_left[2] - 2 * dot * ny;
      U_right[3] = U_left[3];
      break;
    }
    case PB_SW_HUMP:
    case PB_SW_TEST: {
      /* test.cu:63-77 */
      double dot = U_left[1] * nx + U_left[2] * ny;
      U_right[0] = U_left[0];
      U_right[1] = U_left[1] - 2 * dot * nx;
      U_right[2] = U_left[2] - 2 * dot * ny;
      break;
    }
    case PB_MAXWELL_PLANE:
    case PB_MAXWELL_CMIRROR:
    case PB_MAXWELL_WSCATTER: {
      /* maxwells/cmirror/cmirror.cu:63-77: E_z kept, normal H kept,
       * tangential H reversed */
      double dot = U_left[0] * nx + U_left[1] * ny;
      U_right[2] = U_left[2];
      U_right[0] = -U_left[0] + 2 * dot * nx;
      U_right[1] = -U_left[1] + 2 * dot * ny;
      break;
    }
    default:
      break; /* advection: no reflecting walls, ghost stays zero */
  }
}

#if defined(REF_EULER)
double get_GAMMA() { return g_prm[1]; }
#endif
#if defined(REF_ADVECTION) || defined(REF_SHALLOWWATER)
void get_velocity(double *A, double x, double y, double t) {
  if (g_problem == PB_ADV_ROTATINGHILL) { /* rotatinghill.cu:37-40 */
    const double PI = 3.14159265358979323;
    A[0] = -2 * PI * y;
    A[1] = 2 * PI * x;
    return;
  }
  if (g_problem == PB_ADV_SPIN) { /* spin.cu:37-40 */
    const double PI = 3.14159;
    A[0] = -2 * PI * y;
    A[1] = 2 * PI * x;
    return;
  }
  A[0] = g_prm[2];
  A[1] = g_prm[3];
}
#endif
#if defined(REF_MAXWELL)
double get_mu() { return g_prm[4]; }
double get_eps() { return g_prm[5]; }
#endif
#if !defined(REF_EULER)
/* zero source for modules that do not define one */
void source_term(double *S, double *U, double *V, double t, int j) {
  for (int n = 0; n < N; n++) S[n] = 0;
}
#endif

int limiter = 0;
int time_integrator = 1;

/* ------------------------------------------------------------------ */
/* cudaMemcpyToSymbol by name                                          */
/* ------------------------------------------------------------------ */
int cudaMemcpyToSymbol(const char *name, void *src, size_t bytes) {
  struct {
    const char *n;
    void *p;
  } tab[] = {{"N", &N},
             {"n_p", &n_p},
             {"num_elem", &num_elem},
             {"num_sides", &num_sides},
             {"n_quad", &n_quad},
             {"n_quad1d", &n_quad1d},
             {"basis", basis},
             {"basis_grad_x", basis_grad_x},
             {"basis_grad_y", basis_grad_y},
             {"basis_side", basis_side},
             {"basis_vertex", basis_vertex},
             {"w", w},
             {"w_oned", w_oned},
             {"r1", r1},
             {"r2", r2},
             {"r_oned", r_oned}};
  for (auto &e : tab)
    if (!strcmp(e.n, name)) {
      memcpy(e.p, src, bytes);
      return 0;
    }
  fprintf(stderr, "unknown symbol %s\n", name);
  exit(3);
}

/* quadrature selection, restating main.cu:148-193 */
static void select_quadrature(int n, std::vector<double> &rr1, std::vector<double> &rr2,
                              std::vector<double> &ww, std::vector<double> &sr,
                              std::vector<double> &w1, int *nq, int *nq1) {
  static const int nq_tab[6] = {1, 3, 6, 12, 16, 25};
  *nq = nq_tab[n];
  *nq1 = n + 1;
  const double *q2 = quad_2d[n > 0 ? 2 * n - 1 : 0];
  for (int i = 0; i < *nq; i++) {
    rr1.push_back(q2[3 * i]);
    rr2.push_back(q2[3 * i + 1]);
    ww.push_back(q2[3 * i + 2] / 2.);
  }
  for (int i = 0; i < *nq1; i++) {
    sr.push_back(quad_1d[n][2 * i]);
    w1.push_back(quad_1d[n][2 * i + 1]);
  }
}

template <class F>
static void grid(int n, F f) {
  blockDim.x = 1;
  blockIdx.x = 0;
  for (int i = 0; i < n; i++) {
    threadIdx.x = (unsigned)i;
    f();
  }
}

struct Mesh {
  int K, S;
  std::vector<double> V[6];
  std::vector<int> es[3];
  std::vector<double> sx1, sy1, sx2, sy2;
  std::vector<int> le, re, lsn, rsn;
  std::vector<double> J, xr, yr, xs, ys, slen, Nx, Ny;
  double min_r;
};

static void geometry(Mesh &m) {
  int K = m.K, S = m.S;
  m.J.assign(K, 0);
  m.xr.assign(K, 0);
  m.yr.assign(K, 0);
  m.xs.assign(K, 0);
  m.ys.assign(K, 0);
  m.slen.assign(S, 0);
  m.Nx.assign(S, 0);
  m.Ny.assign(S, 0);
  double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
         *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
  grid(K, [&] { preval_inscribed_circles(m.J.data(), V1x, V1y, V2x, V2y, V3x, V3y); });
  m.min_r = m.J[0];
  for (int i = 1; i < K; i++) m.min_r = (m.J[i] < m.min_r) ? m.J[i] : m.min_r;
  grid(K, [&] { preval_jacobian(m.J.data(), V1x, V1y, V2x, V2y, V3x, V3y); });
  grid(S, [&] {
    preval_side_length(m.slen.data(), m.sx1.data(), m.sy1.data(), m.sx2.data(), m.sy2.data());
  });
  grid(S, [&] {
    preval_normals(m.Nx.data(), m.Ny.data(), m.sx1.data(), m.sy1.data(), m.sx2.data(),
                   m.sy2.data(), V1x, V1y, V2x, V2y, V3x, V3y, m.lsn.data());
  });
  grid(S, [&] {
    preval_normals_direction(m.Nx.data(), m.Ny.data(), V1x, V1y, V2x, V2y, V3x, V3y,
                             m.le.data(), m.lsn.data());
  });
  grid(K, [&] {
    preval_partials(V1x, V1y, V2x, V2y, V3x, V3y, m.xr.data(), m.yr.data(), m.xs.data(),
                    m.ys.data());
  });
}

/* k = dt / J (vol + surf of the three sides), restating time_integrator.cu:26-101 */
static void gather_rhs(const Mesh &m, int NN, int np, const double *vol, const double *sl,
                       const double *sr, double dt, double *out) {
  int K = m.K, S = m.S;
  for (int e = 0; e < K; e++) {
    double jj = m.J[e];
    for (int n = 0; n < NN; n++)
      for (int i = 0; i < np; i++) {
        size_t o = (size_t)K * np * n + (size_t)i * K + e;
        double acc = 0.;
        acc += dt / jj * vol[o];
        for (int f = 0; f < 3; f++) {
          int s = m.es[f][e];
          size_t so = (size_t)S * np * n + (size_t)i * S + s;
          acc += dt / jj * ((e == m.le[s]) ? sl[so] : sr[so]);
        }
        out[o] = acc;
      }
  }
}

struct Work {
  std::vector<double> vol, sl, sr;
};

static void dg_operator(Mesh &m, int NN, int np, double *C, double t, double dt, double *out,
                        Work &w) {
  double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
         *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
  w.vol.assign((size_t)NN * np * m.K, 0);
  w.sl.assign((size_t)NN * np * m.S, 0);
  w.sr.assign((size_t)NN * np * m.S, 0);
  grid(m.S, [&] {
    eval_surface(C, w.sl.data(), w.sr.data(), m.slen.data(), V1x, V1y, V2x, V2y, V3x, V3y,
                 m.le.data(), m.re.data(), m.lsn.data(), m.rsn.data(), m.Nx.data(),
                 m.Ny.data(), t);
  });
  grid(m.K, [&] {
    eval_volume(C, w.vol.data(), m.xr.data(), m.yr.data(), m.xs.data(), m.ys.data(), V1x, V1y,
                V2x, V2y, V3x, V3y, m.J.data(), t);
  });
  gather_rhs(m, NN, np, w.vol.data(), w.sl.data(), w.sr.data(), dt, out);
}

static void limit(Mesh &m, double *C) {
  grid(m.K, [&] {
    limit_c(C, m.es[0].data(), m.es[1].data(), m.es[2].data(), m.le.data(), m.re.data());
  });
}

static double max_lambda(Mesh &m, double *C, double t) {
  std::vector<double> lam(m.K);
  double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
         *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
  grid(m.K, [&] { eval_global_lambda(C, lam.data(), V1x, V1y, V2x, V2y, V3x, V3y, t); });
  double ml = lam[0];
  for (int i = 0; i < m.K; i++) ml = (lam[i] > ml) ? lam[i] : ml;
  return ml;
}

static void rd(FILE *f, void *p, size_t bytes) {
  if (bytes && fread(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: ref_driver in.bin out.bin\n");
    return 1;
  }
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 1;
  int hdr[16];
  rd(fi, hdr, sizeof hdr);
  rd(fi, g_prm, sizeof g_prm);
  int p = hdr[1], mode = hdr[4], nsteps = hdr[5];
  g_problem = hdr[7];
  limiter = hdr[6];
  int rk = hdr[8];
  Mesh m;
  m.K = hdr[2];
  m.S = hdr[3];
  for (int k = 0; k < 6; k++) {
    m.V[k].resize(m.K);
    rd(fi, m.V[k].data(), 8 * m.K);
  }
  for (int k = 0; k < 3; k++) {
    m.es[k].resize(m.K);
    rd(fi, m.es[k].data(), 4 * m.K);
  }
  std::vector<double> *sc[4] = {&m.sx1, &m.sy1, &m.sx2, &m.sy2};
  for (auto v : sc) {
    v->resize(m.S);
    rd(fi, v->data(), 8 * m.S);
  }
  std::vector<int> *si[4] = {&m.le, &m.re, &m.lsn, &m.rsn};
  for (auto v : si) {
    v->resize(m.S);
    rd(fi, v->data(), 4 * m.S);
  }
  int NN = local_N;
  int np = (p + 1) * (p + 2) / 2;
  std::vector<double> C((size_t)NN * np * m.K);
  rd(fi, C.data(), 8 * C.size());
  fclose(fi);

  std::vector<double> rr1, rr2, ww, sr, w1;
  int nq, nq1;
  select_quadrature(p, rr1, rr2, ww, sr, w1, &nq, &nq1);
  set_N(NN);
  set_n_p(np);
  set_num_elem(m.K);
  set_num_sides(m.S);
  set_n_quad(nq);
  set_n_quad1d(nq1);
  preval_basis(rr1.data(), rr2.data(), sr.data(), ww.data(), w1.data(), nq, nq1, np);
  geometry(m);

  std::vector<double> out;
  double t = g_prm[0];
  Work wk;
  size_t ndof = (size_t)NN * np * m.K;
  if (mode == 0) { /* right-hand side du/dt */
    out.resize(ndof);
    dg_operator(m, NN, np, C.data(), t, 1.0, out.data(), wk);
  } else if (mode == 1) { /* nsteps of the reference RK loop */
    double cfl = g_prm[7];
    std::vector<double> k1(ndof), k2(ndof), k3(ndof), k4(ndof);
    if (limiter) limit(m, C.data());
    for (int step = 0; step < nsteps; step++) {
      double ml = max_lambda(m, C.data(), t);
      double dt = cfl * m.min_r / ml / (2. * p + 1.);
      t += dt; /* the reference advances t before the stages */
      if (rk == 4) {
        dg_operator(m, NN, np, C.data(), t, dt, k1.data(), wk);
        if (limiter) limit(m, k1.data());
        for (size_t i = 0; i < ndof; i++) k2[i] = C[i] + 0.5 * k1[i];
        dg_operator(m, NN, np, k2.data(), t + 0.5 * dt, dt, k2.data(), wk);
        if (limiter) limit(m, k2.data());
        for (size_t i = 0; i < ndof; i++) k3[i] = C[i] + 0.5 * k2[i];
        dg_operator(m, NN, np, k3.data(), t + 0.5 * dt, dt, k3.data(), wk);
        if (limiter) limit(m, k3.data());
        for (size_t i = 0; i < ndof; i++) k4[i] = C[i] + 1.0 * k3[i];
        dg_operator(m, NN, np, k4.data(), t + dt, dt, k4.data(), wk);
        if (limiter) limit(m, k4.data());
        for (size_t i = 0; i < ndof; i++)
          C[i] += k1[i] / 6. + k2[i] / 3. + k3[i] / 3. + k4[i] / 6.;
        if (limiter) limit(m, C.data());
      } else { /* midpoint RK2 */
        dg_operator(m, NN, np, C.data(), t, dt, k1.data(), wk);
        if (limiter) limit(m, k1.data());
        for (size_t i = 0; i < ndof; i++) k1[i] = C[i] + 0.5 * k1[i];
        dg_operator(m, NN, np, k1.data(), t + 0.5 * dt, dt, k1.data(), wk);
        if (limiter) limit(m, k1.data());
        for (size_t i = 0; i < ndof; i++) C[i] += k1[i];
        if (limiter) limit(m, C.data());
      }
    }
    out = C;
    out.push_back(t);
  } else if (mode == 2) { /* limiter only */
    limit(m, C.data());
    out = C;
  } else if (mode == 3) { /* L2 projection of the initial condition */
    out.assign((size_t)4 * np * m.K, 0); /* init_conditions writes 4 vars */
    double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
           *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
    grid(m.K, [&] { init_conditions(out.data(), m.J.data(), V1x, V1y, V2x, V2y, V3x, V3y); });
    out.resize(ndof);
  } else if (mode == 4) { /* basis / quadrature tabulation */
    auto app = [&](const double *a, int n) { out.insert(out.end(), a, a + n); };
    app(basis, np * nq);
    app(basis_grad_x, np * nq);
    app(basis_grad_y, np * nq);
    app(basis_side, 3 * np * nq1);
    app(basis_vertex, 3 * np);
    app(w, nq);
    app(r1, nq);
    app(r2, nq);
    app(r_oned, nq1);
    app(w_oned, nq1);
  } else if (mode == 5) { /* per-variable L2 error^2 at time t */
    std::vector<double> err(m.K);
    double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
           *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
    for (int n = 0; n < NN; n++) {
      grid(m.K, [&] {
        eval_error_L2(C.data(), err.data(), V1x, V1y, V2x, V2y, V3x, V3y, m.J.data(), n, t);
      });
      double tot = 0;
      for (int e = 0; e < m.K; e++) tot += err[e];
      out.push_back(tot);
    }
  } else if (mode == 6) { /* CFL inputs: per-element wave speed, min diameter */
    std::vector<double> lam(m.K);
    double *V1x = m.V[0].data(), *V1y = m.V[1].data(), *V2x = m.V[2].data(),
           *V2y = m.V[3].data(), *V3x = m.V[4].data(), *V3y = m.V[5].data();
    grid(m.K, [&] { eval_global_lambda(C.data(), lam.data(), V1x, V1y, V2x, V2y, V3x, V3y, t); });
    out = lam;
    out.push_back(m.min_r);
  } else {
    fprintf(stderr, "bad mode\n");
    return 1;
  }
  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 1;
  fwrite(out.data(), 8, out.size(), fo);
  fclose(fo);
  return 0;
}
