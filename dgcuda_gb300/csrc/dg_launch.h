// dg_launch.h -- host-side launch interface of the sm_103a kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "dg_tables_data.h"

namespace dg {

// equation / problem parameters (kernel parameter)
constexpr int kMaxSeries = 16;  // terms of an inflow pressure series
struct EqP {
  double gamma, g, ax, ay, mu, eps;
  int problem;
  int field;        // 1: advection velocity a(x, y) = (ax, ay) + agrad (x, y)
  double prm[8];
  double agrad[4];  // d a_x/dx, d a_x/dy, d a_y/dx, d a_y/dy
  double amax;      // field: the largest element speed (the CFL wave speed)
  // inflow pressure series p(t) = 1 + sum_k amp_k cos(omega_k (t + t0) + phase_k)
  double ser_t0;
  double ser[kMaxSeries][3];  // amp, omega, phase
  int nser, pad;
};

// Device-resident mesh in internal (space-filling-curve) element order.
// Per-element arrays are rows of length Kp (K rounded up to 32) so every
// row of the [var][mode][elem] state starts 256-byte aligned.
struct DevMesh {
  int K = 0, Kp = 0, S = 0, Sb = 0;
  double *geo = nullptr;  // 5 rows: xr, yr, xs, ys, 1/J
  double *vtx = nullptr;  // 6 rows: V1x, V1y, V2x, V2y, V3x, V3y
  double *jac = nullptr;  // 1 row: J
  int *esd = nullptr;     // 3 rows: side index * 2 + (element is the side's right element)
  int *nbr = nullptr;     // 3 rows: neighbour across face f (itself at a boundary)
  int4 *side = nullptr;   // S: left, right (>= 0) or boundary code (< 0), left face, right face
  double *sgeo = nullptr; // 3 rows of S: nx, ny, len / 2
  double *bxy = nullptr;  // 4 rows of Sb: start and end vertex of the left face (boundary sides)
  int *perm = nullptr;    // K: internal index -> caller's (.pmsh) index
  double *bathy = nullptr; // shallow water bed modes [mode][Kp], null = flat
};

// device scalars used by graph-captured steps
struct DevScalars {
  double t;         // current time
  double dt;        // current step
  double one;       // 1.0 (dt of a plain right-hand side)
  double zero;      // 0.0
  double dmin;      // minimum inscribed diameter
  double cfl;       // CFL number
  double fixed_dt;  // > 0: use it instead of the CFL step
  double endtime;   // > 0: shorten the last step to land here
  unsigned long long lam_bits;  // max wave speed (non-negative double as bits)
  long long steps;  // steps taken with dt > 0
  int status;       // 0 ok, 4 NaN or non-positive CFL step
  int last;         // 1 when this step was shortened to land on endtime
};

struct Ctx {
  cudaStream_t st = nullptr;
  DevMesh m;
  int p = 1, eq = 0, N = 1, np = 3;
  int blk = 128;                  // block size of the stage kernels (autotuned)
  const EqP *q = nullptr;         // host copy of the equation parameters
  const void *tab = nullptr;      // host Tab<p> image
  double *T = nullptr;            // traces [elem][face][j][var]
  double *Fh = nullptr;           // face fluxes [side][j][var], scaled by len/2 * w_j
  double *Fs = nullptr;           // per-side sums of Fh over the edge points [side][var]
  double *M = nullptr;            // means of the stage output [var][Kp] (fused limiter)
  DevScalars *ds = nullptr;       // device scalars
  const void *oz = nullptr;       // tensor-core tables of order p (null: FP64 contractions)
};

// one problem of a batched ensemble (device resident)
struct BatchProb {
  int p, K, Kp, S, Sb, pad;
  double *U, *W, *T, *Fh;
  double *Fs, *M;  // per-side flux sums and output means (fused limiter; null elsewhere)
  const double *geo;
  const int *esd, *nbr;
  const int4 *side;
  const double *sgeo, *bxy, *bathy;
  const double *vtx;
  DevScalars *ds;
  EqP q;
};

struct BatchLaunch {
  cudaStream_t st = nullptr;
  const void *tabs = nullptr;       // BatchTabs image (Tab<1>, Tab<2>, Tab<3>)
  BatchProb *probs = nullptr;       // device array
  int nprob = 0, blk = 128, limiter = 0;
  int fused = 0;  // limiter in the element epilogue (face_fs, means, element_lim)
  // element blocks of the element stage: group g = 2 (p - 1) + (K >= 16384)
  // holds the members of order p on small (0) or large (1) meshes, in blocks
  // of blk_g[g] elements, the blocks [eblk_g[g], eblk_g[g + 1])
  const int *eblk2prob = nullptr, *eblk0 = nullptr;
  const int *ublk2prob = nullptr, *ublk0 = nullptr;  // element blocks of size blk (trace, limit)
  const int *sblk2prob = nullptr, *sblk0 = nullptr;  // side blocks of size blk
  const int *lblk2prob = nullptr, *lblk0 = nullptr;  // element blocks of 128 (wave speed)
  int neblk = 0, nublk = 0, nsblk = 0, nlblk = 0;
  static constexpr int kGroups = 6;
  int eblk_g[kGroups + 1] = {0, 0, 0, 0, 0, 0, 0};
  int blk_g[kGroups] = {128, 128, 128, 128, 128, 128};
  // the groups' element launches are independent: the first non-empty group
  // runs on st, every other one on gst[g], forked from st by `fork` and
  // joined back by join[g], so a captured step holds them as parallel
  // branches (fork null: all on st)
  cudaStream_t gst[kGroups] = {};
  cudaEvent_t fork = nullptr, join[kGroups] = {};
};

struct BatchOps {
  void (*trace)(const BatchLaunch &);
  void (*face)(const BatchLaunch &, double tcoef);
  void (*element)(const BatchLaunch &, int stage);
  void (*limit_tr)(const BatchLaunch &, int stage);
  void (*lambda)(const BatchLaunch &);
  // the stage with the limiter in the element epilogue, as Ops::face_fs,
  // means and element_lim (null where an equation has none)
  void (*face_fs)(const BatchLaunch &, double tcoef);
  void (*means)(const BatchLaunch &, int stage);
  void (*element_lim)(const BatchLaunch &, int stage);
};

const BatchOps &batch_ops_advection();
const BatchOps &batch_ops_euler();
const BatchOps &batch_ops_shallow_water();
const BatchOps &batch_ops_maxwell();
size_t batch_tabs_bytes();
// copies the Tab<1>, Tab<2>, Tab<3> images into a BatchTabs image
void build_batch_tabs(const void *t1, const void *t2, const void *t3, void *dst);
void launch_batch_reset_lambda(cudaStream_t st, BatchProb *probs, int n);
void launch_batch_compute_dt(cudaStream_t st, BatchProb *probs, int n);
void launch_batch_advance_t(cudaStream_t st, BatchProb *probs, int n);

struct Ops {
  // edge traces of u; flattens (in u) any element with a non-physical trace
  void (*trace)(const Ctx &, double *u);
  // numerical flux on every side at time *t + tcoef * *dt
  void (*face)(const Ctx &, const double *t, double tcoef);
  // out = ca * un + cb * us + cc * dt * (du/dt of us); out may alias us or un
  void (*element)(const Ctx &, double *us, const double *un, double *out, double ca, double cb,
                  double cc, const double *dtp);
  // Barth-Jespersen limiter in place
  void (*limit)(const Ctx &, double *u);
  // max cell-mean wave speed into ds->lam_bits (atomic max)
  void (*lambda)(const Ctx &, const double *u);
  // L2 projection of the problem's initial condition
  void (*init)(const Ctx &, double *u);
  // per-block partial sums of the squared L2 error, [nblocks][N]; returns nblocks
  int (*l2err)(const Ctx &, const double *u, double t, double *partial);
  // element() that also leaves the traces of `out` in T (the next stage's
  // k_trace, fused); check = apply the positivity rule to them here
  void (*element_tr)(const Ctx &, double *us, const double *un, double *out, double ca,
                     double cb, double cc, const double *dtp, int check);
  // limit() reading and updating the traces in T (after element_tr)
  void (*limit_tr)(const Ctx &, double *u);
  // values of variable var at the three vertices, rows of Kp: out[v][elem]
  void (*vertex)(const Ctx &, const double *u, int var, int mode, double t, double *out);
  // a stage with the limiter in the element stage's epilogue (null where an
  // equation has none): face() that also leaves the per-side flux sums in
  // Fs; the means of the stage output into M (k_means); element_tr() that
  // limits its output (Barth-Jespersen with the neighbours' means from M),
  // applies the positivity rule to the limited traces and writes both
  void (*face_fs)(const Ctx &, const double *t, double tcoef);
  void (*means)(const Ctx &, double *us, const double *un, double ca, double cb, double cc,
                const double *dtp);
  void (*element_lim)(const Ctx &, double *us, const double *un, double *out, double ca,
                      double cb, double cc, const double *dtp);
};

const Ops &ops_advection();
const Ops &ops_euler();
// tensor-core element stage (Euler, p = 1..4): table image size, builder
// from the host Tab<p> image, and the per-device kernel attribute
size_t oz_tabs_bytes();
bool oz_build_tabs(int p, const void *tabimg, void *out, double *dense = nullptr);
cudaError_t oz_prepare_euler(int p);
const Ops &ops_shallow_water();
const Ops &ops_maxwell();

// per-order table image (Tab<p>) built from the generic tabulation
size_t tab_bytes(int p);
void build_tab(int p, const dg_order_tables &src, void *dst);

// helpers (dg_kernels_common.cu)
void launch_permute_in(cudaStream_t st, const double *user, double *internal, const int *perm,
                       int rows, int K, int Kp);
void launch_permute_in_cmp(cudaStream_t st, const double *user, double *internal,
                           const int *perm, int rows, int K, int Kp, int *changed);
void launch_permute_out(cudaStream_t st, const double *internal, double *user, const int *perm,
                        int rows, int K, int Kp);
// y = a * x + b * y over n entries (RK4 / RK2 combinations), dt-scaled when dts != 0
void launch_axpby(cudaStream_t st, int n, double a, const double *x, double b, double *y);
// z = x + a * y
void launch_xpay(cudaStream_t st, int n, const double *x, double a, const double *y, double *z);
void launch_rk4_final(cudaStream_t st, int n, double *c, const double *k1, const double *k2,
                      const double *k3, const double *k4);
// dt from lam_bits (or fixed_dt), clamped to endtime; order p for the (2p+1)
void launch_compute_dt(cudaStream_t st, DevScalars *ds, int p);
void launch_reset_lambda(cudaStream_t st, DevScalars *ds);
void launch_advance_t(cudaStream_t st, DevScalars *ds);

// ---- shallow-water tangent-linear / adjoint operators (dg_adjoint.cu) ----
// (c.T must hold the traces of the linearisation state us; c.Fh carries the
// tangent fluxes between tl_face and tl_element)
bool lin_supported(int p);
bool lin_trace(const Ctx &c, const double *u, const double *scale, double sc, double *Tv);
bool tl_face(const Ctx &c, const double *Tv, double *dFh);
bool adj_face(const Ctx &c, const double *Tbar, double *UbL, double *UbR);
bool tl_element(const Ctx &c, const double *us, const double *dus, const double *db,
                const double *dun, double *dout, double ca, double cb, double ccdt);
bool adj_element(const Ctx &c, const double *us, const double *obar, double *ubar_s,
                 double *bbar, const double *UbL, const double *UbR, double cb, double ccdt);
void launch_sample(cudaStream_t st, const double *u, const int *el, const double *phi, int nrec,
                   int np, int Kp, double *out);
void launch_sample_adj(cudaStream_t st, double *ubar, const int *el, const double *phi, int nrec,
                       int np, int Kp, const double *sbar);

// what other files need to launch a solver's kernels
struct SolverView {
  int device = 0;
  cudaStream_t st = nullptr;
  const Ops *ops = nullptr;
  Ctx ctx;
  int N = 0, np = 0, p = 0, K = 0, S = 0;
};

}  // namespace dg

struct dg_solver;
namespace dg {
SolverView solver_view(dg_solver *s);
}  // namespace dg
