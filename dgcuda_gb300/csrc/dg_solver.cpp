// dg_solver.cpp -- the solver object behind the C ABI (include/dg.h).
//
// Replaces the reference's host driver (run_dgcuda, init_gpu, set_quadrature,
// the preval_* set-up and the time integrators; src/2d/conservation/main.cu,
// time_integrator.cu) with one object per problem that owns its device
// buffers and CUDA stream: no globals, so many solvers coexist.  Geometry is
// computed here in FP64 on the host (the reference computes it on the GPU
// with float sqrtf, conserv_kernels.cu:412-585) and uploaded once.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "dg_device.cuh"
#include "dg_internal.h"
#include "dg_launch.h"

using dg::fail;

namespace {

struct ProfEvent {
  int kind;
  cudaEvent_t a, b;
};
const char *kKindName[] = {"trace", "face", "element", "limit", "cfl", "rk", "means"};
constexpr int kKinds = 7;

}  // namespace

struct dg_solver {
  int device = 0;
  cudaStream_t st = nullptr;
  dg_equation eq = DG_EULER;
  int p = 1, N = 4, np = 3, K = 0, S = 0;
  dg_params prm{};
  dg::EqP q{};
  dg_order_tables tables{};
  std::vector<char> tabimg;
  dg::DevMesh m;
  dg::Ctx ctx;
  const dg::Ops *ops = nullptr;
  double *U = nullptr, *W = nullptr, *k[4] = {nullptr, nullptr, nullptr, nullptr};
  double *ubuf = nullptr, *partial = nullptr, *T = nullptr, *Fh = nullptr, *vbuf = nullptr;
  double *Fs = nullptr, *M = nullptr;  // side-flux sums and output means (fused limiter)
  double *bathy = nullptr;        // bed modes (shallow water), internal order
  double *lin_tv = nullptr, *lin_f0 = nullptr, *lin_f1 = nullptr;  // adjoint work
  bool has_inout_bc = false;      // a side with an inflow or outflow code
  void *oz = nullptr;             // tensor-core tables (Euler, p = 1..4)
  int *flag = nullptr;            // device flag of put_state
  // host transfers of the state: a copy stream and one event per chunk of
  // rows, so that the permutation of one chunk overlaps the copy of the next
  cudaStream_t cst = nullptr;
  std::vector<cudaEvent_t> cev;
  bool tensor = true;             // use them in the fused element stage
  // T holds the traces of U as the last fused SSP-RK3 stage left them (and U
  // is already limited): the next dg_step continues without recomputing
  // them, so a run split over several calls is the uninterrupted run
  bool tr_valid = false;
  std::vector<double> mesh_v;     // vertices per element, .pmsh order (bed projection)
  dg::DevScalars *ds = nullptr;
  double dmin = 0;
  size_t ndof_p = 0;  // N * np * Kp
  // graphs per (scheme, limiter)
  std::map<int, cudaGraphExec_t> graphs;
  std::map<int, long long> graph_launches;
  bool profiling = false;
  std::vector<ProfEvent> pending;
  std::vector<cudaEvent_t> pool;
  long long prof_n[kKinds] = {0};
  double prof_ms[kKinds] = {0};
  long long launches = 0;
  std::vector<void *> allocs;
};

namespace {

dg_status cuda_fail(cudaError_t e, const char *what) {
  return fail(DG_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                           \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
  } while (0)

template <class T>
dg_status dalloc(dg_solver *s, T **ptr, size_t count) {
  void *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  s->allocs.push_back(p);
  *ptr = static_cast<T *>(p);
  return DG_OK;
}

template <class T>
dg_status upload(dg_solver *s, T **ptr, const std::vector<T> &h) {
  dg_status st = dalloc(s, ptr, h.size());
  if (st != DG_OK) return st;
  if (!h.empty()) CK(cudaMemcpy(*ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return DG_OK;
}

const dg::Ops *ops_for(dg_equation eq) {
  switch (eq) {
    case DG_ADVECTION: return &dg::ops_advection();
    case DG_EULER: return &dg::ops_euler();
    case DG_SHALLOW_WATER: return &dg::ops_shallow_water();
    case DG_MAXWELL: return &dg::ops_maxwell();
  }
  return nullptr;
}

// ---- profiling: events around each launch when enabled ----
cudaEvent_t take_event(dg_solver *s) {
  if (!s->pool.empty()) {
    cudaEvent_t e = s->pool.back();
    s->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

template <class F>
void run(dg_solver *s, int kind, F &&f) {
  if (s->profiling) {
    ProfEvent pe{kind, take_event(s), take_event(s)};
    cudaEventRecord(pe.a, s->st);
    f();
    cudaEventRecord(pe.b, s->st);
    s->pending.push_back(pe);
  } else {
    f();
  }
  s->launches++;
}

void collect_profile(dg_solver *s) {
  if (s->pending.empty()) return;
  cudaStreamSynchronize(s->st);
  for (auto &pe : s->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, pe.a, pe.b);
    s->prof_n[pe.kind]++;
    s->prof_ms[pe.kind] += ms;
    s->pool.push_back(pe.a);
    s->pool.push_back(pe.b);
  }
  s->pending.clear();
}

enum { K_TRACE = 0, K_FACE = 1, K_ELEMENT = 2, K_LIMIT = 3, K_CFL = 4, K_RK = 5, K_MEANS = 6 };

// one RK stage of the DG operator: out = ca*un + cb*us + cc*dt*L(us).
// With the tensor-core contractions on, the element stage is the one the
// fused SSP-RK3 step runs (k_element_oz; the traces of `out` it also leaves
// in T are not used, and no positivity rule is applied to them), so dg_rhs
// and the RK4 / RK2 loops evaluate the operator the SSP-RK3 step evaluates.
void stage(dg_solver *s, double *us, const double *un, double *out, double ca, double cb,
           double cc, double tcoef, const double *dtp) {
  run(s, K_TRACE, [&] { s->ops->trace(s->ctx, us); });
  run(s, K_FACE, [&] { s->ops->face(s->ctx, &s->ds->t, tcoef); });
  if (s->ctx.oz)
    run(s, K_ELEMENT, [&] { s->ops->element_tr(s->ctx, us, un, out, ca, cb, cc, dtp, 0); });
  else
    run(s, K_ELEMENT, [&] { s->ops->element(s->ctx, us, un, out, ca, cb, cc, dtp); });
}

void limit(dg_solver *s, double *u) {
  if (s->prm.limiter && s->np >= 3) run(s, K_LIMIT, [&] { s->ops->limit(s->ctx, u); });
}

// a stage whose input traces are already in T (left by the previous stage);
// it leaves the traces of `out` -- limited when the limiter is on -- in T.
// With the limiter on (Euler), the limiter runs in the element stage's
// epilogue: the face kernel also sums each side's fluxes, and
// k_means turns the sums into the output's cell means, which the element
// stage needs for its neighbours' bounds; no separate limiter pass.
void fused_stage(dg_solver *s, double *us, const double *un, double *out, double ca, double cb,
                 double cc, double tcoef, const double *dtp) {
  const bool lim = s->prm.limiter && s->np >= 3;
  if (lim && s->ops->element_lim && s->ctx.M) {
    run(s, K_FACE, [&] { s->ops->face_fs(s->ctx, &s->ds->t, tcoef); });
    run(s, K_MEANS, [&] { s->ops->means(s->ctx, us, un, ca, cb, cc, dtp); });
    run(s, K_ELEMENT, [&] { s->ops->element_lim(s->ctx, us, un, out, ca, cb, cc, dtp); });
    return;
  }
  run(s, K_FACE, [&] { s->ops->face(s->ctx, &s->ds->t, tcoef); });
  run(s, K_ELEMENT,
      [&] { s->ops->element_tr(s->ctx, us, un, out, ca, cb, cc, dtp, lim ? 0 : 1); });
  if (lim) run(s, K_LIMIT, [&] { s->ops->limit_tr(s->ctx, out); });
}

void cfl(dg_solver *s) {
  run(s, K_CFL, [&] { dg::launch_reset_lambda(s->st, s->ds); });
  run(s, K_CFL, [&] { s->ops->lambda(s->ctx, s->U); });
  run(s, K_CFL, [&] { dg::launch_compute_dt(s->st, s->ds, s->p); });
}

// one time step of `scheme` on s->U (launch sequence, capturable)
void one_step(dg_solver *s, int scheme) {
  const int n = (int)s->ndof_p;
  const double *dt = &s->ds->dt;
  cfl(s);
  if (scheme == DG_SSP_RK3) {
    // u1 = u + dt L(u); u2 = 3/4 u + 1/4 (u1 + dt L(u1)); u = 1/3 u + 2/3 (u2 + dt L(u2));
    // T holds the traces of u on entry (run_steps) and of the new u on exit
    fused_stage(s, s->U, nullptr, s->W, 0.0, 1.0, 1.0, 0.0, dt);
    fused_stage(s, s->W, s->U, s->W, 0.75, 0.25, 0.25, 1.0, dt);
    fused_stage(s, s->W, s->U, s->U, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5, dt);
    run(s, K_CFL, [&] { dg::launch_advance_t(s->st, s->ds); });
  } else if (scheme == DG_RK4) {
    // time_integrator.cu:198-400: t advanced first, limiter on each increment
    run(s, K_CFL, [&] { dg::launch_advance_t(s->st, s->ds); });
    double **k = s->k;
    stage(s, s->U, nullptr, k[0], 0, 0, 1, 0.0, dt);
    limit(s, k[0]);
    run(s, K_RK, [&] { dg::launch_xpay(s->st, n, s->U, 0.5, k[0], k[1]); });
    stage(s, k[1], nullptr, k[1], 0, 0, 1, 0.5, dt);
    limit(s, k[1]);
    run(s, K_RK, [&] { dg::launch_xpay(s->st, n, s->U, 0.5, k[1], k[2]); });
    stage(s, k[2], nullptr, k[2], 0, 0, 1, 0.5, dt);
    limit(s, k[2]);
    run(s, K_RK, [&] { dg::launch_xpay(s->st, n, s->U, 1.0, k[2], k[3]); });
    stage(s, k[3], nullptr, k[3], 0, 0, 1, 1.0, dt);
    limit(s, k[3]);
    run(s, K_RK, [&] { dg::launch_rk4_final(s->st, n, s->U, k[0], k[1], k[2], k[3]); });
    limit(s, s->U);
  } else {
    // midpoint RK2, time_integrator.cu:557-690
    run(s, K_CFL, [&] { dg::launch_advance_t(s->st, s->ds); });
    double **k = s->k;
    stage(s, s->U, nullptr, k[0], 0, 0, 1, 0.0, dt);
    limit(s, k[0]);
    run(s, K_RK, [&] { dg::launch_xpay(s->st, n, s->U, 0.5, k[0], k[0]); });
    stage(s, k[0], nullptr, k[0], 0, 0, 1, 0.5, dt);
    limit(s, k[0]);
    run(s, K_RK, [&] { dg::launch_xpay(s->st, n, s->U, 1.0, k[0], s->U); });
    limit(s, s->U);
  }
}

dg_status ensure_rk_buffers(dg_solver *s) {
  if (s->k[0]) return DG_OK;
  for (int i = 0; i < 4; i++) {
    dg_status st = dalloc(s, &s->k[i], s->ndof_p);
    if (st != DG_OK) return st;
    CK(cudaMemset(s->k[i], 0, s->ndof_p * sizeof(double)));
  }
  return DG_OK;
}

// the CFL wave speed of an advection velocity field: the largest speed over
// the elements, each taken at its middle quadrature point x = x1 + (x2 - x1)
// r + (x3 - x1) s (eval_global_lambda, advection.cu:157-183); the field does
// not change in time, so this is found once
static void field_refresh(dg_solver *s) {
  dg::EqP &q = s->q;
  q.field = (q.agrad[0] != 0 || q.agrad[1] != 0 || q.agrad[2] != 0 || q.agrad[3] != 0) ? 1 : 0;
  q.amax = 0.0;
  if (!q.field) return;
  const int k = s->tables.n_q / 2;
  const double r = s->tables.r[k], sv = s->tables.s[k];
  for (int e = 0; e < s->K; e++) {
    const double *v = &s->mesh_v[(size_t)6 * e];
    const double x = std::fma(v[2] - v[0], r, std::fma(v[4] - v[0], sv, v[0]));
    const double y = std::fma(v[3] - v[1], r, std::fma(v[5] - v[1], sv, v[1]));
    const double vx = std::fma(q.agrad[0], x, std::fma(q.agrad[1], y, q.ax));
    const double vy = std::fma(q.agrad[2], x, std::fma(q.agrad[3], y, q.ay));
    q.amax = std::max(q.amax, std::sqrt(std::fma(vx, vx, vy * vy)));
  }
}

void drop_graphs(dg_solver *s) {
  for (auto &g : s->graphs) cudaGraphExecDestroy(g.second);
  s->graphs.clear();
  s->graph_launches.clear();
}

// (re)builds the tensor-core tables from the current basis tables and
// points the fused element stage at them (or back at the FP64 kernel)
dg_status oz_refresh(dg_solver *s) {
  s->ctx.oz = nullptr;
  if (s->eq != DG_EULER || s->p < 1 || s->p > 4) return DG_OK;
  // at p = 1 (3 modes, 3 area points) the FP64 kernel is the faster one:
  // the tensor path is built but off until asked for
  if (!s->oz) s->tensor = s->p >= 2;
  std::vector<char> img(dg::oz_tabs_bytes());
  if (!dg::oz_build_tabs(s->p, s->tabimg.data(), img.data()))
    return fail(DG_UNSUPPORTED, "no tensor-core tables for this order");
  if (!s->oz) {
    dg_status st = dalloc(s, reinterpret_cast<char **>(&s->oz), img.size());
    if (st != DG_OK) return st;
    CK(dg::oz_prepare_euler(s->p));
  }
  CK(cudaMemcpy(s->oz, img.data(), img.size(), cudaMemcpyHostToDevice));
  if (s->tensor) s->ctx.oz = s->oz;
  return DG_OK;
}

dg_status get_graph(dg_solver *s, int scheme, cudaGraphExec_t *out) {
  int key = scheme * 2 + (s->prm.limiter ? 1 : 0);
  auto it = s->graphs.find(key);
  if (it != s->graphs.end()) {
    *out = it->second;
    return DG_OK;
  }
  cudaGraph_t g;
  long long before = s->launches;
  CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
  one_step(s, scheme);
  cudaError_t e = cudaStreamEndCapture(s->st, &g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  s->launches = before;
  s->graph_launches[key] = 0;
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  s->graph_launches[key] = (long long)nn;
  cudaGraphExec_t ex;
  e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  s->graphs[key] = ex;
  *out = ex;
  return DG_OK;
}

dg_status set_scalar(dg_solver *s, size_t offset, const void *v, size_t bytes) {
  CK(cudaMemcpyAsync(reinterpret_cast<char *>(s->ds) + offset, v, bytes, cudaMemcpyHostToDevice,
                     s->st));
  CK(cudaStreamSynchronize(s->st));
  return DG_OK;
}

dg_status read_scalars(dg_solver *s, dg::DevScalars *h) {
  CK(cudaMemcpyAsync(h, s->ds, sizeof *h, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return DG_OK;
}

dg_status sync_check(dg_solver *s) {
  cudaError_t e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return DG_OK;
}

// prepare device scalars for a run, then run nsteps (or until endtime)
dg_status run_steps(dg_solver *s, int nsteps, int scheme, double fixed_dt, double endtime,
                    double *t, int *taken) {
  if (scheme < 0 || scheme > 2) return fail(DG_BAD_ARG, "unknown scheme");
  if (scheme != DG_SSP_RK3) {
    dg_status st = ensure_rk_buffers(s);
    if (st != DG_OK) return st;
  }
  dg::DevScalars h{};
  h.t = *t;
  h.dt = 0;
  h.one = 1.0;
  h.zero = 0.0;
  h.dmin = s->dmin;
  h.cfl = s->prm.cfl;
  h.fixed_dt = fixed_dt;
  h.endtime = endtime;
  dg_status st = set_scalar(s, 0, &h, sizeof h);
  if (st != DG_OK) return st;
  const bool resume = scheme == DG_SSP_RK3 && s->tr_valid;
  s->tr_valid = false;
  if (!resume) {
    // the reference limits once before its step loop (time_integrator.cu:178-184)
    limit(s, s->U);
    // SSP-RK3 stages find their input traces in T (fused_stage)
    if (scheme == DG_SSP_RK3) run(s, K_TRACE, [&] { s->ops->trace(s->ctx, s->U); });
  }
  cudaGraphExec_t g = nullptr;
  if (!s->profiling) {
    st = get_graph(s, scheme, &g);
    if (st != DG_OK) return st;
  }
  int key = scheme * 2 + (s->prm.limiter ? 1 : 0);
  auto launch_one = [&]() -> dg_status {
    if (g) {
      CK(cudaGraphLaunch(g, s->st));
      s->launches += s->graph_launches[key];
    } else {
      one_step(s, scheme);
    }
    return DG_OK;
  };
  if (endtime > 0) {
    const int batch = 8;
    for (;;) {
      for (int i = 0; i < batch; i++) {
        st = launch_one();
        if (st != DG_OK) return st;
      }
      collect_profile(s);
      st = read_scalars(s, &h);
      if (st != DG_OK) return st;
      if (h.status) break;
      if (h.t >= endtime) break;
    }
  } else {
    for (int i = 0; i < nsteps; i++) {
      st = launch_one();
      if (st != DG_OK) return st;
      if (s->profiling && (i % 16) == 15) collect_profile(s);
    }
    collect_profile(s);
    st = read_scalars(s, &h);
    if (st != DG_OK) return st;
  }
  st = sync_check(s);
  if (st != DG_OK) return st;
  *t = h.t;
  if (taken) *taken = (int)h.steps;
  if (h.status == 4) return fail(DG_NAN, "time step is NaN or not positive (non-finite state?)");
  s->tr_valid = scheme == DG_SSP_RK3;
  return DG_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" dg_status dg_solver_create(const dg_mesh *mesh, dg_equation eq, int p,
                                      const dg_params *prm, int device, dg_solver **out) {
  if (!mesh || !out) return fail(DG_BAD_ARG, "null argument");
  *out = nullptr;
  if (p < 0 || p > DG_PMAX) return fail(DG_BAD_ARG, "order p must be 0..5");
  if (eq < DG_ADVECTION || eq > DG_MAXWELL) return fail(DG_BAD_ARG, "unknown equation");
  dg_status vs = dg::validate_mesh(*mesh);
  if (vs != DG_OK) return vs;
  dg_params P;
  if (prm) P = *prm;
  else dg_params_default(&P);
  if (P.problem < 0 || P.problem > DG_PB_EULER_PULSE) return fail(DG_BAD_ARG, "unknown problem");
  if (!(P.cfl > 0)) return fail(DG_BAD_ARG, "cfl must be positive");
  if (eq == DG_EULER && !(P.gamma > 1)) return fail(DG_BAD_ARG, "gamma must be > 1");
  if (eq == DG_SHALLOW_WATER && !(P.gravity > 0)) return fail(DG_BAD_ARG, "gravity must be > 0");
  if (eq == DG_MAXWELL && !(P.mu > 0 && P.eps > 0)) return fail(DG_BAD_ARG, "mu, eps must be > 0");
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) return fail(DG_CUDA_ERROR, "no CUDA device available");
  if (device < 0 || device >= ndev) return fail(DG_BAD_ARG, "device ordinal out of range");
  CK(cudaSetDevice(device));

  dg_solver *s = new dg_solver();
  s->device = device;
  s->eq = eq;
  s->p = p;
  s->prm = P;
  static const int NV[4] = {1, 4, 3, 3};
  s->N = NV[eq];
  s->np = dg::np_of(p);
  s->K = mesh->K;
  s->S = mesh->S;
  s->ops = ops_for(eq);
  s->q.gamma = P.gamma;
  s->q.g = P.gravity;
  s->q.ax = P.ax;
  s->q.ay = P.ay;
  s->q.mu = P.mu;
  s->q.eps = P.eps;
  s->q.problem = P.problem;
  for (int i = 0; i < 8; i++) s->q.prm[i] = P.prm[i];
  if (P.problem == DG_PB_ADV_ROTATINGHILL || P.problem == DG_PB_ADV_SPIN) {
    // the solid rotation (-w y, w x) of rotatinghill.cu:37-40 / spin.cu:37-40
    const double w = P.problem == DG_PB_ADV_SPIN ? dg::kRotSpin : dg::kRotHill;
    s->q.ax = s->q.ay = 0.0;
    s->q.agrad[1] = -w;
    s->q.agrad[2] = w;
  }
  s->tables = DG_TABLES[p];
  s->tabimg.resize(dg::tab_bytes(p));
  dg::build_tab(p, s->tables, s->tabimg.data());

  auto bail = [&](dg_status st) {
    dg_solver_destroy(s);
    return st;
  };
  if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaStreamCreate failed"));

  // ---- internal element order: Morton curve of the centroids ----
  const int K = mesh->K, S = mesh->S;
  const int Kp = (K + 31) / 32 * 32;
  std::vector<int> perm = dg::sfc_order(*mesh);  // new -> old
  std::vector<int> inv(K);
  for (int e = 0; e < K; e++) inv[perm[e]] = e;
  // ---- internal side order: boundary sides first (by code), then interior by first element ----
  std::vector<int> sorder(S);
  std::iota(sorder.begin(), sorder.end(), 0);
  auto skey = [&](int sd) -> long long {
    int r = mesh->right[sd];
    if (r < 0) return (long long)(-r) * 0 - 10 + (-r);  // -9..-6: boundary, by code
    int a = inv[mesh->left[sd]], b = inv[r];
    return (long long)std::min(a, b) * 4 + 3;
  };
  std::stable_sort(sorder.begin(), sorder.end(), [&](int a, int b) { return skey(a) < skey(b); });
  std::vector<int> snew(S);
  for (int i = 0; i < S; i++) snew[sorder[i]] = i;
  int Sb = 0;
  while (Sb < S && mesh->right[sorder[Sb]] < 0) Sb++;
  for (int i = 0; i < Sb; i++) {
    int code = mesh->right[sorder[i]];
    if (code == DG_BC_INFLOW || code == DG_BC_OUTFLOW) s->has_inout_bc = true;
  }

  // ---- element arrays ----
  std::vector<double> geo((size_t)5 * Kp, 0.0), vtx((size_t)6 * Kp, 0.0), jac(Kp, 1.0);
  std::vector<int> esd((size_t)3 * Kp, 0), nbr((size_t)3 * Kp, 0);
  double dmin = 1e300;
  for (int e = 0; e < K; e++) {
    int o = perm[e];
    double x1 = mesh->V[0][o], y1 = mesh->V[1][o], x2 = mesh->V[2][o], y2 = mesh->V[3][o],
           x3 = mesh->V[4][o], y3 = mesh->V[5][o];
    double J = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);  // preval_jacobian
    geo[e] = x2 - x1;                                           // preval_partials
    geo[(size_t)Kp + e] = y2 - y1;
    geo[2 * (size_t)Kp + e] = x3 - x1;
    geo[3 * (size_t)Kp + e] = y3 - y1;
    geo[4 * (size_t)Kp + e] = 1.0 / J;
    jac[e] = J;
    const double v6[6] = {x1, y1, x2, y2, x3, y3};
    for (int k = 0; k < 6; k++) vtx[(size_t)k * Kp + e] = v6[k];
    // inscribed-circle diameter (preval_inscribed_circles, conserv_kernels.cu:428-445)
    double a = std::sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
    double b = std::sqrt((x2 - x3) * (x2 - x3) + (y2 - y3) * (y2 - y3));
    double c = std::sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3));
    double kk = 0.5 * (a + b + c);
    double d = 2 * std::sqrt(kk * (kk - a) * (kk - b) * (kk - c)) / kk;
    dmin = std::min(dmin, d);
    for (int f = 0; f < 3; f++) {
      int so = mesh->es[f][o];
      bool right = !(mesh->left[so] == o && mesh->lsn[so] == f);
      esd[(size_t)f * Kp + e] = snew[so] * 2 + (right ? 1 : 0);
      int other = right ? mesh->left[so] : mesh->right[so];
      nbr[(size_t)f * Kp + e] = other >= 0 ? inv[other] : e;
    }
  }
  s->dmin = dmin;
  s->mesh_v.resize((size_t)6 * K);
  for (int o = 0; o < K; o++)
    for (int k = 0; k < 6; k++) s->mesh_v[(size_t)6 * o + k] = mesh->V[k][o];
  field_refresh(s);
  // ---- side arrays ----
  std::vector<int4> side(S);
  std::vector<double> sgeo((size_t)3 * S), bxy((size_t)4 * std::max(Sb, 1));
  for (int i = 0; i < S; i++) {
    int so = sorder[i];
    int L = mesh->left[so], R = mesh->right[so], lf = mesh->lsn[so];
    side[i] = make_int4(inv[L], R >= 0 ? inv[R] : R, lf, R >= 0 ? mesh->rsn[so] : 0);
    // normal from the side's vertices, pointed away from the left element's
    // third vertex (preval_normals + preval_normals_direction, :481-569)
    double dx = mesh->sx2[so] - mesh->sx1[so], dy = mesh->sy2[so] - mesh->sy1[so];
    double len = std::sqrt(dx * dx + dy * dy);
    double nx = -dy / len, ny = dx / len;
    int va = lf, vb = (lf + 1) % 3, vc = (lf + 2) % 3;
    double ax = mesh->V[2 * va][L], ay = mesh->V[2 * va + 1][L];
    double bx = mesh->V[2 * vb][L], by = mesh->V[2 * vb + 1][L];
    double cx = mesh->V[2 * vc][L], cy = mesh->V[2 * vc + 1][L];
    double mx = (ax + bx) / 2., my = (ay + by) / 2.;
    if (nx * (cx - mx) + ny * (cy - my) > 0) {
      nx = -nx;
      ny = -ny;
    }
    sgeo[i] = nx;
    sgeo[(size_t)S + i] = ny;
    sgeo[2 * (size_t)S + i] = len / 2;
    if (i < Sb) {
      bxy[i] = ax;
      bxy[(size_t)Sb + i] = ay;
      bxy[2 * (size_t)Sb + i] = bx;
      bxy[3 * (size_t)Sb + i] = by;
    }
  }

  // ---- device buffers ----
  dg::DevMesh &m = s->m;
  m.K = K;
  m.Kp = Kp;
  m.S = S;
  m.Sb = Sb;
  dg_status st;
  if ((st = upload(s, &m.geo, geo)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.vtx, vtx)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.jac, jac)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.esd, esd)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.nbr, nbr)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.side, side)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.sgeo, sgeo)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.bxy, bxy)) != DG_OK) return bail(st);
  if ((st = upload(s, &m.perm, perm)) != DG_OK) return bail(st);
  s->ndof_p = (size_t)s->N * s->np * Kp;
  size_t nuser = (size_t)s->N * s->np * K;
  const int n1 = p + 1;
  if ((st = dalloc(s, &s->U, s->ndof_p)) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->W, s->ndof_p)) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->ubuf, nuser)) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->T, (size_t)K * 3 * n1 * s->N)) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->Fh, (size_t)S * n1 * s->N)) != DG_OK) return bail(st);
  if (s->ops->element_lim) {
    if ((st = dalloc(s, &s->Fs, (size_t)S * s->N)) != DG_OK) return bail(st);
    if ((st = dalloc(s, &s->M, (size_t)s->N * Kp)) != DG_OK) return bail(st);
  }
  if ((st = dalloc(s, &s->partial, (size_t)s->N * ((K + 127) / 128 + 1))) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->ds, 1)) != DG_OK) return bail(st);
  if ((st = dalloc(s, &s->vbuf, (size_t)6 * Kp)) != DG_OK) return bail(st);
  if (cudaMemset(s->U, 0, s->ndof_p * sizeof(double)) != cudaSuccess ||
      cudaMemset(s->W, 0, s->ndof_p * sizeof(double)) != cudaSuccess ||
      cudaMemset(s->ds, 0, sizeof(dg::DevScalars)) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaMemset failed"));
  dg::DevScalars h{};
  h.one = 1.0;
  h.dmin = dmin;
  h.cfl = P.cfl;
  if (cudaMemcpy(s->ds, &h, sizeof h, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaMemcpy failed"));

  dg::Ctx &c = s->ctx;
  c.st = s->st;
  c.m = m;
  c.p = p;
  c.eq = eq;
  c.N = s->N;
  c.np = s->np;
  c.q = &s->q;
  c.tab = s->tabimg.data();
  c.T = s->T;
  c.Fh = s->Fh;
  c.Fs = s->Fs;
  c.M = s->M;
  c.ds = s->ds;
  dg_status ozs = oz_refresh(s);
  if (ozs != DG_OK) return bail(ozs);
  *out = s;
  return DG_OK;
}

extern "C" void dg_solver_destroy(dg_solver *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->st) cudaStreamSynchronize(s->st);
  drop_graphs(s);
  for (auto &pe : s->pending) {
    cudaEventDestroy(pe.a);
    cudaEventDestroy(pe.b);
  }
  for (auto e : s->pool) cudaEventDestroy(e);
  if (s->cst) cudaStreamSynchronize(s->cst);
  for (auto e : s->cev) cudaEventDestroy(e);
  if (s->cst) cudaStreamDestroy(s->cst);
  for (void *p : s->allocs) cudaFree(p);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

extern "C" dg_status dg_solver_sizes(const dg_solver *s, int *N, int *n_p, int *K, int *S) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  if (N) *N = s->N;
  if (n_p) *n_p = s->np;
  if (K) *K = s->K;
  if (S) *S = s->S;
  return DG_OK;
}

extern "C" void *dg_solver_stream(dg_solver *s) { return s ? (void *)s->st : nullptr; }

extern "C" dg_status dg_solver_set_tables(dg_solver *s, int n_q, int n_1, const double *basis,
                                          const double *grad_x, const double *grad_y,
                                          const double *side, const double *vertex,
                                          const double *w, const double *r1, const double *r2,
                                          const double *r_oned, const double *w_oned) {
  if (!s || !basis || !grad_x || !grad_y || !side || !vertex || !w || !r1 || !r2 || !r_oned ||
      !w_oned)
    return fail(DG_BAD_ARG, "null argument");
  s->tr_valid = false;
  if (n_q != dg::nq_of(s->p) || n_1 != s->p + 1)
    return fail(DG_BAD_ARG, "table sizes do not match the order p");
  dg_order_tables t{};
  int np = s->np;
  t.n_p = np;
  t.n_q = n_q;
  t.n_1 = n_1;
  for (int q = 0; q < n_q; q++) {
    t.r[q] = r1[q];
    t.s[q] = r2[q];
    t.w[q] = w[q];
    for (int i = 0; i < np; i++) {
      t.B[q][i] = basis[i * n_q + q];
      t.GR[q][i] = grad_x[i * n_q + q];
      t.GS[q][i] = grad_y[i * n_q + q];
    }
  }
  for (int j = 0; j < n_1; j++) {
    t.t1[j] = r_oned[j];
    t.w1[j] = w_oned[j];
    for (int f = 0; f < 3; f++)
      for (int i = 0; i < np; i++) t.E[f][j][i] = side[f * np * n_1 + i * n_1 + j];
  }
  for (int v = 0; v < 3; v++)
    for (int i = 0; i < np; i++) t.V[v][i] = vertex[i * 3 + v];
  // the kernels use that basis function 0 is a positive constant (one edge
  // value; the limiter's mean bounds need phi_0 > 0)
  if (!(t.B[0][0] > 0))
    return fail(DG_BAD_ARG, "basis function 0 must be positive");
  for (int f = 0; f < 3; f++)
    for (int j = 0; j < n_1; j++)
      if (t.E[f][j][0] != t.E[0][0][0])
        return fail(DG_BAD_ARG, "basis function 0 must take one value on every edge point");
  s->tables = t;
  dg::build_tab(s->p, s->tables, s->tabimg.data());
  field_refresh(s);
  drop_graphs(s);
  {
    dg_status ozs = oz_refresh(s);
    if (ozs != DG_OK) return ozs;
  }
  return DG_OK;
}

extern "C" dg_status dg_init(dg_solver *s) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  run(s, K_RK, [&] { s->ops->init(s->ctx, s->U); });
  collect_profile(s);
  return sync_check(s);
}

// rows [r0, r0 + nr) of the state from the caller's layout into U; with
// `flag`, sets *flag when a value changes
static void put_rows(dg_solver *s, const double *user, int r0, int nr, int *flag) {
  const double *src = user + (size_t)r0 * s->K;
  double *dst = s->U + (size_t)r0 * s->m.Kp;
  if (flag) dg::launch_permute_in_cmp(s->st, src, dst, s->m.perm, nr, s->K, s->m.Kp, flag);
  else dg::launch_permute_in(s->st, src, dst, s->m.perm, nr, s->K, s->m.Kp);
}

// before a put: when the stored traces were current, a flag (cleared here)
// that records whether the state changes
static dg_status begin_put(dg_solver *s, bool &keep) {
  keep = s->tr_valid;
  s->tr_valid = false;
  if (!keep) return DG_OK;
  if (!s->flag) {
    dg_status st = dalloc(s, &s->flag, 1);
    if (st != DG_OK) return st;
  }
  CK(cudaMemsetAsync(s->flag, 0, sizeof(int), s->st));
  return DG_OK;
}

// after a put: when the stored traces were current and the new state is
// bitwise the old one (a state read out and handed back unchanged), they
// stay current, so the next dg_step continues exactly as if the state had
// never left the device
static dg_status end_put(dg_solver *s, bool keep) {
  if (!keep) return sync_check(s);
  int changed = 1;
  CK(cudaMemcpyAsync(&changed, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  dg_status st = sync_check(s);
  if (st == DG_OK) s->tr_valid = changed == 0;
  return st;
}

static dg_status put_state(dg_solver *s, const double *user) {
  bool keep;
  dg_status st = begin_put(s, keep);
  if (st != DG_OK) return st;
  put_rows(s, user, 0, s->N * s->np, keep ? s->flag : nullptr);
  return end_put(s, keep);
}

// rows per chunk of a host transfer (the whole state below 16 MB) and the
// copy stream with its events
static int transfer_chunks(dg_solver *s, int &per) {
  const int rows = s->N * s->np;
  const size_t bytes = (size_t)rows * s->K * sizeof(double);
  per = bytes < ((size_t)16 << 20) ? rows : (rows + 7) / 8;
  const int n = (rows + per - 1) / per;
  if (!s->cst && cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking) != cudaSuccess) {
    s->cst = nullptr;
    return 0;
  }
  while ((int)s->cev.size() < n + 1) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return 0;
    s->cev.push_back(e);
  }
  return n;
}

// host -> device in chunks of rows on the copy stream, each chunk permuted
// on the solver stream as soon as it has arrived
extern "C" dg_status dg_set_state(dg_solver *s, const double *C) {
  if (!s || !C) return fail(DG_BAD_ARG, "null argument");
  CK(cudaSetDevice(s->device));
  int per = 0;
  const int nch = transfer_chunks(s, per);
  if (!nch) return fail(DG_CUDA_ERROR, "copy stream or events");
  bool keep;
  dg_status st = begin_put(s, keep);
  if (st != DG_OK) return st;
  const int rows = s->N * s->np;
  const size_t K = s->K;
  // ubuf may still be read by earlier work on the solver stream
  CK(cudaEventRecord(s->cev[nch], s->st));
  CK(cudaStreamWaitEvent(s->cst, s->cev[nch], 0));
  for (int c = 0; c < nch; c++) {
    const int r0 = c * per, nr = std::min(per, rows - r0);
    CK(cudaMemcpyAsync(s->ubuf + r0 * K, C + r0 * K, nr * K * sizeof(double),
                       cudaMemcpyHostToDevice, s->cst));
    CK(cudaEventRecord(s->cev[c], s->cst));
    CK(cudaStreamWaitEvent(s->st, s->cev[c], 0));
    put_rows(s, s->ubuf, r0, nr, keep ? s->flag : nullptr);
  }
  return end_put(s, keep);
}

// device -> host: each chunk of rows permuted on the solver stream, then
// copied on the copy stream while the next chunk is permuted
extern "C" dg_status dg_get_state(dg_solver *s, double *C) {
  if (!s || !C) return fail(DG_BAD_ARG, "null argument");
  CK(cudaSetDevice(s->device));
  int per = 0;
  const int nch = transfer_chunks(s, per);
  if (!nch) return fail(DG_CUDA_ERROR, "copy stream or events");
  const int rows = s->N * s->np;
  const size_t K = s->K, Kp = s->m.Kp;
  for (int c = 0; c < nch; c++) {
    const int r0 = c * per, nr = std::min(per, rows - r0);
    dg::launch_permute_out(s->st, s->U + r0 * Kp, s->ubuf + r0 * K, s->m.perm, nr, s->K, s->m.Kp);
    CK(cudaEventRecord(s->cev[c], s->st));
    CK(cudaStreamWaitEvent(s->cst, s->cev[c], 0));
    CK(cudaMemcpyAsync(C + r0 * K, s->ubuf + r0 * K, nr * K * sizeof(double),
                       cudaMemcpyDeviceToHost, s->cst));
  }
  // the solver stream waits for the copies (later work may overwrite ubuf)
  CK(cudaEventRecord(s->cev[nch], s->cst));
  CK(cudaStreamWaitEvent(s->st, s->cev[nch], 0));
  return sync_check(s);
}

extern "C" dg_status dg_set_state_device(dg_solver *s, const double *C) {
  if (!s || !C) return fail(DG_BAD_ARG, "null argument");
  CK(cudaSetDevice(s->device));
  return put_state(s, C);
}

extern "C" dg_status dg_get_state_device(dg_solver *s, double *C) {
  if (!s || !C) return fail(DG_BAD_ARG, "null argument");
  CK(cudaSetDevice(s->device));
  dg::launch_permute_out(s->st, s->U, C, s->m.perm, s->N * s->np, s->K, s->m.Kp);
  return sync_check(s);
}

extern "C" dg_status dg_rhs(dg_solver *s, double t, const double *C, double *dCdt) {
  if (!s || !C || !dCdt) return fail(DG_BAD_ARG, "null argument");
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  size_t n = (size_t)s->N * s->np * s->K;
  double *in = s->W, *out = nullptr;
  dg_status st = ensure_rk_buffers(s);
  if (st != DG_OK) return st;
  out = s->k[0];
  st = set_scalar(s, offsetof(dg::DevScalars, t), &t, sizeof t);
  if (st != DG_OK) return st;
  CK(cudaMemcpyAsync(s->ubuf, C, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  dg::launch_permute_in(s->st, s->ubuf, in, s->m.perm, s->N * s->np, s->K, s->m.Kp);
  stage(s, in, nullptr, out, 0.0, 0.0, 1.0, 0.0, &s->ds->one);
  dg::launch_permute_out(s->st, out, s->ubuf, s->m.perm, s->N * s->np, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(dCdt, s->ubuf, n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  collect_profile(s);
  return sync_check(s);
}

extern "C" dg_status dg_limit(dg_solver *s) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  if (s->np >= 3) run(s, K_LIMIT, [&] { s->ops->limit(s->ctx, s->U); });
  collect_profile(s);
  return sync_check(s);
}

extern "C" dg_status dg_step(dg_solver *s, int nsteps, dg_scheme scheme, double fixed_dt,
                             double *t) {
  if (!s || !t) return fail(DG_BAD_ARG, "null argument");
  if (nsteps < 0) return fail(DG_BAD_ARG, "nsteps must be >= 0");
  CK(cudaSetDevice(s->device));
  return run_steps(s, nsteps, scheme, fixed_dt, 0.0, t, nullptr);
}

extern "C" dg_status dg_advance_to(dg_solver *s, double T, dg_scheme scheme, double *t,
                                   int *nsteps) {
  if (!s || !t) return fail(DG_BAD_ARG, "null argument");
  if (!(T > *t)) {
    if (nsteps) *nsteps = 0;
    return DG_OK;
  }
  CK(cudaSetDevice(s->device));
  return run_steps(s, 0, scheme, 0.0, T, t, nsteps);
}

extern "C" dg_status dg_cfl(dg_solver *s, double *dt, double *lambda_max, double *d_min) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  CK(cudaSetDevice(s->device));
  dg::DevScalars h{};
  dg_status st = read_scalars(s, &h);
  if (st != DG_OK) return st;
  h.fixed_dt = 0;
  h.endtime = 0;
  h.cfl = s->prm.cfl;
  h.dmin = s->dmin;
  h.status = 0;
  st = set_scalar(s, 0, &h, sizeof h);
  if (st != DG_OK) return st;
  cfl(s);
  collect_profile(s);
  st = read_scalars(s, &h);
  if (st != DG_OK) return st;
  if (dt) *dt = h.dt;
  if (lambda_max) *lambda_max = __builtin_bit_cast(double, h.lam_bits);
  if (d_min) *d_min = s->dmin;
  if (h.status == 4) return fail(DG_NAN, "wave speed is NaN");
  return DG_OK;
}

extern "C" dg_status dg_l2_error(dg_solver *s, double t, double *err) {
  if (!s || !err) return fail(DG_BAD_ARG, "null argument");
  CK(cudaSetDevice(s->device));
  int nb = s->ops->l2err(s->ctx, s->U, t, s->partial);
  s->launches++;
  std::vector<double> h((size_t)nb * s->N);
  CK(cudaMemcpyAsync(h.data(), s->partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                     s->st));
  dg_status st = sync_check(s);
  if (st != DG_OK) return st;
  for (int n = 0; n < s->N; n++) {
    double a = 0;
    for (int b = 0; b < nb; b++) a += h[(size_t)b * s->N + n];
    err[n] = std::sqrt(a);
  }
  return DG_OK;
}

// ---- shallow-water bed ---------------------------------------------------
extern "C" dg_status dg_set_bathymetry(dg_solver *s, const double *b) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  if (s->eq != DG_SHALLOW_WATER) return fail(DG_UNSUPPORTED, "bathymetry needs shallow water");
  CK(cudaSetDevice(s->device));
  if (!b) {
    s->m.bathy = nullptr;
  } else {
    if (!s->bathy) {
      dg_status st = dalloc(s, &s->bathy, (size_t)s->np * s->m.Kp);
      if (st != DG_OK) return st;
    }
    CK(cudaMemcpyAsync(s->ubuf, b, (size_t)s->np * s->K * sizeof(double),
                       cudaMemcpyHostToDevice, s->st));
    dg::launch_permute_in(s->st, s->ubuf, s->bathy, s->m.perm, s->np, s->K, s->m.Kp);
    s->m.bathy = s->bathy;
  }
  s->ctx.m.bathy = s->m.bathy;
  drop_graphs(s);
  return sync_check(s);
}

extern "C" dg_status dg_get_bathymetry(dg_solver *s, double *b) {
  if (!s || !b) return fail(DG_BAD_ARG, "null argument");
  if (!s->m.bathy) {
    std::memset(b, 0, sizeof(double) * (size_t)s->np * s->K);
    return DG_OK;
  }
  CK(cudaSetDevice(s->device));
  dg::launch_permute_out(s->st, s->m.bathy, s->ubuf, s->m.perm, s->np, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(b, s->ubuf, (size_t)s->np * s->K * sizeof(double), cudaMemcpyDeviceToHost,
                     s->st));
  return sync_check(s);
}

extern "C" dg_status dg_bathymetry_project(dg_solver *s, int kind, const double *prm) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  if (kind == DG_BED_FLAT) return dg_set_bathymetry(s, nullptr);
  if (!prm) return fail(DG_BAD_ARG, "null parameters");
  if (kind != DG_BED_SINE && kind != DG_BED_LINEAR) return fail(DG_BAD_ARG, "unknown bed kind");
  // b_i = sum_q w_q b(x_q) phi_i(q) per element (orthonormal basis, as evalU0)
  const dg_order_tables &T = s->tables;
  std::vector<double> b((size_t)s->np * s->K);
  for (int e = 0; e < s->K; e++) {
    const double *V = s->mesh_v.data() + (size_t)6 * e;
    for (int i = 0; i < s->np; i++) {
      double acc = 0;
      for (int q = 0; q < T.n_q; q++) {
        double r = T.r[q], ss = T.s[q];
        double x = V[2] * r + V[4] * ss + V[0] * (1 - r - ss);
        double y = V[3] * r + V[5] * ss + V[1] * (1 - r - ss);
        double bv = kind == DG_BED_SINE
                        ? prm[0] * std::sin(2 * dg::kPi * prm[1] * x) * std::sin(2 * dg::kPi * prm[2] * y)
                        : prm[0] + prm[1] * x + prm[2] * y;
        acc += T.w[q] * bv * T.B[q][i];
      }
      b[(size_t)i * s->K + e] = acc;
    }
  }
  return dg_set_bathymetry(s, b.data());
}

// ---- block-size autotuner --------------------------------------------------
namespace {
template <class F>
dg_status time_steps(cudaStream_t st, F &&step, float *ms) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, st);
  dg_status r = step();
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return r;
}
const int kTuneBlocks[] = {64, 128, 256};
}  // namespace

namespace {
// times SSP-RK3 steps from the state `save` at each block size of the stage
// kernels; the best block and its time
dg_status tune_blocks(dg_solver *s, const double *save, int *best, float *best_ms) {
  *best_ms = 1e30f;
  for (int blk : kTuneBlocks) {
    s->ctx.blk = blk;
    drop_graphs(s);
    double t = 0;
    dg_status st = run_steps(s, 1, DG_SSP_RK3, 0.0, 0.0, &t, nullptr);  // capture + warm
    float ms = 0;
    if (st == DG_OK)
      st = time_steps(s->st, [&] { return run_steps(s, 3, DG_SSP_RK3, 0.0, 0.0, &t, nullptr); },
                      &ms);
    cudaMemcpyAsync(s->U, save, s->ndof_p * sizeof(double), cudaMemcpyDeviceToDevice, s->st);
    s->tr_valid = false;  // T belongs to the advanced state
    if (st != DG_OK) return st;
    if (ms < *best_ms) {
      *best_ms = ms;
      *best = blk;
    }
  }
  return DG_OK;
}
}  // namespace

extern "C" dg_status dg_autotune(dg_solver *s, int *block) {
  return dg_autotune_stage(s, block, nullptr);
}

// threads_per_element == nullptr: block size only, with the element stage
// as it is; else also the element stage itself where there is a choice
extern "C" dg_status dg_autotune_stage(dg_solver *s, int *block, int *threads_per_element) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  double *save = nullptr;
  CK(cudaMalloc(&save, s->ndof_p * sizeof(double)));
  CK(cudaMemcpyAsync(save, s->U, s->ndof_p * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
  std::vector<int> variants;  // 1: the FP64 element stage, 2: the tensor-core one
  if (threads_per_element && s->oz) variants = {1, 2};
  else variants = {s->ctx.oz ? 2 : 1};
  int best_blk = s->ctx.blk, best_v = variants[0];
  float best_ms = 1e30f;
  for (int v : variants) {
    s->tensor = v == 2;
    s->ctx.oz = s->tensor ? s->oz : nullptr;
    int blk = s->ctx.blk;
    float ms = 0;
    dg_status st = tune_blocks(s, save, &blk, &ms);
    if (st != DG_OK) {
      cudaStreamSynchronize(s->st);
      cudaFree(save);
      return st;
    }
    if (ms < best_ms) {
      best_ms = ms;
      best_blk = blk;
      best_v = v;
    }
  }
  cudaStreamSynchronize(s->st);
  cudaFree(save);
  s->tensor = best_v == 2;
  s->ctx.oz = s->tensor ? s->oz : nullptr;
  s->ctx.blk = best_blk;
  drop_graphs(s);
  if (block) *block = best_blk;
  if (threads_per_element) *threads_per_element = best_v;
  return DG_OK;
}

// ---- batched ensembles -------------------------------------------------------
struct dg_batch {
  std::vector<dg_solver *> m;
  int device = 0, blk = 128, limiter = 0;
  dg_equation eq = DG_SHALLOW_WATER;
  cudaStream_t st = nullptr;
  const dg::BatchOps *ops = nullptr;
  std::vector<char> tabs;
  dg::BatchProb *probs = nullptr;
  int *maps = nullptr;  // device: element/side/lambda block maps
  dg::BatchLaunch bl;
  cudaGraphExec_t graph = nullptr;
  long long graph_nodes = 0, launches = 0;
};

namespace {
const dg::BatchOps *batch_ops_for(dg_equation eq) {
  switch (eq) {
    case DG_ADVECTION: return &dg::batch_ops_advection();
    case DG_EULER: return &dg::batch_ops_euler();
    case DG_SHALLOW_WATER: return &dg::batch_ops_shallow_water();
    case DG_MAXWELL: return &dg::batch_ops_maxwell();
  }
  return nullptr;
}

// block -> problem maps for blocks of `blk` elements (or sides), the
// problems visited in `order` (each problem's blocks stay contiguous)
void block_maps(const std::vector<int> &count, const std::vector<int> &order, int blk,
                std::vector<int> &b2p, std::vector<int> &b0) {
  b2p.clear();
  b0.assign(count.size(), 0);
  for (int i : order) {
    b0[i] = (int)b2p.size();
    int nb = (count[i] + blk - 1) / blk;
    for (int k = 0; k < nb; k++) b2p.push_back(i);
  }
}

// the element-stage group of a member: order and mesh size
constexpr int kSmallMesh = 16384;
int batch_group(const dg_solver *s) { return 2 * (s->p - 1) + (s->K >= kSmallMesh ? 1 : 0); }

dg_status batch_build_maps(dg_batch *b) {
  std::vector<int> ke, ks;
  for (auto *s : b->m) {
    ke.push_back(s->K);
    ks.push_back(s->S);
  }
  // problems of one group (order, mesh size) next to each other, so that the
  // element stage is one launch per group at its own block size and register
  // count; within a group, larger problems first
  std::vector<int> order(b->m.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const int gx = batch_group(b->m[x]), gy = batch_group(b->m[y]);
    if (gx != gy) return gx < gy;
    return b->m[x]->K > b->m[y]->K;
  });
  dg::BatchLaunch &L = b->bl;
  std::vector<int> e2p, e0(b->m.size(), 0), u2p, u0, s2p, s0, l2p, l0;
  for (int g = 0; g < dg::BatchLaunch::kGroups; g++) {
    L.eblk_g[g] = (int)e2p.size();
    for (int i : order) {
      if (batch_group(b->m[i]) != g) continue;
      e0[i] = (int)e2p.size();
      const int nb = (ke[i] + L.blk_g[g] - 1) / L.blk_g[g];
      for (int k = 0; k < nb; k++) e2p.push_back(i);
    }
  }
  L.eblk_g[dg::BatchLaunch::kGroups] = (int)e2p.size();
  block_maps(ke, order, b->blk, u2p, u0);
  block_maps(ks, order, b->blk, s2p, s0);
  block_maps(ke, order, 128, l2p, l0);
  std::vector<int> all;
  size_t oe2p = 0, oe0 = oe2p + e2p.size(), ou2p = oe0 + e0.size(), ou0 = ou2p + u2p.size(),
         os2p = ou0 + u0.size(), os0 = os2p + s2p.size(), ol2p = os0 + s0.size(),
         ol0 = ol2p + l2p.size();
  for (auto *v : {&e2p, &e0, &u2p, &u0, &s2p, &s0, &l2p, &l0})
    all.insert(all.end(), v->begin(), v->end());
  if (b->maps) cudaFree(b->maps);
  b->maps = nullptr;
  CK(cudaMalloc(&b->maps, all.size() * sizeof(int)));
  CK(cudaMemcpy(b->maps, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
  L.eblk2prob = b->maps + oe2p;
  L.eblk0 = b->maps + oe0;
  L.ublk2prob = b->maps + ou2p;
  L.ublk0 = b->maps + ou0;
  L.sblk2prob = b->maps + os2p;
  L.sblk0 = b->maps + os0;
  L.lblk2prob = b->maps + ol2p;
  L.lblk0 = b->maps + ol0;
  L.neblk = (int)e2p.size();
  L.nublk = (int)u2p.size();
  L.nsblk = (int)s2p.size();
  L.nlblk = (int)l2p.size();
  L.blk = b->blk;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return DG_OK;
}

// one SSP-RK3 step of every member (launch sequence, capturable)
void batch_step_seq(dg_batch *b) {
  const dg::BatchLaunch &L = b->bl;
  dg::launch_batch_reset_lambda(L.st, L.probs, L.nprob);
  b->ops->lambda(L);
  dg::launch_batch_compute_dt(L.st, L.probs, L.nprob);
  const double tc[3] = {0.0, 1.0, 0.5};
  for (int stage = 0; stage < 3; stage++) {
    if (L.fused) {  // the limiter in the element epilogue, as the members' own steps
      b->ops->face_fs(L, tc[stage]);
      b->ops->means(L, stage);
      b->ops->element_lim(L, stage);
      continue;
    }
    b->ops->face(L, tc[stage]);
    b->ops->element(L, stage);
    if (L.limiter) b->ops->limit_tr(L, stage);
  }
  dg::launch_batch_advance_t(L.st, L.probs, L.nprob);
}

dg_status batch_run(dg_batch *b, int nsteps, double *t) {
  CK(cudaSetDevice(b->device));
  for (size_t i = 0; i < b->m.size(); i++) {
    dg_solver *s = b->m[i];
    CK(cudaStreamSynchronize(s->st));
    dg::DevScalars h{};
    h.t = t ? t[i] : 0.0;
    h.one = 1.0;
    h.dmin = s->dmin;
    h.cfl = s->prm.cfl;
    CK(cudaMemcpyAsync(s->ds, &h, sizeof h, cudaMemcpyHostToDevice, b->st));
    // the reference limits once before its step loop (time_integrator.cu:178-184)
    if (b->limiter && s->np >= 3) {
      dg::Ctx c = s->ctx;
      c.st = b->st;
      s->ops->limit(c, s->U);
      b->launches++;
    }
  }
  b->ops->trace(b->bl);
  b->launches++;
  if (!b->graph) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    batch_step_seq(b);
    cudaError_t e = cudaStreamEndCapture(b->st, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    b->graph_nodes = (long long)nn;
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  }
  for (int k = 0; k < nsteps; k++) {
    CK(cudaGraphLaunch(b->graph, b->st));
    b->launches += b->graph_nodes;
  }
  cudaError_t e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return cuda_fail(e, "batched step");
  int nan = 0;
  for (size_t i = 0; i < b->m.size(); i++) {
    dg::DevScalars h{};
    CK(cudaMemcpy(&h, b->m[i]->ds, sizeof h, cudaMemcpyDeviceToHost));
    if (t) t[i] = h.t;
    if (h.status == 4) nan = 1;
  }
  if (nan) return fail(DG_NAN, "a batch member's time step is NaN or not positive");
  return DG_OK;
}
}  // namespace

extern "C" dg_status dg_batch_create(int n, dg_solver *const *members, dg_batch **out) {
  if (!out || !members || n <= 0) return fail(DG_BAD_ARG, "bad batch arguments");
  *out = nullptr;
  dg_batch *b = new dg_batch();
  auto bail = [&](dg_status st) {
    dg_batch_destroy(b);
    return st;
  };
  const void *timg[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int i = 0; i < n; i++) {
    dg_solver *s = members[i];
    if (!s) return bail(fail(DG_BAD_ARG, "null batch member"));
    if (i == 0) {
      b->device = s->device;
      b->eq = s->eq;
      b->limiter = s->prm.limiter ? 1 : 0;
    }
    if (s->device != b->device || s->eq != b->eq)
      return bail(fail(DG_BAD_ARG, "batch members must share device and equation"));
    if ((s->prm.limiter ? 1 : 0) != b->limiter)
      return bail(fail(DG_BAD_ARG, "batch members must agree on the limiter"));
    if (s->p < 1 || s->p > 3) return bail(fail(DG_UNSUPPORTED, "batched orders are p = 1..3"));
    if (!timg[s->p]) timg[s->p] = s->tabimg.data();
    b->m.push_back(s);
  }
  if (cudaSetDevice(b->device) != cudaSuccess) return bail(fail(DG_CUDA_ERROR, "cudaSetDevice"));
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaStreamCreate"));
  b->ops = batch_ops_for(b->eq);
  b->tabs.resize(dg::batch_tabs_bytes());
  dg::build_batch_tabs(timg[1], timg[2], timg[3], b->tabs.data());
  std::vector<dg::BatchProb> hp(n);
  for (int i = 0; i < n; i++) {
    dg_solver *s = b->m[i];
    dg::BatchProb &q = hp[i];
    std::memset(&q, 0, sizeof q);
    q.p = s->p;
    q.K = s->K;
    q.Kp = s->m.Kp;
    q.S = s->S;
    q.Sb = s->m.Sb;
    q.U = s->U;
    q.W = s->W;
    q.T = s->T;
    q.Fh = s->Fh;
    q.Fs = s->Fs;
    q.M = s->M;
    q.geo = s->m.geo;
    q.esd = s->m.esd;
    q.nbr = s->m.nbr;
    q.side = s->m.side;
    q.sgeo = s->m.sgeo;
    q.bxy = s->m.bxy;
    q.bathy = s->m.bathy;
    q.vtx = s->m.vtx;
    q.ds = s->ds;
    q.q = s->q;
  }
  if (cudaMalloc(&b->probs, sizeof(dg::BatchProb) * n) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaMalloc"));
  if (cudaMemcpy(b->probs, hp.data(), sizeof(dg::BatchProb) * n, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "cudaMemcpy"));
  b->bl.st = b->st;
  for (int g = 0; g < dg::BatchLaunch::kGroups; g++) {
    if (cudaStreamCreateWithFlags(&b->bl.gst[g], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->bl.join[g], cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(DG_CUDA_ERROR, "batch group streams"));
  }
  if (cudaEventCreateWithFlags(&b->bl.fork, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(DG_CUDA_ERROR, "batch group streams"));
  b->bl.tabs = b->tabs.data();
  b->bl.probs = b->probs;
  b->bl.nprob = n;
  b->bl.limiter = b->limiter;
  // with the limiter, the members' own steps limit in the element epilogue
  // where their equation has that stage (fused_stage): the batch does the same
  {
    bool all = b->limiter && b->ops->element_lim;
    for (auto *s : b->m) all = all && s->M && s->np >= 3;
    b->bl.fused = all ? 1 : 0;
  }
  dg_status st = batch_build_maps(b);
  if (st != DG_OK) return bail(st);
  *out = b;
  return DG_OK;
}

extern "C" dg_status dg_batch_step(dg_batch *b, int nsteps, double *t) {
  if (!b || nsteps < 0) return fail(DG_BAD_ARG, "bad batch step arguments");
  for (dg_solver *s : b->m) s->tr_valid = false;
  return batch_run(b, nsteps, t);
}

// Block sizes of a batch, timed on SSP-RK3 steps from the members' current
// states (restored afterwards): first the one shared by the face, trace and
// limiter launches, then each element-stage group's (order, mesh size) in
// turn, each trying 64, 128 and 256 elements per block.
extern "C" dg_status dg_batch_autotune(dg_batch *b, int *block) {
  if (!b) return fail(DG_BAD_ARG, "null batch");
  CK(cudaSetDevice(b->device));
  std::vector<double *> save(b->m.size(), nullptr);
  for (size_t i = 0; i < b->m.size(); i++) {
    CK(cudaMalloc(&save[i], b->m[i]->ndof_p * sizeof(double)));
    CK(cudaMemcpy(save[i], b->m[i]->U, b->m[i]->ndof_p * sizeof(double),
                  cudaMemcpyDeviceToDevice));
  }
  bool used[dg::BatchLaunch::kGroups] = {false};
  for (auto *s : b->m) used[batch_group(s)] = true;
  std::vector<double> t(b->m.size(), 0.0);
  dg_status st = DG_OK;
  // times 3 steps with the current settings
  auto trial = [&](float *ms) -> dg_status {
    dg_status r = batch_build_maps(b);
    if (r == DG_OK) r = batch_run(b, 1, t.data());  // capture + warm
    if (r == DG_OK) r = time_steps(b->st, [&] { return batch_run(b, 3, t.data()); }, ms);
    for (size_t i = 0; i < b->m.size(); i++)
      cudaMemcpy(b->m[i]->U, save[i], b->m[i]->ndof_p * sizeof(double),
                 cudaMemcpyDeviceToDevice);
    return r;
  };
  for (int knob = -1; knob < dg::BatchLaunch::kGroups && st == DG_OK; knob++) {
    if (knob >= 0 && !used[knob]) continue;
    int &v = knob < 0 ? b->blk : b->bl.blk_g[knob];
    int best = v;
    float best_ms = 1e30f;
    for (int blk : kTuneBlocks) {
      v = blk;
      float ms = 0;
      if ((st = trial(&ms)) != DG_OK) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = blk;
      }
    }
    v = best;
  }
  for (auto *p : save) cudaFree(p);
  if (st != DG_OK) return st;
  st = batch_build_maps(b);
  if (block) *block = b->blk;
  return st;
}

extern "C" dg_status dg_batch_blocks(const dg_batch *b, int *blocks) {
  if (!b || !blocks) return fail(DG_BAD_ARG, "null argument");
  blocks[0] = b->blk;
  for (int g = 0; g < dg::BatchLaunch::kGroups; g++) blocks[1 + g] = b->bl.blk_g[g];
  return DG_OK;
}

extern "C" long long dg_batch_launches(const dg_batch *b) { return b ? b->launches : 0; }

extern "C" void dg_batch_destroy(dg_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->maps) cudaFree(b->maps);
  if (b->probs) cudaFree(b->probs);
  for (int g = 0; g < dg::BatchLaunch::kGroups; g++) {
    if (b->bl.gst[g]) cudaStreamDestroy(b->bl.gst[g]);
    if (b->bl.join[g]) cudaEventDestroy(b->bl.join[g]);
  }
  if (b->bl.fork) cudaEventDestroy(b->bl.fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

// ---- tangent-linear and adjoint of the shallow-water step ----------------
namespace {

struct LinBufs {
  double *Tv = nullptr, *F0 = nullptr, *F1 = nullptr;
};

dg_status lin_bufs(dg_solver *s, LinBufs *b) {
  static_assert(sizeof(LinBufs) > 0, "");
  const size_t nt = (size_t)s->K * 3 * (s->p + 1) * s->N, nf = (size_t)s->S * (s->p + 1) * s->N;
  if (!s->lin_tv) {
    dg_status st;
    if ((st = dalloc(s, &s->lin_tv, nt)) != DG_OK) return st;
    if ((st = dalloc(s, &s->lin_f0, nf)) != DG_OK) return st;
    if ((st = dalloc(s, &s->lin_f1, nf)) != DG_OK) return st;
  }
  b->Tv = s->lin_tv;
  b->F0 = s->lin_f0;
  b->F1 = s->lin_f1;
  return DG_OK;
}

// forward traces of the linearisation state (into s->T)
void fwd_traces(dg_solver *s, double *u) {
  run(s, K_TRACE, [&] { s->ops->trace(s->ctx, u); });
}

// dout = ca dun + cb dus + ccdt (dL/du dus + dL/db db), linearised at us
void tl_stage(dg_solver *s, double *us, const double *dus, const double *db, const double *dun,
              double *dout, double ca, double cb, double ccdt, const LinBufs &lb) {
  fwd_traces(s, us);
  dg::Ctx c = s->ctx;
  c.Fh = lb.F0;
  run(s, K_TRACE, [&] { dg::lin_trace(c, dus, nullptr, 1.0, lb.Tv); });
  run(s, K_FACE, [&] { dg::tl_face(c, lb.Tv, lb.F0); });
  run(s, K_ELEMENT, [&] { dg::tl_element(c, us, dus, db, dun, dout, ca, cb, ccdt); });
}

// ubar_s = cb obar + ccdt (dL/du)^T obar ; bbar += ccdt (dL/db)^T obar
void adj_stage(dg_solver *s, double *us, const double *obar, double *ubar_s, double *bbar,
               double cb, double ccdt, const LinBufs &lb) {
  fwd_traces(s, us);
  const dg::Ctx &c = s->ctx;
  run(s, K_TRACE, [&] { dg::lin_trace(c, obar, s->m.geo + 4 * (size_t)s->m.Kp, ccdt, lb.Tv); });
  run(s, K_FACE, [&] { dg::adj_face(c, lb.Tv, lb.F0, lb.F1); });
  run(s, K_ELEMENT, [&] { dg::adj_element(c, us, obar, ubar_s, bbar, lb.F0, lb.F1, cb, ccdt); });
}

dg_status lin_check(dg_solver *s) {
  if (s->eq != DG_SHALLOW_WATER)
    return fail(DG_UNSUPPORTED, "tangent-linear / adjoint operators are for shallow water");
  if (!dg::lin_supported(s->p)) return fail(DG_UNSUPPORTED, "adjoint orders are p = 1..4");
  if (s->prm.limiter) return fail(DG_UNSUPPORTED, "adjoint of the limiter is not provided");
  if (s->has_inout_bc)
    return fail(DG_UNSUPPORTED, "adjoint supports reflect, transmissive and periodic sides");
  return DG_OK;
}

}  // namespace

extern "C" dg_status dg_rhs_tl(dg_solver *s, double t, const double *C, const double *dC,
                               const double *db, double *dL) {
  if (!s || !C || !dC || !dL) return fail(DG_BAD_ARG, "null argument");
  s->tr_valid = false;
  dg_status st = lin_check(s);
  if (st != DG_OK) return st;
  CK(cudaSetDevice(s->device));
  LinBufs lb;
  if ((st = lin_bufs(s, &lb)) != DG_OK) return st;
  if ((st = ensure_rk_buffers(s)) != DG_OK) return st;
  const size_t n = (size_t)s->N * s->np * s->K;
  const int rows = s->N * s->np;
  double *u = s->k[0], *du = s->k[1], *out = s->k[2], *dbi = s->k[3];
  CK(cudaMemcpyAsync(s->ubuf, C, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  dg::launch_permute_in(s->st, s->ubuf, u, s->m.perm, rows, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(s->ubuf, dC, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  dg::launch_permute_in(s->st, s->ubuf, du, s->m.perm, rows, s->K, s->m.Kp);
  const double *dbp = nullptr;
  if (db) {
    CK(cudaMemcpyAsync(s->ubuf, db, (size_t)s->np * s->K * sizeof(double),
                       cudaMemcpyHostToDevice, s->st));
    dg::launch_permute_in(s->st, s->ubuf, dbi, s->m.perm, s->np, s->K, s->m.Kp);
    dbp = dbi;
  }
  (void)t;
  tl_stage(s, u, du, dbp, nullptr, out, 0.0, 0.0, 1.0, lb);
  dg::launch_permute_out(s->st, out, s->ubuf, s->m.perm, rows, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(dL, s->ubuf, n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  collect_profile(s);
  return sync_check(s);
}

extern "C" dg_status dg_rhs_adjoint(dg_solver *s, double t, const double *C, const double *Lbar,
                                    double *Cbar, double *bbar) {
  if (!s || !C || !Lbar || !Cbar) return fail(DG_BAD_ARG, "null argument");
  s->tr_valid = false;
  dg_status st = lin_check(s);
  if (st != DG_OK) return st;
  CK(cudaSetDevice(s->device));
  LinBufs lb;
  if ((st = lin_bufs(s, &lb)) != DG_OK) return st;
  if ((st = ensure_rk_buffers(s)) != DG_OK) return st;
  const size_t n = (size_t)s->N * s->np * s->K;
  const int rows = s->N * s->np;
  double *u = s->k[0], *lb_in = s->k[1], *out = s->k[2], *bb = s->k[3];
  CK(cudaMemcpyAsync(s->ubuf, C, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  dg::launch_permute_in(s->st, s->ubuf, u, s->m.perm, rows, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(s->ubuf, Lbar, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
  dg::launch_permute_in(s->st, s->ubuf, lb_in, s->m.perm, rows, s->K, s->m.Kp);
  CK(cudaMemsetAsync(bb, 0, (size_t)s->np * s->m.Kp * sizeof(double), s->st));
  (void)t;
  adj_stage(s, u, lb_in, out, bb, 0.0, 1.0, lb);
  dg::launch_permute_out(s->st, out, s->ubuf, s->m.perm, rows, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(Cbar, s->ubuf, n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  if (bbar) {
    CK(cudaStreamSynchronize(s->st));
    dg::launch_permute_out(s->st, bb, s->ubuf, s->m.perm, s->np, s->K, s->m.Kp);
    CK(cudaMemcpyAsync(bbar, s->ubuf, (size_t)s->np * s->K * sizeof(double),
                       cudaMemcpyDeviceToHost, s->st));
  }
  collect_profile(s);
  return sync_check(s);
}

// ---- the time-stepping adjoint with checkpoints ------------------------------
struct dg_adjoint {
  dg_solver *s = nullptr;
  int nrec = 0, nsteps = 0, every = 1, ckpt = 50;
  double dt = 0, t0 = 0;
  int *rec_el = nullptr;
  double *rec_phi = nullptr, *samples = nullptr, *sbar = nullptr;
  std::vector<double *> cks;                  // checkpoints u^{k ckpt}
  std::vector<double *> seg;                  // 3 ckpt states of a segment: u^n, u1, u2
  // every step's u^n, u1, u2 ([3 nsteps][ndof_p]) when they fit in device
  // memory (keep != 0): the reverse sweep then recomputes nothing
  int keep = 1;
  bool stored = false;
  double *store = nullptr;
  size_t store_n = 0;
  double *ufinal = nullptr;                   // the forward run's final state
  double t_end = 0;                           // and its time
  double *ub = nullptr, *ub1 = nullptr, *ub2 = nullptr, *acc = nullptr, *bbar = nullptr;
  double *du = nullptr, *dw = nullptr, *dbi = nullptr;
  std::vector<void *> mem;
};

namespace {
template <class T>
dg_status amalloc(dg_adjoint *a, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  a->mem.push_back(q);
  *p = static_cast<T *>(q);
  return DG_OK;
}

// one SSP-RK3 step of fixed dt through the fused stages (the adjoint
// excludes the limiter, and without it a fused stage gives the bits of the
// unfused one: its element epilogue writes the traces k_trace would compute);
// keeps the stage inputs u1, u2 when given.  T must hold the traces of U, or
// need_trace asks for them (the first step of a run or of a segment).
void plain_step(dg_solver *s, double *u1keep, double *u2keep, bool need_trace) {
  const size_t bytes = s->ndof_p * sizeof(double);
  const double *dt = &s->ds->dt;
  if (need_trace) run(s, K_TRACE, [&] { s->ops->trace(s->ctx, s->U); });
  fused_stage(s, s->U, nullptr, s->W, 0.0, 1.0, 1.0, 0.0, dt);
  if (u1keep) cudaMemcpyAsync(u1keep, s->W, bytes, cudaMemcpyDeviceToDevice, s->st);
  fused_stage(s, s->W, s->U, s->W, 0.75, 0.25, 0.25, 1.0, dt);
  if (u2keep) cudaMemcpyAsync(u2keep, s->W, bytes, cudaMemcpyDeviceToDevice, s->st);
  fused_stage(s, s->W, s->U, s->U, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5, dt);
  run(s, K_CFL, [&] { dg::launch_advance_t(s->st, s->ds); });
}

dg_status set_fixed_dt(dg_solver *s, double t, double dt) {
  dg::DevScalars h{};
  h.t = t;
  h.dt = dt;
  h.one = 1.0;
  h.dmin = s->dmin;
  h.cfl = s->prm.cfl;
  h.fixed_dt = dt;
  return set_scalar(s, 0, &h, sizeof h);
}
}  // namespace

extern "C" dg_status dg_adjoint_create(dg_solver *s, int nrec, const double *rx,
                                       const double *ry, dg_adjoint **out) {
  if (!s || !out || nrec < 0 || (nrec && (!rx || !ry))) return fail(DG_BAD_ARG, "bad arguments");
  *out = nullptr;
  dg_status st = lin_check(s);
  if (st != DG_OK) return st;
  CK(cudaSetDevice(s->device));
  dg_adjoint *a = new dg_adjoint();
  a->s = s;
  a->nrec = nrec;
  // locate receivers: element containing the point, reference coordinates
  std::vector<int> inv(s->K);
  std::vector<int> perm(s->K);
  CK(cudaMemcpy(perm.data(), s->m.perm, sizeof(int) * s->K, cudaMemcpyDeviceToHost));
  for (int e = 0; e < s->K; e++) inv[perm[e]] = e;
  std::vector<int> el(nrec);
  std::vector<double> phi((size_t)nrec * s->np);
  for (int r = 0; r < nrec; r++) {
    int found = -1;
    double rr = 0, ss = 0;
    for (int o = 0; o < s->K && found < 0; o++) {
      const double *V = s->mesh_v.data() + (size_t)6 * o;
      double xr = V[2] - V[0], xs = V[4] - V[0], yr = V[3] - V[1], ys = V[5] - V[1];
      double J = xr * ys - xs * yr, dx = rx[r] - V[0], dy = ry[r] - V[1];
      double a1 = (ys * dx - xs * dy) / J, a2 = (-yr * dx + xr * dy) / J;
      const double tol = -1e-12;
      if (a1 >= tol && a2 >= tol && a1 + a2 <= 1 - tol) {
        found = o;
        rr = a1;
        ss = a2;
      }
    }
    if (found < 0) {
      delete a;
      return fail(DG_BAD_ARG, "receiver " + std::to_string(r) + " lies outside the mesh");
    }
    el[r] = inv[found];
    for (int i = 0; i < s->np; i++) {
      long double v = 0;
      for (int m = 0; m <= i; m++) {
        long double term = DG_COEF[i][m];
        for (int k = 0; k < DG_MONO[m][0]; k++) term *= rr;
        for (int k = 0; k < DG_MONO[m][1]; k++) term *= ss;
        v += term;
      }
      phi[(size_t)r * s->np + i] = (double)v;
    }
  }
  if ((st = amalloc(a, &a->rec_el, (size_t)nrec)) != DG_OK) return st;
  if ((st = amalloc(a, &a->rec_phi, (size_t)nrec * s->np)) != DG_OK) return st;
  if (nrec) {
    CK(cudaMemcpy(a->rec_el, el.data(), sizeof(int) * nrec, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a->rec_phi, phi.data(), sizeof(double) * phi.size(), cudaMemcpyHostToDevice));
  }
  *out = a;
  return DG_OK;
}

extern "C" void dg_adjoint_destroy(dg_adjoint *a) {
  if (!a) return;
  cudaSetDevice(a->s->device);
  cudaStreamSynchronize(a->s->st);
  for (void *p : a->mem) cudaFree(p);
  delete a;
}

extern "C" dg_status dg_adjoint_set_storage(dg_adjoint *a, int keep_stages) {
  if (!a || keep_stages < 0 || keep_stages > 1) return fail(DG_BAD_ARG, "bad arguments");
  a->keep = keep_stages;
  if (!keep_stages && a->store) {
    cudaSetDevice(a->s->device);
    cudaStreamSynchronize(a->s->st);
    cudaFree(a->store);
    a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)a->store));
    a->store = nullptr;
    a->store_n = 0;
    a->stored = false;
  }
  return DG_OK;
}

extern "C" dg_status dg_adjoint_stored(const dg_adjoint *a, int *kept) {
  if (!a || !kept) return fail(DG_BAD_ARG, "null argument");
  *kept = a->stored ? 1 : 0;
  return DG_OK;
}

// forward run from the solver's state: nsteps SSP-RK3 steps of fixed dt,
// h sampled at the receivers after every `every` steps, the state saved
// every `ckpt` steps; samples = nsteps/every x nrec
extern "C" dg_status dg_adjoint_forward(dg_adjoint *a, int nsteps, double dt, int every,
                                        int ckpt, double t0, double *samples) {
  if (!a || nsteps <= 0 || !(dt > 0) || every <= 0 || ckpt <= 0)
    return fail(DG_BAD_ARG, "bad forward arguments");
  dg_solver *s = a->s;
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  dg_status st;
  const int nck = (nsteps + ckpt - 1) / ckpt, nsamp = nsteps / every;
  if (a->nsteps != nsteps || a->ckpt != ckpt || a->every != every || a->cks.empty()) {
    for (double *p : a->cks) {
      cudaFree(p);
      a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)p));
    }
    a->cks.assign(nck, nullptr);
    for (int k = 0; k < nck; k++)
      if ((st = amalloc(a, &a->cks[k], s->ndof_p)) != DG_OK) return st;
    for (double *p : a->seg) {
      cudaFree(p);
      a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)p));
    }
    a->seg.assign(3 * (size_t)ckpt, nullptr);
    for (auto &p : a->seg)
      if ((st = amalloc(a, &p, s->ndof_p)) != DG_OK) return st;
    if (!a->samples) {
      // (re)sized below
    }
  }
  if (a->samples) {
    cudaFree(a->samples);
    a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)a->samples));
    cudaFree(a->sbar);
    a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)a->sbar));
  }
  if ((st = amalloc(a, &a->samples, (size_t)std::max(nsamp, 1) * std::max(a->nrec, 1))) != DG_OK)
    return st;
  if ((st = amalloc(a, &a->sbar, (size_t)std::max(nsamp, 1) * std::max(a->nrec, 1))) != DG_OK)
    return st;
  a->nsteps = nsteps;
  a->every = every;
  a->ckpt = ckpt;
  a->dt = dt;
  a->t0 = t0;
  if (!a->ufinal && (st = amalloc(a, &a->ufinal, s->ndof_p)) != DG_OK) return st;
  // keep every stage state when that fits in free device memory (leaving
  // 4 GiB for everything else); otherwise the checkpoints alone
  const size_t need = (size_t)3 * nsteps * s->ndof_p;
  a->stored = false;
  if (a->keep) {
    if (a->store && a->store_n < need) {
      cudaFree(a->store);
      a->mem.erase(std::find(a->mem.begin(), a->mem.end(), (void *)a->store));
      a->store = nullptr;
      a->store_n = 0;
    }
    if (!a->store) {
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && need * sizeof(double) + ((size_t)4 << 30) < fr) {
        void *q = nullptr;
        if (cudaMalloc(&q, need * sizeof(double)) == cudaSuccess) {
          a->mem.push_back(q);
          a->store = static_cast<double *>(q);
          a->store_n = need;
        } else {
          cudaGetLastError();  // not enough after all: checkpoints only
        }
      }
    }
    a->stored = a->store != nullptr;
  }
  if ((st = set_fixed_dt(s, t0, dt)) != DG_OK) return st;
  const size_t bytes = s->ndof_p * sizeof(double);
  for (int n = 0; n < nsteps; n++) {
    if (n % ckpt == 0)
      CK(cudaMemcpyAsync(a->cks[n / ckpt], s->U, bytes, cudaMemcpyDeviceToDevice, s->st));
    if (a->stored) {
      double *u = a->store + (size_t)3 * n * s->ndof_p;
      CK(cudaMemcpyAsync(u, s->U, bytes, cudaMemcpyDeviceToDevice, s->st));
      plain_step(s, u + s->ndof_p, u + 2 * s->ndof_p, n == 0);
    } else {
      plain_step(s, nullptr, nullptr, n == 0);
    }
    if ((n + 1) % every == 0)
      dg::launch_sample(s->st, s->U, a->rec_el, a->rec_phi, a->nrec, s->np, s->m.Kp,
                        a->samples + (size_t)((n + 1) / every - 1) * a->nrec);
  }
  CK(cudaMemcpyAsync(a->ufinal, s->U, bytes, cudaMemcpyDeviceToDevice, s->st));
  CK(cudaMemcpyAsync(&a->t_end, &s->ds->t, sizeof(double), cudaMemcpyDeviceToHost, s->st));
  if (samples && nsamp && a->nrec)
    CK(cudaMemcpyAsync(samples, a->samples, sizeof(double) * nsamp * a->nrec,
                       cudaMemcpyDeviceToHost, s->st));
  collect_profile(s);
  return sync_check(s);
}

// gradients of sum_k,r sbar[k][r] * sample[k][r] with respect to the initial
// state (all variables, [var][mode][elem]) and the bed modes ([mode][elem]);
// the forward run must have been made by dg_adjoint_forward
extern "C" dg_status dg_adjoint_backward(dg_adjoint *a, const double *sbar, double *grad_u0,
                                         double *grad_b) {
  if (!a || !sbar || a->cks.empty()) return fail(DG_BAD_ARG, "no forward run to differentiate");
  dg_solver *s = a->s;
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  dg_status st;
  LinBufs lb;
  if ((st = lin_bufs(s, &lb)) != DG_OK) return st;
  const size_t bytes = s->ndof_p * sizeof(double);
  if (!a->ub) {
    if ((st = amalloc(a, &a->ub, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->ub1, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->ub2, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->acc, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->bbar, (size_t)s->np * s->m.Kp)) != DG_OK) return st;
  }
  const int nsamp = a->nsteps / a->every;
  if (nsamp && a->nrec)
    CK(cudaMemcpyAsync(a->sbar, sbar, sizeof(double) * nsamp * a->nrec, cudaMemcpyHostToDevice,
                       s->st));
  CK(cudaMemsetAsync(a->ub, 0, bytes, s->st));
  CK(cudaMemsetAsync(a->bbar, 0, (size_t)s->np * s->m.Kp * sizeof(double), s->st));
  const int n = (int)s->ndof_p;
  const double dt = a->dt;
  const int nck = (int)a->cks.size();
  for (int k = nck - 1; k >= 0; k--) {
    const int n0 = k * a->ckpt, n1 = std::min(n0 + a->ckpt, a->nsteps);
    if (!a->stored) {
      // recompute the segment, keeping u^n, u1, u2 of every step
      CK(cudaMemcpyAsync(s->U, a->cks[k], bytes, cudaMemcpyDeviceToDevice, s->st));
      if ((st = set_fixed_dt(s, a->t0 + n0 * dt, dt)) != DG_OK) return st;
      for (int m = n0; m < n1; m++) {
        const int j = m - n0;
        CK(cudaMemcpyAsync(a->seg[3 * j], s->U, bytes, cudaMemcpyDeviceToDevice, s->st));
        plain_step(s, a->seg[3 * j + 1], a->seg[3 * j + 2], m == n0);
      }
    }
    for (int m = n1 - 1; m >= n0; m--) {
      const int j = m - n0;
      if ((m + 1) % a->every == 0)  // adjoint of the sample taken from u^{m+1}
        dg::launch_sample_adj(s->st, a->ub, a->rec_el, a->rec_phi, a->nrec, s->np, s->m.Kp,
                              a->sbar + (size_t)((m + 1) / a->every - 1) * a->nrec);
      double *un = a->seg[3 * j], *u1 = a->seg[3 * j + 1], *u2 = a->seg[3 * j + 2];
      if (a->stored) {
        un = a->store + (size_t)3 * m * s->ndof_p;
        u1 = un + s->ndof_p;
        u2 = un + 2 * s->ndof_p;
      }
      // u^{n+1} = 1/3 u^n + 2/3 u2 + 2/3 dt L(u2)
      adj_stage(s, u2, a->ub, a->ub2, a->bbar, 2.0 / 3.0, 2.0 / 3.0 * dt, lb);
      dg::launch_axpby(s->st, n, 1.0 / 3.0, a->ub, 0.0, a->acc);
      // u2 = 3/4 u^n + 1/4 u1 + 1/4 dt L(u1)
      adj_stage(s, u1, a->ub2, a->ub1, a->bbar, 0.25, 0.25 * dt, lb);
      dg::launch_axpby(s->st, n, 0.75, a->ub2, 1.0, a->acc);
      // u1 = u^n + dt L(u^n)
      adj_stage(s, un, a->ub1, a->ub, a->bbar, 1.0, dt, lb);
      dg::launch_axpby(s->st, n, 1.0, a->acc, 1.0, a->ub);
    }
  }
  const int rows = s->N * s->np;
  if (grad_u0) {
    dg::launch_permute_out(s->st, a->ub, s->ubuf, s->m.perm, rows, s->K, s->m.Kp);
    CK(cudaMemcpyAsync(grad_u0, s->ubuf, sizeof(double) * rows * s->K, cudaMemcpyDeviceToHost,
                       s->st));
    CK(cudaStreamSynchronize(s->st));
  }
  if (grad_b) {
    dg::launch_permute_out(s->st, a->bbar, s->ubuf, s->m.perm, s->np, s->K, s->m.Kp);
    CK(cudaMemcpyAsync(grad_b, s->ubuf, sizeof(double) * s->np * s->K, cudaMemcpyDeviceToHost,
                       s->st));
  }
  // leave the solver at the final state (and time) of the forward run
  CK(cudaMemcpyAsync(s->U, a->ufinal, bytes, cudaMemcpyDeviceToDevice, s->st));
  if ((st = set_fixed_dt(s, a->t_end, dt)) != DG_OK) return st;
  collect_profile(s);
  return sync_check(s);
}

// tangent-linear run: directional derivative of the samples along (du0, db)
// from the initial state of the last dg_adjoint_forward
extern "C" dg_status dg_adjoint_tangent(dg_adjoint *a, const double *du0, const double *db,
                                        double *dsamples) {
  if (!a || a->cks.empty()) return fail(DG_BAD_ARG, "no forward run to differentiate");
  dg_solver *s = a->s;
  s->tr_valid = false;
  CK(cudaSetDevice(s->device));
  dg_status st;
  LinBufs lb;
  if ((st = lin_bufs(s, &lb)) != DG_OK) return st;
  if (!a->du) {
    if ((st = amalloc(a, &a->du, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->dw, s->ndof_p)) != DG_OK) return st;
    if ((st = amalloc(a, &a->dbi, (size_t)s->np * s->m.Kp)) != DG_OK) return st;
  }
  const size_t bytes = s->ndof_p * sizeof(double);
  const int rows = s->N * s->np;
  CK(cudaMemsetAsync(a->du, 0, bytes, s->st));
  if (du0) {
    CK(cudaMemcpyAsync(s->ubuf, du0, sizeof(double) * rows * s->K, cudaMemcpyHostToDevice,
                       s->st));
    dg::launch_permute_in(s->st, s->ubuf, a->du, s->m.perm, rows, s->K, s->m.Kp);
  }
  const double *dbp = nullptr;
  if (db) {
    CK(cudaStreamSynchronize(s->st));
    CK(cudaMemcpyAsync(s->ubuf, db, sizeof(double) * s->np * s->K, cudaMemcpyHostToDevice,
                       s->st));
    dg::launch_permute_in(s->st, s->ubuf, a->dbi, s->m.perm, s->np, s->K, s->m.Kp);
    dbp = a->dbi;
  }
  CK(cudaMemcpyAsync(s->U, a->cks[0], bytes, cudaMemcpyDeviceToDevice, s->st));
  if ((st = set_fixed_dt(s, a->t0, a->dt)) != DG_OK) return st;
  const double dt = a->dt;
  const double *dtp = &s->ds->dt;
  for (int m = 0; m < a->nsteps; m++) {
    // the tangent stage reads the stage input before the forward stage overwrites it
    tl_stage(s, s->U, a->du, dbp, nullptr, a->dw, 0.0, 1.0, dt, lb);
    stage(s, s->U, nullptr, s->W, 0.0, 1.0, 1.0, 0.0, dtp);
    tl_stage(s, s->W, a->dw, dbp, a->du, a->dw, 0.75, 0.25, 0.25 * dt, lb);
    stage(s, s->W, s->U, s->W, 0.75, 0.25, 0.25, 1.0, dtp);
    tl_stage(s, s->W, a->dw, dbp, a->du, a->du, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0 * dt, lb);
    stage(s, s->W, s->U, s->U, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0.5, dtp);
    run(s, K_CFL, [&] { dg::launch_advance_t(s->st, s->ds); });
    if ((m + 1) % a->every == 0)
      dg::launch_sample(s->st, a->du, a->rec_el, a->rec_phi, a->nrec, s->np, s->m.Kp,
                        a->sbar + (size_t)((m + 1) / a->every - 1) * a->nrec);
  }
  const int nsamp = a->nsteps / a->every;
  if (dsamples && nsamp && a->nrec)
    CK(cudaMemcpyAsync(dsamples, a->sbar, sizeof(double) * nsamp * a->nrec,
                       cudaMemcpyDeviceToHost, s->st));
  collect_profile(s);
  return sync_check(s);
}

extern "C" dg_status dg_eval_vertices(dg_solver *s, int var, double *uv) {
  return dg_eval_vertices_view(s, var, DG_VIEW_SOLUTION, 0.0, uv);
}

extern "C" dg_status dg_eval_vertices_view(dg_solver *s, int var, int view, double t,
                                           double *uv) {
  if (!s || !uv) return fail(DG_BAD_ARG, "null argument");
  if (var < 0 || var >= s->N) return fail(DG_BAD_ARG, "variable index out of range");
  if (view < DG_VIEW_SOLUTION || view > DG_VIEW_ERROR) return fail(DG_BAD_ARG, "unknown view");
  CK(cudaSetDevice(s->device));
  run(s, K_RK, [&] { s->ops->vertex(s->ctx, s->U, var, view, t, s->vbuf); });
  double *user = s->vbuf + (size_t)3 * s->m.Kp;
  dg::launch_permute_out(s->st, s->vbuf, user, s->m.perm, 3, s->K, s->m.Kp);
  CK(cudaMemcpyAsync(uv, user, (size_t)3 * s->K * sizeof(double), cudaMemcpyDeviceToHost,
                     s->st));
  collect_profile(s);
  return sync_check(s);
}

extern "C" dg_status dg_profile_enable(dg_solver *s, int on) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  collect_profile(s);
  s->profiling = on != 0;
  return DG_OK;
}

extern "C" dg_status dg_profile_get(dg_solver *s, const char *kernel, long long *launches,
                                    double *ms) {
  if (!s || !kernel) return fail(DG_BAD_ARG, "null argument");
  collect_profile(s);
  for (int k = 0; k < kKinds; k++)
    if (!std::strcmp(kernel, kKindName[k])) {
      if (launches) *launches = s->prof_n[k];
      if (ms) *ms = s->prof_ms[k];
      return DG_OK;
    }
  return fail(DG_BAD_ARG, std::string("unknown kernel name ") + kernel);
}

extern "C" dg_status dg_profile_reset(dg_solver *s) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  collect_profile(s);
  for (int k = 0; k < kKinds; k++) {
    s->prof_n[k] = 0;
    s->prof_ms[k] = 0;
  }
  return DG_OK;
}

extern "C" long long dg_kernel_launches(const dg_solver *s) { return s ? s->launches : 0; }

namespace dg {
// read-only view of a solver for entry points defined in other files
SolverView solver_view(dg_solver *s) {
  SolverView v;
  v.device = s->device;
  v.st = s->st;
  v.ops = s->ops;
  v.ctx = s->ctx;
  v.N = s->N;
  v.np = s->np;
  v.p = s->p;
  v.K = s->K;
  v.S = s->S;
  return v;
}
}  // namespace dg

// ---------------------------------------------------------------------------
// binary checkpoint / restart (the reference has none: its -V output is
// vertex values only, time_integrator.cu:426-432).  Little-endian file:
//   "DGCKPT01", int32 eq, p, N, n_p, K, has_bed, double t,
//   N*n_p*K doubles of state [var][mode][elem] (.pmsh element order),
//   n_p*K doubles of bed modes when has_bed,
//   uint64 FNV-1a hash of every byte before it.
namespace {
constexpr char kCkptMagic[8] = {'D', 'G', 'C', 'K', 'P', 'T', '0', '1'};

uint64_t fnv1a(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 0x100000001b3ull;
  return h;
}
}  // namespace

extern "C" dg_status dg_save_checkpoint(dg_solver *s, const char *path, double t) {
  if (!s || !path) return fail(DG_BAD_ARG, "null argument");
  const size_t n = (size_t)s->N * s->np * s->K, nb = (size_t)s->np * s->K;
  const int32_t hdr[6] = {(int32_t)s->eq, s->p, s->N, s->np, s->K, s->m.bathy ? 1 : 0};
  std::vector<double> u(n), b(hdr[5] ? nb : 0);
  dg_status st = dg_get_state(s, u.data());
  if (st != DG_OK) return st;
  if (hdr[5] && (st = dg_get_bathymetry(s, b.data())) != DG_OK) return st;
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(DG_IO_ERROR, std::string("cannot write ") + path);
  uint64_t h = 0xcbf29ce484222325ull;
  auto put = [&](const void *p, size_t bytes) {
    h = fnv1a(h, p, bytes);
    return std::fwrite(p, 1, bytes, f) == bytes;
  };
  bool ok = put(kCkptMagic, 8) && put(hdr, sizeof hdr) && put(&t, sizeof t) &&
            put(u.data(), n * sizeof(double)) && (b.empty() || put(b.data(), nb * sizeof(double)));
  ok = ok && std::fwrite(&h, 1, sizeof h, f) == sizeof h;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? DG_OK : fail(DG_IO_ERROR, std::string("write failed: ") + path);
}

extern "C" dg_status dg_load_checkpoint(dg_solver *s, const char *path, double *t) {
  if (!s || !path) return fail(DG_BAD_ARG, "null argument");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(DG_IO_ERROR, std::string("cannot open ") + path);
  uint64_t h = 0xcbf29ce484222325ull;
  auto get = [&](void *p, size_t bytes) {
    if (std::fread(p, 1, bytes, f) != bytes) return false;
    h = fnv1a(h, p, bytes);
    return true;
  };
  char magic[8];
  int32_t hdr[6];
  double tt = 0;
  if (!get(magic, 8) || std::memcmp(magic, kCkptMagic, 8) || !get(hdr, sizeof hdr) ||
      !get(&tt, sizeof tt)) {
    std::fclose(f);
    return fail(DG_IO_ERROR, std::string("not a checkpoint file: ") + path);
  }
  if (hdr[0] != (int32_t)s->eq || hdr[1] != s->p || hdr[2] != s->N || hdr[3] != s->np ||
      hdr[4] != s->K || (hdr[5] && s->eq != DG_SHALLOW_WATER)) {
    std::fclose(f);
    return fail(DG_BAD_ARG, "checkpoint was written for another equation, order or mesh");
  }
  const size_t n = (size_t)s->N * s->np * s->K, nb = (size_t)s->np * s->K;
  std::vector<double> u(n), b(hdr[5] ? nb : 0);
  uint64_t stored = 0;
  bool ok = get(u.data(), n * sizeof(double)) && (b.empty() || get(b.data(), nb * sizeof(double)));
  const uint64_t computed = h;
  ok = ok && std::fread(&stored, 1, sizeof stored, f) == sizeof stored;
  std::fclose(f);
  if (!ok) return fail(DG_IO_ERROR, std::string("truncated checkpoint: ") + path);
  if (stored != computed) return fail(DG_IO_ERROR, std::string("checkpoint checksum mismatch: ") + path);
  dg_status st = dg_set_state(s, u.data());
  if (st != DG_OK) return st;
  if (s->eq == DG_SHALLOW_WATER && (st = dg_set_bathymetry(s, hdr[5] ? b.data() : nullptr)) != DG_OK)
    return st;
  if (t) *t = tt;
  return DG_OK;
}

// the fused element stage's basis contractions on the tensor cores (exact
// slices, FP64 accuracy) or in FP64 FMAs; Euler p = 1..4 have the former
extern "C" dg_status dg_set_tensor_contractions(dg_solver *s, int on) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  s->tr_valid = false;
  if (on && !s->oz) return fail(DG_UNSUPPORTED, "tensor-core contractions are for Euler, p = 1..4");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->st));
  s->tensor = on != 0;
  s->ctx.oz = s->tensor ? s->oz : nullptr;
  drop_graphs(s);
  return DG_OK;
}

extern "C" dg_status dg_get_tensor_contractions(dg_solver *s, int *on) {
  if (!s || !on) return fail(DG_BAD_ARG, "null argument");
  *on = s->ctx.oz != nullptr;
  return DG_OK;
}

// advection velocity a(x, y) = (ax, ay) + grad (x, y): the reference's
// get_velocity (advection.cu:12) for fields affine in space, which covers
// every reference problem (constant in exact.cu and squarehill.cu, a solid
// rotation in rotatinghill.cu and spin.cu)
extern "C" dg_status dg_set_velocity_field(dg_solver *s, double ax, double ay,
                                           const double *grad) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  if (s->eq != DG_ADVECTION) return fail(DG_UNSUPPORTED, "a velocity field is for advection");
  if (!std::isfinite(ax) || !std::isfinite(ay)) return fail(DG_BAD_ARG, "velocity not finite");
  for (int i = 0; grad && i < 4; i++)
    if (!std::isfinite(grad[i])) return fail(DG_BAD_ARG, "velocity gradient not finite");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->st));
  s->q.ax = ax;
  s->q.ay = ay;
  for (int i = 0; i < 4; i++) s->q.agrad[i] = grad ? grad[i] : 0.0;
  field_refresh(s);
  drop_graphs(s);
  return DG_OK;
}

extern "C" dg_status dg_get_velocity_field(const dg_solver *s, double out[7]) {
  if (!s || !out) return fail(DG_BAD_ARG, "null argument");
  out[0] = s->q.ax;
  out[1] = s->q.ay;
  for (int i = 0; i < 4; i++) out[2 + i] = s->q.agrad[i];
  out[6] = s->q.field ? s->q.amax : std::sqrt(std::fma(s->q.ax, s->q.ax, s->q.ay * s->q.ay));
  return DG_OK;
}

// inflow pressure series of DG_PB_EULER_PULSE (the tube and trumpet problems'
// U_inflow, tube.cu:52-97): p(t) = 1 + sum_k amp_k cos(omega_k (t + t0) + phase_k)
extern "C" dg_status dg_set_inflow_series(dg_solver *s, int n, const double *amp,
                                          const double *omega, const double *phase, double t0) {
  if (!s) return fail(DG_BAD_ARG, "null solver");
  if (n < 0 || n > dg::kMaxSeries) return fail(DG_BAD_ARG, "the series has 0..16 terms");
  if (n > 0 && (!amp || !omega || !phase)) return fail(DG_BAD_ARG, "null argument");
  if (!std::isfinite(t0)) return fail(DG_BAD_ARG, "t0 not finite");
  for (int k = 0; k < n; k++)
    if (!std::isfinite(amp[k]) || !std::isfinite(omega[k]) || !std::isfinite(phase[k]))
      return fail(DG_BAD_ARG, "series coefficient not finite");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->st));
  s->q.nser = n;
  s->q.ser_t0 = t0;
  for (int k = 0; k < dg::kMaxSeries; k++) {
    s->q.ser[k][0] = k < n ? amp[k] : 0.0;
    s->q.ser[k][1] = k < n ? omega[k] : 0.0;
    s->q.ser[k][2] = k < n ? phase[k] : 0.0;
  }
  drop_graphs(s);
  return DG_OK;
}
