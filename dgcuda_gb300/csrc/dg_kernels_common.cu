// dg_kernels_common.cu -- table images, layout permutation, RK combinations
// and the device-side CFL step.
#include <cstring>

#include "dg_device.cuh"
#include "dg_launch.h"

namespace dg {

template <int P>
static void fill_tab(const dg_order_tables &s, Tab<P> *t) {
  constexpr int NP = Tab<P>::NP, NQ = Tab<P>::NQ, N1 = Tab<P>::N1;
  for (int q = 0; q < NQ; q++) {
    for (int i = 0; i < NP; i++) {
      t->B[q][i] = s.B[q][i];
      t->GR[q][i] = s.GR[q][i];
      t->GS[q][i] = s.GS[q][i];
    }
    t->r[q] = s.r[q];
    t->s[q] = s.s[q];
    t->w[q] = s.w[q];
  }
  for (int f = 0; f < 3; f++)
    for (int j = 0; j < N1; j++)
      for (int i = 0; i < NP; i++) t->E[f][j][i] = s.E[f][j][i];
  for (int j = 0; j < N1; j++) {
    t->t1[j] = s.t1[j];
    t->w1[j] = s.w1[j];
  }
  for (int v = 0; v < 3; v++)
    for (int i = 0; i < NP; i++) t->V[v][i] = s.V[v][i];
}

size_t tab_bytes(int p) {
  switch (p) {
    case 0: return sizeof(Tab<0>);
    case 1: return sizeof(Tab<1>);
    case 2: return sizeof(Tab<2>);
    case 3: return sizeof(Tab<3>);
    case 4: return sizeof(Tab<4>);
    case 5: return sizeof(Tab<5>);
  }
  return 0;
}

void build_tab(int p, const dg_order_tables &src, void *dst) {
  switch (p) {
    case 0: fill_tab<0>(src, static_cast<Tab<0> *>(dst)); break;
    case 1: fill_tab<1>(src, static_cast<Tab<1> *>(dst)); break;
    case 2: fill_tab<2>(src, static_cast<Tab<2> *>(dst)); break;
    case 3: fill_tab<3>(src, static_cast<Tab<3> *>(dst)); break;
    case 4: fill_tab<4>(src, static_cast<Tab<4> *>(dst)); break;
    case 5: fill_tab<5>(src, static_cast<Tab<5> *>(dst)); break;
  }
}

static constexpr int kB = 256;
static unsigned grid_for(size_t n) { return (unsigned)((n + kB - 1) / kB); }

__global__ void k_permute_in(const double *__restrict__ user, double *__restrict__ in,
                             const int *__restrict__ perm, int rows, int K, int Kp) {
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)rows * Kp) return;
  int r = (int)(idx / Kp), e = (int)(idx % Kp);
  in[idx] = e < K ? user[(size_t)r * K + perm[e]] : 0.0;
}

__global__ void k_permute_out(const double *__restrict__ in, double *__restrict__ user,
                              const int *__restrict__ perm, int rows, int K, int Kp) {
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)rows * K) return;
  int r = (int)(idx / K), e = (int)(idx % K);
  user[(size_t)r * K + perm[e]] = in[(size_t)r * Kp + e];
}

void launch_permute_in(cudaStream_t st, const double *user, double *internal, const int *perm,
                       int rows, int K, int Kp) {
  size_t n = (size_t)rows * Kp;
  if (n) k_permute_in<<<grid_for(n), kB, 0, st>>>(user, internal, perm, rows, K, Kp);
}

// permute_in that also sets *changed when any value differs (bitwise) from
// the one it overwrites
__global__ void k_permute_in_cmp(const double *__restrict__ user, double *__restrict__ in,
                                 const int *__restrict__ perm, int rows, int K, int Kp,
                                 int *changed) {
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)rows * Kp) return;
  int r = (int)(idx / Kp), e = (int)(idx % Kp);
  const double v = e < K ? user[(size_t)r * K + perm[e]] : 0.0;
  if (__double_as_longlong(in[idx]) != __double_as_longlong(v)) *changed = 1;
  in[idx] = v;
}

void launch_permute_in_cmp(cudaStream_t st, const double *user, double *internal,
                           const int *perm, int rows, int K, int Kp, int *changed) {
  size_t n = (size_t)rows * Kp;
  if (n) k_permute_in_cmp<<<grid_for(n), kB, 0, st>>>(user, internal, perm, rows, K, Kp, changed);
}

void launch_permute_out(cudaStream_t st, const double *internal, double *user, const int *perm,
                        int rows, int K, int Kp) {
  size_t n = (size_t)rows * K;
  if (n) k_permute_out<<<grid_for(n), kB, 0, st>>>(internal, user, perm, rows, K, Kp);
}

__global__ void k_axpby(int n, double a, const double *__restrict__ x, double b, double *y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}
__global__ void k_xpay(int n, const double *x, double a, const double *y, double *z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = x[i] + a * y[i];  // rk_tempstorage, time_integrator.cu:107-113
}
__global__ void k_rk4_final(int n, double *c, const double *__restrict__ k1,
                            const double *__restrict__ k2, const double *__restrict__ k3,
                            const double *__restrict__ k4) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;  // rk4, time_integrator.cu:124-130
  if (i < n) c[i] += k1[i] / 6. + k2[i] / 3. + k3[i] / 3. + k4[i] / 6.;
}

void launch_axpby(cudaStream_t st, int n, double a, const double *x, double b, double *y) {
  if (n) k_axpby<<<grid_for(n), kB, 0, st>>>(n, a, x, b, y);
}
void launch_xpay(cudaStream_t st, int n, const double *x, double a, const double *y, double *z) {
  if (n) k_xpay<<<grid_for(n), kB, 0, st>>>(n, x, a, y, z);
}
void launch_rk4_final(cudaStream_t st, int n, double *c, const double *k1, const double *k2,
                      const double *k3, const double *k4) {
  if (n) k_rk4_final<<<grid_for(n), kB, 0, st>>>(n, c, k1, k2, k3, k4);
}

// dt = cfl * d_min / lambda_max / (2p + 1) (time_integrator.cu:217), the
// last step shortened to land on endtime (:226-231)
__device__ __forceinline__ void compute_dt_body(DevScalars *ds, int p) {
  double lam = __longlong_as_double((long long)ds->lam_bits);
  double dt = ds->fixed_dt > 0 ? ds->fixed_dt : ds->cfl * ds->dmin / lam / (2. * p + 1.);
  if (!(dt == dt) || !(dt > 0) || isinf(dt)) {
    ds->status = 4;
    dt = 0.0;
  }
  ds->last = 0;
  if (ds->endtime > 0) {
    if (ds->t + dt > ds->endtime) {
      dt = ds->endtime - ds->t;
      ds->last = 1;
    }
    if (dt < 0) dt = 0;
  }
  ds->dt = dt;
}
__device__ __forceinline__ void advance_t_body(DevScalars *ds) {
  if (ds->dt > 0) ds->steps++;
  ds->t = ds->last ? ds->endtime : ds->t + ds->dt;
}
__global__ void k_compute_dt(DevScalars *ds, int p) { compute_dt_body(ds, p); }
__global__ void k_reset_lambda(DevScalars *ds) { ds->lam_bits = 0ull; }
__global__ void k_advance_t(DevScalars *ds) { advance_t_body(ds); }

// one thread per problem of a batch
__global__ void k_batch_reset_lambda(BatchProb *pr, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pr[i].ds->lam_bits = 0ull;
}
__global__ void k_batch_compute_dt(BatchProb *pr, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) compute_dt_body(pr[i].ds, pr[i].p);
}
__global__ void k_batch_advance_t(BatchProb *pr, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) advance_t_body(pr[i].ds);
}
void launch_batch_reset_lambda(cudaStream_t st, BatchProb *probs, int n) {
  if (n) k_batch_reset_lambda<<<grid_for(n), kB, 0, st>>>(probs, n);
}
void launch_batch_compute_dt(cudaStream_t st, BatchProb *probs, int n) {
  if (n) k_batch_compute_dt<<<grid_for(n), kB, 0, st>>>(probs, n);
}
void launch_batch_advance_t(cudaStream_t st, BatchProb *probs, int n) {
  if (n) k_batch_advance_t<<<grid_for(n), kB, 0, st>>>(probs, n);
}

struct BatchTabsImage {
  Tab<1> t1;
  Tab<2> t2;
  Tab<3> t3;
};
size_t batch_tabs_bytes() { return sizeof(BatchTabsImage); }
void build_batch_tabs(const void *t1, const void *t2, const void *t3, void *dst) {
  BatchTabsImage *b = static_cast<BatchTabsImage *>(dst);
  if (t1) std::memcpy(&b->t1, t1, sizeof(Tab<1>));
  if (t2) std::memcpy(&b->t2, t2, sizeof(Tab<2>));
  if (t3) std::memcpy(&b->t3, t3, sizeof(Tab<3>));
}

void launch_compute_dt(cudaStream_t st, DevScalars *ds, int p) { k_compute_dt<<<1, 1, 0, st>>>(ds, p); }
void launch_reset_lambda(cudaStream_t st, DevScalars *ds) { k_reset_lambda<<<1, 1, 0, st>>>(ds); }
void launch_advance_t(cudaStream_t st, DevScalars *ds) { k_advance_t<<<1, 1, 0, st>>>(ds); }

}  // namespace dg
