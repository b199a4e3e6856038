// dg_adjoint.cu -- launchers of the shallow-water tangent-linear and
// adjoint kernels (dg_adjoint.cuh), orders p = 1..4.
#include "dg_adjoint.cuh"

namespace dg {

namespace {
template <int P>
const Tab<P> &tabp(const Ctx &c) {
  return *reinterpret_cast<const Tab<P> *>(c.tab);
}
#define DG_LIN_P(expr)                             \
  switch (c.p) {                                   \
    case 1: { constexpr int P = 1; expr; } break;  \
    case 2: { constexpr int P = 2; expr; } break;  \
    case 3: { constexpr int P = 3; expr; } break;  \
    case 4: { constexpr int P = 4; expr; } break;  \
    default: return false;                         \
  }
}  // namespace

bool lin_supported(int p) { return p >= 1 && p <= 4; }

bool lin_trace(const Ctx &c, const double *u, const double *scale, double sc, double *Tv) {
  DG_LIN_P((k_lin_trace<P><<<nblk(c.m.K), kBlock, 0, c.st>>>(tabp<P>(c), u, scale, sc, Tv,
                                                              c.m.K, c.m.Kp)));
  return true;
}

bool tl_face(const Ctx &c, const double *Tv, double *dFh) {
  DG_LIN_P((k_sw_face_lin<P, false><<<nblk(c.m.S), kBlock, 0, c.st>>>(
      tabp<P>(c), *c.q, c.T, Tv, c.m.side, c.m.sgeo, dFh, nullptr, c.m.S)));
  return true;
}

bool adj_face(const Ctx &c, const double *Tbar, double *UbL, double *UbR) {
  DG_LIN_P((k_sw_face_lin<P, true><<<nblk(c.m.S), kBlock, 0, c.st>>>(
      tabp<P>(c), *c.q, c.T, Tbar, c.m.side, c.m.sgeo, UbL, UbR, c.m.S)));
  return true;
}

bool tl_element(const Ctx &c, const double *us, const double *dus, const double *db,
                const double *dun, double *dout, double ca, double cb, double ccdt) {
  DG_LIN_P((k_sw_element_lin<P, false><<<nblk(c.m.K), kBlock, 0, c.st>>>(
      tabp<P>(c), *c.q, us, c.m.bathy, dus, db, dun, dout, nullptr, c.Fh, nullptr, c.m.esd,
      c.m.geo, ca, cb, ccdt, c.m.K, c.m.Kp)));
  return true;
}

bool adj_element(const Ctx &c, const double *us, const double *obar, double *ubar_s,
                 double *bbar, const double *UbL, const double *UbR, double cb, double ccdt) {
  DG_LIN_P((k_sw_element_lin<P, true><<<nblk(c.m.K), kBlock, 0, c.st>>>(
      tabp<P>(c), *c.q, us, c.m.bathy, obar, nullptr, obar, ubar_s, bbar, UbL, UbR, c.m.esd,
      c.m.geo, 0.0, cb, ccdt, c.m.K, c.m.Kp)));
  return true;
}

// ---- receivers: h at points, and the adjoint of that sampling ----
__global__ void k_sample(const double *__restrict__ u, const int *__restrict__ el,
                         const double *__restrict__ phi, int nrec, int np, int Kp,
                         double *__restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  double a = 0.0;
  for (int i = 0; i < np; i++) a = fma(u[(size_t)i * Kp + el[r]], phi[(size_t)r * np + i], a);
  out[r] = a;
}
// one thread: receivers that share an element add in a fixed order
__global__ void k_sample_adj(double *__restrict__ ubar, const int *__restrict__ el,
                             const double *__restrict__ phi, int nrec, int np, int Kp,
                             const double *__restrict__ sbar) {
  if (blockIdx.x * blockDim.x + threadIdx.x != 0) return;
  for (int r = 0; r < nrec; r++)
    for (int i = 0; i < np; i++)
      ubar[(size_t)i * Kp + el[r]] = fma(sbar[r], phi[(size_t)r * np + i],
                                          ubar[(size_t)i * Kp + el[r]]);
}

void launch_sample(cudaStream_t st, const double *u, const int *el, const double *phi, int nrec,
                   int np, int Kp, double *out) {
  if (nrec) k_sample<<<(nrec + 127) / 128, 128, 0, st>>>(u, el, phi, nrec, np, Kp, out);
}
void launch_sample_adj(cudaStream_t st, double *ubar, const int *el, const double *phi, int nrec,
                       int np, int Kp, const double *sbar) {
  if (nrec) k_sample_adj<<<1, 32, 0, st>>>(ubar, el, phi, nrec, np, Kp, sbar);
}

}  // namespace dg
