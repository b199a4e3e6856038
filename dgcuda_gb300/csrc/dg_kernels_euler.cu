// dg_kernels_euler.cu -- kernel instances for the Euler module, p = 0..5;
// the fused element stage runs on the tensor cores (dg_ozaki.cuh, one
// translation unit per order: dg_ozaki_euler_p*.cu) for p = 1..4 when the
// solver has built its tables (Ctx::oz), with the limiter in its epilogue
// when the limiter is on (element_lim).
#include "dg_ozaki_euler.cuh"

namespace dg {
namespace {

using L = Launch<Euler>;

void oz_element(const Ctx &c, const ElemArgs &a, bool lim) {
  switch (c.p) {
    case 1: oz::euler_element<1>(c, a, lim); break;
    case 2: oz::euler_element<2>(c, a, lim); break;
    case 3: oz::euler_element<3>(c, a, lim); break;
    case 4: oz::euler_element<4>(c, a, lim); break;
  }
}

void element_tr(const Ctx &c, double *us, const double *un, double *out, double ca, double cb,
                double cc, const double *dtp, int check) {
  if (!c.oz || c.p < 1 || c.p > 4) {
    L::element_tr(c, us, un, out, ca, cb, cc, dtp, check);
    return;
  }
  if (!c.m.K) return;
  oz_element(c, L::eargs(c, us, un, out, ca, cb, cc, dtp, c.T, check), false);
}

// the element stage with the limiter in its epilogue (M holds the output's
// means from k_means): the tensor-core kernel, or the FP64 one
void element_lim(const Ctx &c, double *us, const double *un, double *out, double ca, double cb,
                 double cc, const double *dtp) {
  if (!c.oz || c.p < 1 || c.p > 4) {
    L::element_lim(c, us, un, out, ca, cb, cc, dtp);
    return;
  }
  if (!c.m.K) return;
  oz_element(c, L::eargs(c, us, un, out, ca, cb, cc, dtp, c.T, 0), true);
}

void trace(const Ctx &c, double *u) {
  if (!c.oz || c.p < 1 || c.p > 4) {
    L::trace(c, u);
    return;
  }
  if (!c.m.K) return;
  switch (c.p) {
    case 1: oz::euler_trace<1>(c, u); break;
    case 2: oz::euler_trace<2>(c, u); break;
    case 3: oz::euler_trace<3>(c, u); break;
    case 4: oz::euler_trace<4>(c, u); break;
  }
}

Ops make_ops() {
  Ops o = L::ops();
  o.element_tr = element_tr;
  o.trace = trace;
  o.face_fs = L::face_fs;
  o.means = L::means;
  o.element_lim = element_lim;
  return o;
}

}  // namespace

const Ops &ops_euler() {
  static const Ops o = make_ops();
  return o;
}
const BatchOps &batch_ops_euler() {
  static const BatchOps o = [] {
    BatchOps b = Launch<Euler>::batch_ops();
    b.face_fs = Launch<Euler>::b_face_fs;
    b.means = Launch<Euler>::b_means;
    b.element_lim = Launch<Euler>::b_element_lim;
    return b;
  }();
  return o;
}

// allows the tensor-core element kernels of order p their shared memory
// (once per device, before any capture)
cudaError_t oz_prepare_euler(int p) {
  switch (p) {
    case 1: return oz::euler_prepare<1>();
    case 2: return oz::euler_prepare<2>();
    case 3: return oz::euler_prepare<3>();
    case 4: return oz::euler_prepare<4>();
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace dg
