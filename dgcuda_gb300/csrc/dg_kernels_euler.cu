// dg_kernels_euler.cu -- kernel instances for the Euler module, p = 0..5;
// the fused element stage runs on the tensor cores (dg_ozaki.cuh) for
// p = 1..4 when the solver has built its tables (Ctx::oz).
#include "dg_ozaki.cuh"

namespace dg {
namespace {

using L = Launch<Euler>;

template <int P>
void oz_element(const Ctx &c, const ElemArgs &a) {
  const unsigned blocks = (unsigned)((c.m.K + oz::kOzElems - 1) / oz::kOzElems);
  oz::k_element_oz<Euler, P><<<blocks, oz::kOzThreads, oz::oz_smem_bytes<Euler, P>(), c.st>>>(
      L::tab<P>(c), *c.q, a, static_cast<const oz::Tabs *>(c.oz));
}

void element_tr(const Ctx &c, double *us, const double *un, double *out, double ca, double cb,
                double cc, const double *dtp, int check) {
  if (!c.oz || c.p < 1 || c.p > 4) {
    L::element_tr(c, us, un, out, ca, cb, cc, dtp, check);
    return;
  }
  if (!c.m.K) return;
  const ElemArgs a = L::eargs(c, us, un, out, ca, cb, cc, dtp, c.T, check);
  switch (c.p) {
    case 1: oz_element<1>(c, a); break;
    case 2: oz_element<2>(c, a); break;
    case 3: oz_element<3>(c, a); break;
    case 4: oz_element<4>(c, a); break;
  }
}

void trace(const Ctx &c, double *u) {
  if (!c.oz || c.p < 1 || c.p > 4) {
    L::trace(c, u);
    return;
  }
  if (!c.m.K) return;
  const unsigned blocks = (unsigned)((c.m.K + oz::kOzElems - 1) / oz::kOzElems);
  const oz::Tabs *t = static_cast<const oz::Tabs *>(c.oz);
  switch (c.p) {
    case 1: oz::k_trace_oz<Euler, 1><<<blocks, oz::kOzThreads, 0, c.st>>>(L::tab<1>(c), *c.q, u, c.T, c.m.K, c.m.Kp, t); break;
    case 2: oz::k_trace_oz<Euler, 2><<<blocks, oz::kOzThreads, 0, c.st>>>(L::tab<2>(c), *c.q, u, c.T, c.m.K, c.m.Kp, t); break;
    case 3: oz::k_trace_oz<Euler, 3><<<blocks, oz::kOzThreads, 0, c.st>>>(L::tab<3>(c), *c.q, u, c.T, c.m.K, c.m.Kp, t); break;
    case 4: oz::k_trace_oz<Euler, 4><<<blocks, oz::kOzThreads, 0, c.st>>>(L::tab<4>(c), *c.q, u, c.T, c.m.K, c.m.Kp, t); break;
  }
}

Ops make_ops() {
  Ops o = L::ops();
  o.element_tr = element_tr;
  o.trace = trace;
  return o;
}

template <int P>
cudaError_t oz_attr() {
  return cudaFuncSetAttribute(oz::k_element_oz<Euler, P>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)oz::oz_smem_bytes<Euler, P>());
}

}  // namespace

const Ops &ops_euler() {
  static const Ops o = make_ops();
  return o;
}
const BatchOps &batch_ops_euler() { return Launch<Euler>::batch_ops(); }

// allows the tensor-core element kernel of order p its shared memory (once
// per device, before any capture)
cudaError_t oz_prepare_euler(int p) {
  switch (p) {
    case 1: return oz_attr<1>();
    case 2: return oz_attr<2>();
    case 3: return oz_attr<3>();
    case 4: return oz_attr<4>();
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace dg
