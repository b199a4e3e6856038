// dg_ozaki_euler.cuh -- launchers of the tensor-core Euler kernels of one
// order P (dg_ozaki.cuh): the fused element stage, with or without the
// limiter in its epilogue, and the start-of-run traces.  Each order is
// instantiated in a translation unit of its own (dg_ozaki_euler_p<P>.cu) so
// that the heaviest kernels compile in parallel; dg_kernels_euler.cu
// dispatches on p.
#pragma once
#include "dg_ozaki.cuh"

namespace dg {
namespace oz {

template <int P>
void euler_element(const Ctx &c, const ElemArgs &a, bool lim) {
  using B = OzBlock<P>;
  const unsigned blocks = (unsigned)((c.m.K + B::kElems - 1) / B::kElems);
  const Tab<P> &tab = *reinterpret_cast<const Tab<P> *>(c.tab);
  const Tabs *t = static_cast<const Tabs *>(c.oz);
  if (lim)
    k_element_oz<Euler, P, true><<<blocks, B::kThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, t);
  else
    k_element_oz<Euler, P, false><<<blocks, B::kThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, t);
}

template <int P>
void euler_trace(const Ctx &c, double *u) {
  const unsigned blocks = (unsigned)((c.m.K + kOzElems - 1) / kOzElems);
  const Tab<P> &tab = *reinterpret_cast<const Tab<P> *>(c.tab);
  k_trace_oz<Euler, P><<<blocks, kOzThreads, 0, c.st>>>(tab, *c.q, u, c.T, c.m.K, c.m.Kp,
                                                        static_cast<const Tabs *>(c.oz));
}

// allows both element kernels of order P their shared memory (once per
// device, before any capture)
template <int P>
cudaError_t euler_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_element_oz<Euler, P, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)oz_smem_bytes<Euler, P>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_element_oz<Euler, P, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)oz_smem_bytes<Euler, P>());
}

#define DG_OZ_EULER_INSTANCES(P)                                        \
  template void euler_element<P>(const Ctx &, const ElemArgs &, bool); \
  template void euler_trace<P>(const Ctx &, double *);                 \
  template cudaError_t euler_prepare<P>();

#define DG_OZ_EULER_DECLARE(P)                                                \
  extern template void euler_element<P>(const Ctx &, const ElemArgs &, bool); \
  extern template void euler_trace<P>(const Ctx &, double *);                 \
  extern template cudaError_t euler_prepare<P>();

DG_OZ_EULER_DECLARE(1)
DG_OZ_EULER_DECLARE(2)
DG_OZ_EULER_DECLARE(3)
DG_OZ_EULER_DECLARE(4)

}  // namespace oz
}  // namespace dg
