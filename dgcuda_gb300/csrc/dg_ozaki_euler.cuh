// dg_ozaki_euler.cuh -- launchers of the tensor-core Euler kernels of one
// order P (dg_ozaki.cuh): the fused element stage, with or without the
// limiter in its epilogue, and the start-of-run traces.  Each order is
// instantiated in a translation unit of its own (dg_ozaki_euler_p<P>.cu) so
// that the heaviest kernels compile in parallel; dg_kernels_euler.cu
// dispatches on p.
#pragma once
#include "dg_pipeline.cuh"

namespace dg {
namespace oz {

template <int P>
void euler_element(const Ctx &c, const ElemArgs &a, bool lim) {
  const unsigned blocks = (unsigned)((c.m.K + kOzElems - 1) / kOzElems);
  const Tab<P> &tab = *reinterpret_cast<const Tab<P> *>(c.tab);
  const Tabs *t = static_cast<const Tabs *>(c.oz);
  if (lim)
    k_element_oz<Euler, P, true><<<blocks, kOzThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, t);
  else
    k_element_oz<Euler, P, false><<<blocks, kOzThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, t);
}

template <int P>
void euler_trace(const Ctx &c, double *u) {
  const unsigned blocks = (unsigned)((c.m.K + kOzElems - 1) / kOzElems);
  const Tab<P> &tab = *reinterpret_cast<const Tab<P> *>(c.tab);
  k_trace_oz<Euler, P><<<blocks, kOzThreads, 0, c.st>>>(tab, *c.q, u, c.T, c.m.K, c.m.Kp,
                                                        static_cast<const Tabs *>(c.oz));
}

// the pipelined stage: one persistent launch over the work list c.pipe[lim]
template <int P>
void euler_stage_pipe(const Ctx &c, const ElemArgs &a, const FaceArgs &fa, int lim) {
  const Tab<P> &tab = *reinterpret_cast<const Tab<P> *>(c.tab);
  const Tabs *t = static_cast<const Tabs *>(c.oz);
  const PipeArgs &pa = c.pipe[lim ? 1 : 0];
  if (lim)
    k_stage_oz<Euler, P, true><<<pa.grid, kOzThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, fa, pa, c.M, t);
  else
    k_stage_oz<Euler, P, false><<<pa.grid, kOzThreads, oz_smem_bytes<Euler, P>(), c.st>>>(
        tab, *c.q, a, fa, pa, c.M, t);
}

template <class F>
cudaError_t smem_attr(F *f, int bytes) {
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// allows the element and pipelined-stage kernels of order P their shared
// memory (once per device, before any capture); *per_sm: resident blocks of
// the pipelined stage per SM
template <int P>
cudaError_t euler_prepare(int *per_sm) {
  const int b = (int)oz_smem_bytes<Euler, P>();
  cudaError_t e;
  if ((e = smem_attr(k_element_oz<Euler, P, false>, b)) != cudaSuccess) return e;
  if ((e = smem_attr(k_element_oz<Euler, P, true>, b)) != cudaSuccess) return e;
  if ((e = smem_attr(k_stage_oz<Euler, P, false>, b)) != cudaSuccess) return e;
  if ((e = smem_attr(k_stage_oz<Euler, P, true>, b)) != cudaSuccess) return e;
  int n0 = 0, n1 = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_stage_oz<Euler, P, false>,
                                                         kOzThreads, b)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_stage_oz<Euler, P, true>,
                                                         kOzThreads, b)) != cudaSuccess)
    return e;
  *per_sm = n0 < n1 ? n0 : n1;
  return cudaSuccess;
}

#define DG_OZ_EULER_INSTANCES(P)                                                  \
  template void euler_element<P>(const Ctx &, const ElemArgs &, bool);           \
  template void euler_trace<P>(const Ctx &, double *);                           \
  template void euler_stage_pipe<P>(const Ctx &, const ElemArgs &, const FaceArgs &, int); \
  template cudaError_t euler_prepare<P>(int *);

#define DG_OZ_EULER_DECLARE(P)                                                           \
  extern template void euler_element<P>(const Ctx &, const ElemArgs &, bool);             \
  extern template void euler_trace<P>(const Ctx &, double *);                             \
  extern template void euler_stage_pipe<P>(const Ctx &, const ElemArgs &, const FaceArgs &, \
                                           int);                                          \
  extern template cudaError_t euler_prepare<P>(int *);

DG_OZ_EULER_DECLARE(1)
DG_OZ_EULER_DECLARE(2)
DG_OZ_EULER_DECLARE(3)
DG_OZ_EULER_DECLARE(4)

}  // namespace oz
}  // namespace dg
