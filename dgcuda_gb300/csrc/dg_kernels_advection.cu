// dg_kernels_advection.cu -- kernel instances for the Advection module, p = 0..5.
#include "dg_kernels.cuh"

namespace dg {
const Ops &ops_advection() { return Launch<Advection>::ops(); }
const BatchOps &batch_ops_advection() { return Launch<Advection>::batch_ops(); }
}  // namespace dg
