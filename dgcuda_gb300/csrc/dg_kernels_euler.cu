// dg_kernels_euler.cu -- kernel instances for the Euler module, p = 0..5.
#include "dg_kernels.cuh"

namespace dg {
const Ops &ops_euler() { return Launch<Euler>::ops(); }
const BatchOps &batch_ops_euler() { return Launch<Euler>::batch_ops(); }
}  // namespace dg
