// dg_kernels_maxwell.cu -- kernel instances for the Maxwell module, p = 0..5.
#include "dg_kernels.cuh"

namespace dg {
const Ops &ops_maxwell() { return Launch<Maxwell>::ops(); }
const BatchOps &batch_ops_maxwell() { return Launch<Maxwell>::batch_ops(); }
}  // namespace dg
