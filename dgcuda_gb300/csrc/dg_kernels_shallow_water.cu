// dg_kernels_shallow_water.cu -- kernel instances for the ShallowWater module, p = 0..5.
#include "dg_kernels.cuh"

namespace dg {
const Ops &ops_shallow_water() { return Launch<ShallowWater>::ops(); }
const BatchOps &batch_ops_shallow_water() { return Launch<ShallowWater>::batch_ops(); }
}  // namespace dg
