// dg_ozaki_euler_p1.cu -- the tensor-core Euler kernels of order 1.
#include "dg_ozaki_euler.cuh"

namespace dg {
namespace oz {
DG_OZ_EULER_INSTANCES(1)
}  // namespace oz
}  // namespace dg
