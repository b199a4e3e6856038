// dg_ozaki_euler_p2.cu -- the tensor-core Euler kernels of order 2.
#include "dg_ozaki_euler.cuh"

namespace dg {
namespace oz {
DG_OZ_EULER_INSTANCES(2)
}  // namespace oz
}  // namespace dg
