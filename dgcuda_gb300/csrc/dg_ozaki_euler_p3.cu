// dg_ozaki_euler_p3.cu -- the tensor-core Euler kernels of order 3.
#include "dg_ozaki_euler.cuh"

namespace dg {
namespace oz {
DG_OZ_EULER_INSTANCES(3)
}  // namespace oz
}  // namespace dg
