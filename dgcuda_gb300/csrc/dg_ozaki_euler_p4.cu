// dg_ozaki_euler_p4.cu -- the tensor-core Euler kernels of order 4.
#include "dg_ozaki_euler.cuh"

namespace dg {
namespace oz {
DG_OZ_EULER_INSTANCES(4)
}  // namespace oz
}  // namespace dg
