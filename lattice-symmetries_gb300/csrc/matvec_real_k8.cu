// matvec_real_k8.cu -- float64 packed gather kernels (real-part semantics) for 8 and 16
// right-hand sides per orbit scan.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_real_k8, false, 8)
LSG_DEFINE_PACKED(launch_packed_real_k16, false, 16)

}  // namespace lsg
