// matvec_real_k.cu -- float64 packed gather kernels (real-part semantics) for 2 and 4 right-hand
// sides per orbit scan (several real vectors through one reference-facing call).
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_real_k2, false, 2)
LSG_DEFINE_PACKED(launch_packed_real_k4, false, 4)

}  // namespace lsg
