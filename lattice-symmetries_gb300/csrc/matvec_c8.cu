// matvec_c8.cu -- complex128 gather kernels, 8 right-hand sides per orbit scan.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_cplx_k8, true, 8)

}  // namespace lsg
