// matvec_c4.cu -- complex128 gather kernels, 4 right-hand sides per orbit scan.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_cplx_k4, true, 4)

}  // namespace lsg
