// matvec_c16.cu -- complex128 gather kernels, 16 right-hand sides per orbit scan.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_cplx_k16, true, 16)

}  // namespace lsg
