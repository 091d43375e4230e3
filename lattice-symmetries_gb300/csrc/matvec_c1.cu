// matvec_c1.cu -- complex128 gather kernels, one right-hand side per orbit scan.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_cplx_k1, true, 1)
LSG_DEFINE_FALLBACK(launch_projected_cplx_k1, true)

}  // namespace lsg
