// matvec_pairs_k8.cu -- complex128 gather kernels, 8 right-hand sides per orbit scan, FP32-pair
// accumulation.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED_PAIR(launch_packed_pair_k8, 8)

}  // namespace lsg
