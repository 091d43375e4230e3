// matvec_pairs_k16.cu -- complex128 gather kernels, 16 right-hand sides per orbit scan, FP32-pair
// accumulation (the FP64 form of this block is bound by GB300's FP64 pipe).
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED_PAIR(launch_packed_pair_k16, 16)

}  // namespace lsg
