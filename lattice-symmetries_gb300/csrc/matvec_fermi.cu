// matvec_fermi.cu -- packed gather kernels for spinful fermions with lattice symmetries (the
// group acts with fermionic permutation signs): complex K in {1, 4, 8, 16} and the real K = 1
// path, groups of up to 128 elements.
#include <type_traits>

#include "matvec_launch.cuh"

namespace lsg {

int launch_packed_fermi(bool cplx, int k, int gpl, const MatvecProblem& p, const double* x, int64_t ldx, double* y,
                        int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {
  auto with_k = [&](auto gtag) -> int {
    constexpr int G = decltype(gtag)::value;
    auto go = [&](auto kern, int max_threads) {
      return launch_packed_kernel(kern, max_threads, "k_matvec_packed<fermi>", p, x, ldx, y, ldy, err, binom, s);
    };
    if (!cplx) {
      if (k != 1) return LS_GPU_ERR_INVALID;
      return go(k_matvec_packed<G, false, false, 1, true>, PackedBounds<G, 1, false, false>::threads);
    }
    switch (k) {
      case 1: return go(k_matvec_packed<G, false, true, 1, true>, PackedBounds<G, 1, false>::threads);
      case 4: return go(k_matvec_packed<G, false, true, 4, true>, PackedBounds<G, 4, false>::threads);
      case 8: return go(k_matvec_packed<G, false, true, 8, true>, PackedBounds<G, 8, false>::threads);
      case 16: return go(k_matvec_packed<G, false, true, 16, true>, PackedBounds<G, 16, false>::threads);
      default: return LS_GPU_ERR_INVALID;
    }
  };
  switch (gpl) {
    case 1: return with_k(std::integral_constant<int, 1>{});
    case 2: return with_k(std::integral_constant<int, 2>{});
    case 3: return with_k(std::integral_constant<int, 3>{});
    case 4: return with_k(std::integral_constant<int, 4>{});
    default: return fail(LS_GPU_ERR_INVALID, "fermionic lattice symmetries: at most 128 group elements");
  }
}

}  // namespace lsg
