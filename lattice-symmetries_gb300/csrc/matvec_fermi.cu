// matvec_fermi.cu -- packed gather kernels for spinful fermions with lattice symmetries (the
// group acts with fermionic permutation signs): complex K in {1, 4, 8, 16} and the real K = 1
// path, groups of up to 128 elements.
#include <type_traits>

#include "matvec_launch.cuh"

namespace lsg {

int launch_packed_fermi(bool cplx, int k, int gpl, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,
                        const double* x, int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom,
                        cudaStream_t s) {
  auto with_k = [&](auto gtag) -> int {
    constexpr int G = decltype(gtag)::value;
    if (!cplx) {
      if (k != 1) return LS_GPU_ERR_INVALID;
      return launch_with_smem(k_matvec_packed<G, false, false, 1, true>, "k_matvec_packed<fermi>", p, L, sh, x,
                              ldx, y, ldy, err, binom, s);
    }
    switch (k) {
      case 1: return launch_with_smem(k_matvec_packed<G, false, true, 1, true>, "k_matvec_packed<fermi>", p, L, sh,
                                      x, ldx, y, ldy, err, binom, s);
      case 4: return launch_with_smem(k_matvec_packed<G, false, true, 4, true>, "k_matvec_packed<fermi>", p, L, sh,
                                      x, ldx, y, ldy, err, binom, s);
      case 8: return launch_with_smem(k_matvec_packed<G, false, true, 8, true>, "k_matvec_packed<fermi>", p, L, sh,
                                      x, ldx, y, ldy, err, binom, s);
      case 16: return launch_with_smem(k_matvec_packed<G, false, true, 16, true>, "k_matvec_packed<fermi>", p, L,
                                       sh, x, ldx, y, ldy, err, binom, s);
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
