// matvec_pairs_sec.cu -- FP32-pair variants of the batched multi-sector kernel and of the
// fermionic packed kernel (complex, K in {8, 16}), and the dispatch of the FP32-pair kernels.
#include <type_traits>

#include "matvec_launch.cuh"

namespace lsg {

LSG_DECLARE_PACKED(launch_packed_pair_k8)
LSG_DECLARE_PACKED(launch_packed_pair_k16)

int launch_packed_pair(int k, int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx, double* y,
                       int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {
  if (p.xs == nullptr) return fail(LS_GPU_ERR_INVALID, "pair kernels gather from a prescaled pair copy of x");
  if (p.group.fermionic) {
    if (inv) return fail(LS_GPU_ERR_INVALID, "fermionic groups have no spin inversion");
    auto with_k = [&](auto gtag) -> int {
      constexpr int G = decltype(gtag)::value;
      switch (k) {
        case 8: return launch_packed_kernel(k_matvec_packed<G, false, true, 8, true, true>,
                                            PackedBounds<G, 8, true>::threads, "k_matvec_packed<fermi,pair>", p, x,
                                            ldx, y, ldy, err, binom, s);
        case 16: return launch_packed_kernel(k_matvec_packed<G, false, true, 16, true, true>,
                                             PackedBounds<G, 16, true>::threads, "k_matvec_packed<fermi,pair>", p, x,
                                             ldx, y, ldy, err, binom, s);
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
  switch (k) {
    case 8: return launch_packed_pair_k8(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    case 16: return launch_packed_pair_k16(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    default: return LS_GPU_ERR_INVALID;
  }
}

int launch_sectors_pair(int k, int gpl, bool inv, const MatvecProblem& p, int n_sectors_layout,
                        const SectorDesc* d_desc, int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy,
                        int* err, const uint64_t* binom, const double* xs_all, int64_t ldxs, int col,
                        cudaStream_t s) {
  if (xs_all == nullptr) return fail(LS_GPU_ERR_INVALID, "pair kernels gather from a prescaled pair copy of x");
  auto go = [&](auto kern) -> int {
    LaunchShape sh{};
    PackedLayout L{};
    const int rc = packed_launch_shape((const void*)kern, 320, p, n_sectors_layout, total_rows, &sh, &L);
    if (rc != 0) return rc;
    kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, d_desc, n_sectors, total_rows, ldx, ldy, err, binom, xs_all,
                                                ldxs, col);
    return cuda_ok(cudaGetLastError(), "k_matvec_sectors<pair>") ? 0 : LS_GPU_ERR_CUDA;
  };
  auto with_k = [&](auto gtag, auto itag) -> int {
    constexpr int G = decltype(gtag)::value;
    constexpr bool I = decltype(itag)::value;
    switch (k) {
      case 8: return go(k_matvec_sectors<G, I, 8, true>);
      case 16: return go(k_matvec_sectors<G, I, 16, true>);
      default: return LS_GPU_ERR_INVALID;
    }
  };
  auto with_inv = [&](auto gtag) -> int {
    return inv ? with_k(gtag, std::true_type{}) : with_k(gtag, std::false_type{});
  };
  switch (gpl) {
    case 1: return with_inv(std::integral_constant<int, 1>{});
    case 2: return with_inv(std::integral_constant<int, 2>{});
    case 3: return with_inv(std::integral_constant<int, 3>{});
    case 4: return with_inv(std::integral_constant<int, 4>{});
    default: return LS_GPU_ERR_INVALID;
  }
}

}  // namespace lsg
