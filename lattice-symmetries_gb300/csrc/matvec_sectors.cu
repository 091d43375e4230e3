// matvec_sectors.cu -- the batched (multi-sector) persistent matvec kernel: complex128,
// K in {1, 4, 8, 16} right-hand sides with FP64 accumulation, groups of up to 128 elements
// (GPL <= 4).  The FP32-pair variants (K in {8, 16}) are in matvec_pairs_sec.cu.
#include <type_traits>

#include "matvec_launch.cuh"

namespace lsg {

int launch_sectors(int k, int gpl, bool inv, const MatvecProblem& p, int n_sectors_layout, const SectorDesc* d_desc,
                   int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy, int* err, const uint64_t* binom,
                   const double* xs_all, int64_t ldxs, int col, cudaStream_t s) {
  auto go = [&](auto kern) -> int {
    LaunchShape sh{};
    PackedLayout L{};
    const int rc = packed_launch_shape((const void*)kern, 320, p, n_sectors_layout, total_rows, &sh, &L);
    if (rc != 0) return rc;
    kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, d_desc, n_sectors, total_rows, ldx, ldy, err, binom, xs_all,
                                                ldxs, col);
    return cuda_ok(cudaGetLastError(), "k_matvec_sectors") ? 0 : LS_GPU_ERR_CUDA;
  };
  auto with_k = [&](auto gtag, auto itag) -> int {
    constexpr int G = decltype(gtag)::value;
    constexpr bool I = decltype(itag)::value;
    switch (k) {
      case 1: return go(k_matvec_sectors<G, I, 1>);
      case 4: return go(k_matvec_sectors<G, I, 4>);
      case 8: return go(k_matvec_sectors<G, I, 8>);
      case 16: return go(k_matvec_sectors<G, I, 16>);
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
