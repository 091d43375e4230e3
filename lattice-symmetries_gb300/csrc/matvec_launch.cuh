// matvec_launch.cuh -- launch helpers shared by the matvec translation units.
#pragma once
#include <array>
#include <type_traits>
#include <unordered_map>

#include "matvec_dispatch.h"
#include "matvec_impl.cuh"

namespace lsg {

// Raises a kernel's dynamic shared-memory limit once per (kernel, device, size): later launches,
// including ones recorded in a CUDA graph, make no attribute call.  Callers hold the library lock.
inline bool ensure_smem_limit(const void* kern, size_t bytes) {
  static std::unordered_map<const void*, std::array<int, 64>> set_bytes;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  auto it = set_bytes.find(kern);
  if (it != set_bytes.end() && it->second[dev] >= (int)bytes) return true;
  if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
               "smem attribute"))
    return false;
  if (it == set_bytes.end()) it = set_bytes.emplace(kern, std::array<int, 64>{}).first;
  it->second[dev] = (int)bytes;
  return true;
}

template <typename Kernel, typename Layout>
static int launch_with_smem(Kernel kern, const char* name, const MatvecProblem& p, const Layout& L,
                            LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                            const uint64_t* binom, cudaStream_t s) {
  if (!ensure_smem_limit((const void*)kern, L.total)) return LS_GPU_ERR_CUDA;
  kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, x, ldx, y, ldy, err, binom);
  return cuda_ok(cudaGetLastError(), name) ? 0 : LS_GPU_ERR_CUDA;
}

// Launches the packed single-sector kernel `kern` (compiled for at most max_threads threads per
// CTA) with the shape and shared-memory layout that packed_launch_shape picks.
template <typename Kernel>
static int launch_packed_kernel(Kernel kern, int max_threads, const char* name, const MatvecProblem& p,
                                const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                                const uint64_t* binom, cudaStream_t s) {
  LaunchShape sh{};
  PackedLayout L{};
  const int rc = packed_launch_shape((const void*)kern, max_threads, p, 0, p.n_rows, &sh, &L);
  if (rc != 0) return rc;
  kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, x, ldx, y, ldy, err, binom);
  return cuda_ok(cudaGetLastError(), name) ? 0 : LS_GPU_ERR_CUDA;
}

}  // namespace lsg

// Defines NAME(gpl, inv, ...) launching k_matvec_packed<GPL, INV, CPLX, K>.
#define LSG_DEFINE_PACKED(NAME, CPLX, K)                                                          \
  int NAME(int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx, double* y,    \
           int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {                        \
    auto run = [&](auto gtag) -> int {                                                            \
      constexpr int G = decltype(gtag)::value;                                                    \
      constexpr int MT = PackedBounds<G, K, false, CPLX>::threads;                                \
      return inv ? launch_packed_kernel(k_matvec_packed<G, true, CPLX, K>, MT, #NAME, p, x, ldx,  \
                                        y, ldy, err, binom, s)                                   \
                 : launch_packed_kernel(k_matvec_packed<G, false, CPLX, K>, MT, #NAME, p, x, ldx, \
                                        y, ldy, err, binom, s);                                  \
    };                                                                                            \
    switch (gpl) {                                                                                \
      case 1: return run(std::integral_constant<int, 1>{});                                       \
      case 2: return run(std::integral_constant<int, 2>{});                                       \
      case 3: return run(std::integral_constant<int, 3>{});                                       \
      case 4: return run(std::integral_constant<int, 4>{});                                       \
      case 6: return run(std::integral_constant<int, 6>{});                                       \
      case 9: return run(std::integral_constant<int, 9>{});                                       \
      case 12: return run(std::integral_constant<int, 12>{});                                     \
      case 16: return run(std::integral_constant<int, 16>{});                                     \
      default: return LS_GPU_ERR_INVALID;                                                         \
    }                                                                                             \
  }

// Defines NAME(gpl, inv, ...) launching the FP32-pair k_matvec_packed<GPL, INV, true, K, false, true>.
#define LSG_DEFINE_PACKED_PAIR(NAME, K)                                                           \
  int NAME(int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx, double* y,    \
           int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {                        \
    auto run = [&](auto gtag) -> int {                                                            \
      constexpr int G = decltype(gtag)::value;                                                    \
      constexpr int MT = PackedBounds<G, K, true>::threads;                                       \
      return inv ? launch_packed_kernel(k_matvec_packed<G, true, true, K, false, true>, MT, #NAME, \
                                        p, x, ldx, y, ldy, err, binom, s)                        \
                 : launch_packed_kernel(k_matvec_packed<G, false, true, K, false, true>, MT,       \
                                        #NAME, p, x, ldx, y, ldy, err, binom, s);                \
    };                                                                                            \
    switch (gpl) {                                                                                \
      case 1: return run(std::integral_constant<int, 1>{});                                       \
      case 2: return run(std::integral_constant<int, 2>{});                                       \
      case 3: return run(std::integral_constant<int, 3>{});                                       \
      case 4: return run(std::integral_constant<int, 4>{});                                       \
      case 6: return run(std::integral_constant<int, 6>{});                                       \
      case 9: return run(std::integral_constant<int, 9>{});                                       \
      case 12: return run(std::integral_constant<int, 12>{});                                     \
      case 16: return run(std::integral_constant<int, 16>{});                                     \
      default: return LS_GPU_ERR_INVALID;                                                         \
    }                                                                                             \
  }

// Defines NAME(gpl, inv, ...) launching the fallback k_matvec_projected<GPL, INV, CPLX, 1>.
#define LSG_DEFINE_FALLBACK(NAME, CPLX)                                                          \
  int NAME(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L, LaunchShape sh,       \
           const double* x, int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom, \
           cudaStream_t s) {                                                                      \
    auto run = [&](auto gtag) -> int {                                                            \
      constexpr int G = decltype(gtag)::value;                                                    \
      return inv ? launch_with_smem(k_matvec_projected<G, true, CPLX, 1>, #NAME, p, L, sh, x, ldx, \
                                    y, ldy, err, binom, s)                                       \
                 : launch_with_smem(k_matvec_projected<G, false, CPLX, 1>, #NAME, p, L, sh, x,    \
                                    ldx, y, ldy, err, binom, s);                                 \
    };                                                                                            \
    switch (gpl) {                                                                                \
      case 1: return run(std::integral_constant<int, 1>{});                                       \
      case 2: return run(std::integral_constant<int, 2>{});                                       \
      case 3: return run(std::integral_constant<int, 3>{});                                       \
      case 4: return run(std::integral_constant<int, 4>{});                                       \
      case 6: return run(std::integral_constant<int, 6>{});                                       \
      case 9: return run(std::integral_constant<int, 9>{});                                       \
      case 12: return run(std::integral_constant<int, 12>{});                                     \
      case 16: return run(std::integral_constant<int, 16>{});                                     \
      default: return LS_GPU_ERR_INVALID;                                                         \
    }                                                                                             \
  }
