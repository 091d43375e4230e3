// matvec_real.cu -- float64 gather kernels with the reference's real-part semantics
// (DistributedMatrixVector.chpl:126: complex coefficients contribute their real part).
#include "matvec_impl.cuh"
#include "matvec_dispatch.h"

namespace lsg {

template <int GPL, bool INV>
static int run_real(const MatvecProblem& p, const SmemLayout& L, LaunchShape sh, const double* x,
                    int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom,
                    cudaStream_t s) {
  auto kern = k_matvec_projected<GPL, INV, false, 1>;
  if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total),
               "smem attribute"))
    return LS_GPU_ERR_CUDA;
  kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, x, ldx, y, ldy, err, binom);
  return cuda_ok(cudaGetLastError(), "k_matvec_projected<real>") ? 0 : LS_GPU_ERR_CUDA;
}

#define LSG_REAL_CASE(G)                                                                   \
  case G:                                                                                  \
    return inv ? run_real<G, true>(p, L, sh, x, ldx, y, ldy, err, binom, s)               \
               : run_real<G, false>(p, L, sh, x, ldx, y, ldy, err, binom, s);

int launch_projected_real(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L,
                          LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy,
                          int* err, const uint64_t* binom, cudaStream_t s) {
  switch (gpl) {
    LSG_REAL_CASE(1)
    LSG_REAL_CASE(2)
    LSG_REAL_CASE(3)
    LSG_REAL_CASE(4)
    LSG_REAL_CASE(6)
    LSG_REAL_CASE(9)
    LSG_REAL_CASE(12)
    LSG_REAL_CASE(16)
    default:
      return LS_GPU_ERR_INVALID;
  }
}

template <bool CPLX, bool INV>
static int run_plain(const MatvecProblem& p, const SmemLayout& L, LaunchShape sh, const double* x,
                     int64_t ldx, double* y, int64_t ldy, int k, int* err, const uint64_t* binom,
                     cudaStream_t s) {
  auto kern = k_matvec_plain<CPLX, INV>;
  if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total),
               "smem attribute"))
    return LS_GPU_ERR_CUDA;
  kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, x, ldx, y, ldy, k, err, binom);
  return cuda_ok(cudaGetLastError(), "k_matvec_plain") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_plain(bool cplx, bool inv, int k, const MatvecProblem& p, const SmemLayout& L,
                 LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                 const uint64_t* binom, cudaStream_t s) {
  if (cplx)
    return inv ? run_plain<true, true>(p, L, sh, x, ldx, y, ldy, k, err, binom, s)
               : run_plain<true, false>(p, L, sh, x, ldx, y, ldy, k, err, binom, s);
  return inv ? run_plain<false, true>(p, L, sh, x, ldx, y, ldy, k, err, binom, s)
             : run_plain<false, false>(p, L, sh, x, ldx, y, ldy, k, err, binom, s);
}

}  // namespace lsg
