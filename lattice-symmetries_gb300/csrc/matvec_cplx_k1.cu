// matvec_cplx_k1.cu -- complex128 gather kernels, 1 right-hand side(s) per orbit scan.
#include "matvec_impl.cuh"
#include "matvec_dispatch.h"

namespace lsg {

template <int GPL, bool INV>
static int run_c(const MatvecProblem& p, const SmemLayout& L, LaunchShape sh, const double* x,
                 int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom,
                 cudaStream_t s) {
  auto kern = k_matvec_projected<GPL, INV, true, 1>;
  if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total),
               "smem attribute"))
    return LS_GPU_ERR_CUDA;
  kern<<<sh.blocks, sh.threads, L.total, s>>>(p, L, x, ldx, y, ldy, err, binom);
  return cuda_ok(cudaGetLastError(), "k_matvec_projected<complex,1>") ? 0 : LS_GPU_ERR_CUDA;
}

#define LSG_C_CASE(G)                                                                      \
  case G:                                                                                  \
    return inv ? run_c<G, true>(p, L, sh, x, ldx, y, ldy, err, binom, s)                  \
               : run_c<G, false>(p, L, sh, x, ldx, y, ldy, err, binom, s);

int launch_projected_cplx_k1(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L,
                              LaunchShape sh, const double* x, int64_t ldx, double* y,
                              int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {
  switch (gpl) {
    LSG_C_CASE(1)
    LSG_C_CASE(2)
    LSG_C_CASE(3)
    LSG_C_CASE(4)
    LSG_C_CASE(6)
    LSG_C_CASE(9)
    LSG_C_CASE(12)
    LSG_C_CASE(16)
    default:
      return LS_GPU_ERR_INVALID;
  }
}

}  // namespace lsg
