// matvec_real.cu -- float64 gather kernels with the reference's real-part semantics
// (DistributedMatrixVector.chpl:126: complex coefficients contribute their real part), plus the
// unprojected / spin-inversion-only kernels.
#include "matvec_launch.cuh"

namespace lsg {

LSG_DEFINE_PACKED(launch_packed_real, false, 1)
LSG_DEFINE_FALLBACK(launch_projected_real, false)

template <bool CPLX, bool INV>
static int run_plain(const MatvecProblem& p, const SmemLayout& L, LaunchShape sh, const double* x,
                     int64_t ldx, double* y, int64_t ldy, int k, int* err, const uint64_t* binom,
                     cudaStream_t s) {
  auto kern = k_matvec_plain<CPLX, INV>;
  if (!ensure_smem_limit((const void*)kern, L.total)) return LS_GPU_ERR_CUDA;
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
