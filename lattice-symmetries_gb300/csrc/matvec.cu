// matvec.cu -- launch policy of the gather kernels (kernel choice, grid shape, RHS blocking).
#include <algorithm>

#include "matvec_dispatch.h"
#include "matvec_impl.cuh"

namespace lsg {

int launch_packed(bool cplx, int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L,
                  LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                  const uint64_t* binom, cudaStream_t s) {
  if (!cplx) {
    if (k != 1) return LS_GPU_ERR_INVALID;
    return launch_packed_real(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
  }
  switch (k) {
    case 1: return launch_packed_cplx_k1(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
    case 4: return launch_packed_cplx_k4(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
    case 8: return launch_packed_cplx_k8(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
    case 16: return launch_packed_cplx_k16(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
    default: return LS_GPU_ERR_INVALID;
  }
}

static int g_threads_override = 0;
static int g_blocks_per_sm_override = 0;

int set_matvec_config(int threads, int blocks_per_sm) {
  g_threads_override = threads;
  g_blocks_per_sm_override = blocks_per_sm;
  return 0;
}

extern const uint64_t* device_binomials();

constexpr size_t kMaxDynamicSmem = 200 * 1024;

// Splits k right-hand sides into launches of 16, 8, 4 and 1 columns.
int launch_matvec(const MatvecProblem& p, Scalar sc, int k, const double* d_x, int64_t ldx,
                  double* d_y, int64_t ldy, int* d_err, cudaStream_t s) {
  if (p.n_rows == 0 || k == 0) return 0;
  const uint64_t* binom = device_binomials();
  if (binom == nullptr) return LS_GPU_ERR_CUDA;
  const bool cplx = sc == Scalar::Complex;
  const size_t scalar_words = cplx ? 2 : 1;  // doubles per element
  if (p.projection == 2) {
    const bool inv = p.group.spin_inversion != 0;
    const int threads = g_threads_override > 0 ? g_threads_override : 256;
    const int warps_per_block = threads / 32;
    // two resident CTAs per SM; `waves` grids of that size balance the per-row work
    const int waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : 4;
    int64_t blocks = (int64_t)num_sms() * 2 * waves;
    blocks = std::min<int64_t>(blocks, (p.n_rows + warps_per_block - 1) / warps_per_block);
    blocks = std::max<int64_t>(blocks, 1);
    const LaunchShape sh{(int)blocks, threads};
    const PackedLayout PL = make_packed_layout(p);
    const bool packed = p.group.gpl > 0 && p.group.onehot_packed != nullptr && PL.total <= kMaxDynamicSmem;
    if (packed) {
      int done = 0;
      while (done < k) {
        const int left = k - done;
        int chunk = 1;
        if (cplx) chunk = left >= 16 ? 16 : left >= 8 ? 8 : left >= 4 ? 4 : 1;
        const double* xs = d_x + (size_t)done * scalar_words;
        double* ys = d_y + (size_t)done * scalar_words;
        int rc = launch_packed(cplx, chunk, p.group.gpl, inv, p, PL, sh, xs, ldx, ys, ldy, d_err, binom, s);
        if (rc != 0) return rc;
        done += chunk;
      }
      return 0;
    }
    const int gpl = pick_gpl_for(p.group.n_elems);
    if (gpl < 0) return fail(LS_GPU_ERR_INVALID, "symmetry group too large for the matvec kernels");
    const SmemLayout L = make_layout(p, true);
    if (L.total > kMaxDynamicSmem) return fail(LS_GPU_ERR_INVALID, "term tables too large for shared memory");
    for (int c = 0; c < k; ++c) {
      const double* xs = d_x + (size_t)c * scalar_words;
      double* ys = d_y + (size_t)c * scalar_words;
      int rc = cplx ? launch_projected_cplx_k1(gpl, inv, p, L, sh, xs, ldx, ys, ldy, d_err, binom, s)
                    : launch_projected_real(gpl, inv, p, L, sh, xs, ldx, ys, ldy, d_err, binom, s);
      if (rc != 0) return rc;
    }
    return 0;
  }
  const SmemLayout L = make_layout(p, false);
  if (L.total > kMaxDynamicSmem) return fail(LS_GPU_ERR_INVALID, "term tables too large for shared memory");
  const int threads = 256;
  int64_t blocks = (p.n_rows + threads - 1) / threads;
  blocks = std::min<int64_t>(blocks, (int64_t)num_sms() * 16);
  blocks = std::max<int64_t>(blocks, 1);
  const LaunchShape sh{(int)blocks, threads};
  return launch_plain(cplx, p.projection == 1, k, p, L, sh, d_x, ldx, d_y, ldy, d_err, binom, s);
}

}  // namespace lsg
