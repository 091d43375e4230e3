// apply.cu -- per-state term application on device batches: for every input state alpha the
// diagonal value sum_t Re(v_t) (-1)^popcount(alpha & s_t) [(alpha & m_t) == r_t], and the
// off-diagonal targets beta = alpha ^ x_t with coefficients v_t (-1)^popcount(alpha & s_t), in
// compressed rows (offsets).  Same results, term order and layout as
// ls_internal_operator_apply_{diag,off_diag}_x1 (reference.c:67-135), for batches that already
// live on the GPU (variational Monte Carlo style local energies).  One thread per input state;
// the off-diagonal pass counts, scans and writes.
#include <algorithm>

#include "lsg.h"

namespace lsg {

__global__ void k_apply_diag(DeviceTerms t, int64_t count, const uint64_t* __restrict__ alphas,
                             double* __restrict__ ys) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = alphas[i];
    double acc = 0.0;
    for (int k = 0; k < t.n; ++k) {
      if ((a & __ldg(t.m + k)) == __ldg(t.r + k)) {
        const double v = __ldg(&t.v[k].x);
        acc += (__popcll(a & __ldg(t.s + k)) & 1) ? -v : v;
      }
    }
    ys[i] = acc;
  }
}

__global__ void k_apply_count(DeviceTerms t, int64_t count, const uint64_t* __restrict__ alphas,
                              int32_t* __restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = alphas[i];
    int c = 0;
    for (int k = 0; k < t.n; ++k) c += (a & __ldg(t.m + k)) == __ldg(t.r + k);
    counts[i] = c;
  }
}

__global__ void k_apply_write(DeviceTerms t, int64_t count, const uint64_t* __restrict__ alphas,
                              const int64_t* __restrict__ offsets, uint64_t* __restrict__ betas,
                              double2* __restrict__ coeffs) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = alphas[i];
    int64_t o = offsets[i];
    for (int k = 0; k < t.n; ++k) {
      if ((a & __ldg(t.m + k)) == __ldg(t.r + k)) {
        double2 v = __ldg(t.v + k);
        if (__popcll(a & __ldg(t.s + k)) & 1) v = make_double2(-v.x, -v.y);
        coeffs[o] = v;
        betas[o] = a ^ __ldg(t.x + k);
        ++o;
      }
    }
  }
}

static int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 16;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

int launch_apply_diag(const DeviceTerms& diag, int64_t count, const uint64_t* d_alphas, double* d_ys, cudaStream_t s) {
  if (count <= 0) return 0;
  k_apply_diag<<<blocks_for(count), 256, 0, s>>>(diag, count, d_alphas, d_ys);
  return cuda_ok(cudaGetLastError(), "k_apply_diag") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_apply_off_diag(const DeviceTerms& off, int64_t count, const uint64_t* d_alphas, uint64_t* d_betas,
                          double* d_coeffs, int64_t* d_offsets, cudaStream_t s) {
  if (count <= 0) {
    return cuda_ok(cudaMemsetAsync(d_offsets, 0, sizeof(int64_t), s), "offsets") ? 0 : LS_GPU_ERR_CUDA;
  }
  int32_t* counts = (int32_t*)scratch((size_t)count * sizeof(int32_t), 7);
  if (counts == nullptr) return LS_GPU_ERR_CUDA;
  k_apply_count<<<blocks_for(count), 256, 0, s>>>(off, count, d_alphas, counts);
  if (!cuda_ok(cudaGetLastError(), "k_apply_count")) return LS_GPU_ERR_CUDA;
  int rc = exclusive_scan_counts(counts, count, d_offsets, s);
  if (rc != 0) return rc;
  k_apply_write<<<blocks_for(count), 256, 0, s>>>(off, count, d_alphas, d_offsets, d_betas,
                                                  reinterpret_cast<double2*>(d_coeffs));
  return cuda_ok(cudaGetLastError(), "k_apply_write") ? 0 : LS_GPU_ERR_CUDA;
}

// out[c][r] = in[r][c] for an in matrix of rows x cols doubles (row-major).
__global__ void k_transpose(const double* __restrict__ in, double* __restrict__ out, int64_t rows, int64_t cols) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / cols, c = e - r * cols;
    out[c * rows + r] = in[e];
  }
}

int launch_transpose(const double* d_in, double* d_out, int64_t rows, int64_t cols, cudaStream_t s) {
  if (rows * cols == 0) return 0;
  k_transpose<<<blocks_for(rows * cols), 256, 0, s>>>(d_in, d_out, rows, cols);
  return cuda_ok(cudaGetLastError(), "k_transpose") ? 0 : LS_GPU_ERR_CUDA;
}

}  // namespace lsg
