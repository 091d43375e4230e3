// blockops.cu -- dense products of the block-Lanczos driver on tall complex128 blocks.
//
// A block-Lanczos step on S sectors with blocks of k <= 16 columns and D rows per sector spends
// its dense work in two shapes:
//
//     G[s] = X[s]^H Y[s]                          (k x k Gram matrices; inner dimension D)
//     W[s] <- beta W[s] + X1[s] M1[s] + X2[s] M2[s]   (tall block times small k x k matrices)
//
// Both are 8 D k^2 real operations per product.  GB300's FP64 pipe is narrow (a small fraction of
// its FP32 rate), so FP64 GEMMs on these shapes run at the FP64 roofline.  These kernels keep the
// blocks in FP64 in memory but evaluate the products in "FP32-pair" arithmetic on the FP32 pipe:
// every FP64 input is split into an unevaluated sum hi + lo of two floats (48 significant bits;
// the split uses integer instructions only), products are formed with an exact hi*hi term
// (fmaf error term) plus the first-order cross terms, and running sums use an error-free
// two-sum.  The relative error of one product is below 2^-45 (3e-14).  The Gram kernel keeps a pair sum
// over one tile of 32 rows at a time and adds the tiles in FP64, so the error of a Gram entry
// stays near that bound relative to the sum of magnitudes of its terms.  Results are converted back to FP64
// (integer conversion + one FP64 add).
//
// Determinism: every CTA reduces a fixed row range; the partial Gram matrices are summed in
// FP64 in a fixed order.  No atomics.
//
// No reference counterpart: the reference's eigensolvers are scipy's eigsh over the matvec
// (python/lattice_symmetries/__init__.py:751-752) and PRIMME (chapel/src/Diagonalize.chpl).
#include "lsg.h"
#include "pairs.cuh"

#include <algorithm>

namespace lsg {
namespace {

constexpr int kMaxK = 16;      // columns per block handled by these kernels
constexpr int kThreads = 256;  // threads per CTA
constexpr int kTileRows = 32;  // rows of X / Y staged per tile (Gram)

// Partial Gram matrices: CTA (c, s) sums conj(X[s, r, i]) Y[s, r, j] over its rows.
// Thread o < k*k of row group g owns output (i, j) = (o / k, o % k) for rows r = g (mod groups).
__global__ void __launch_bounds__(kThreads) k_block_gram(int64_t D, int k, int64_t rows_per_chunk, int chunks,
                                                          const double2* __restrict__ X,
                                                          const double2* __restrict__ Y, bool same,
                                                          double2* __restrict__ partial) {
  __shared__ float4 xs[kTileRows * kMaxK];
  __shared__ float4 ys[kTileRows * kMaxK];
  const int s = blockIdx.y;
  const int c = blockIdx.x;
  const int tid = threadIdx.x;
  const int nout = k * k;
  const int groups = kThreads / nout;
  const int o = tid % nout;
  const int grp = tid / nout;
  const bool active = grp < groups;
  const int i = o / k, j = o % k;
  const int64_t r0 = (int64_t)c * rows_per_chunk;
  const int64_t r1 = r0 + rows_per_chunk < D ? r0 + rows_per_chunk : D;
  const double2* Xs = X + (size_t)s * D * k;
  const double2* Ys = Y + (size_t)s * D * k;
  const float4* yt = same ? xs : ys;
  double dre = 0.0, dim = 0.0;  // FP64 sum of the per-tile pair sums
  for (int64_t rt = r0; rt < r1; rt += kTileRows) {
    const int n = (int)(r1 - rt < kTileRows ? r1 - rt : kTileRows);
    const int ne = n * k;
    for (int e = tid; e < ne; e += kThreads) {
      xs[e] = split_c(Xs[rt * k + e]);
      if (!same) ys[e] = split_c(Ys[rt * k + e]);
    }
    __syncthreads();
    if (active) {
      // a pair sum over at most one tile of rows keeps the low word small, then FP64
      F2 re{0.0f, 0.0f}, im{0.0f, 0.0f};
      for (int rr = grp; rr < n; rr += groups) {
        const float4 x = xs[rr * k + i];
        const float4 y = yt[rr * k + j];
        // conj(x) y = (xr yr + xi yi) + i (xr yi - xi yr)
        mac(re, x.x, x.y, y.x, y.y);
        mac(re, x.z, x.w, y.z, y.w);
        mac(im, x.x, x.y, y.z, y.w);
        mac(im, -x.z, -x.w, y.x, y.y);
        renorm(re);
        renorm(im);
      }
      dre += join(re);
      dim += join(im);
    }
    __syncthreads();
  }
  // sum the row groups in FP64
  double2* red = reinterpret_cast<double2*>(xs);  // kThreads double2 entries fit in xs
  red[tid] = make_double2(dre, dim);
  __syncthreads();
  if (tid < nout) {
    double sre = 0.0, sim = 0.0;
    for (int g = 0; g < groups; ++g) {
      const double2 v = red[g * nout + tid];
      sre += v.x;
      sim += v.y;
    }
    partial[((size_t)s * chunks + c) * nout + tid] = make_double2(sre, sim);
  }
}

// G[s][o] = sum over chunks of partial[s][c][o]: block (s, o / 32), lane = o % 32; the 32 warps
// of the block sum interleaved chunks, then lane o adds the 32 warp sums in order (fixed
// summation order: deterministic).
__global__ void __launch_bounds__(1024) k_block_gram_sum(const double2* __restrict__ partial, int chunks, int nout,
                                                         double2* __restrict__ G) {
  __shared__ double2 warp_sums[32][32];
  const int s = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int o = blockIdx.y * 32 + lane;
  double re = 0.0, im = 0.0;
  if (o < nout) {
    const double2* p = partial + (size_t)s * chunks * nout + o;
    for (int c = warp; c < chunks; c += 32) {
      const double2 v = p[(size_t)c * nout];
      re += v.x;
      im += v.y;
    }
  }
  warp_sums[warp][lane] = make_double2(re, im);
  __syncthreads();
  if (warp == 0 && o < nout) {
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < 32; ++w) {
      t.x += warp_sums[w][lane].x;
      t.y += warp_sums[w][lane].y;
    }
    G[(size_t)s * nout + o] = t;
  }
}

// out[s, r, j] = beta W[s, r, j] + sum_i X1[s, r, i] M1[s, i, j] (+ X2 M2).  Thread t handles
// column j = t % k of rows t / k (mod 256 / k) of each tile; the tile's rows of X1 and X2 are
// staged (split) in shared memory before any output of the tile is written, so `out` may alias
// W, X1 or X2.
__global__ void __launch_bounds__(kThreads) k_block_update(int64_t D, int k, int64_t rows_per_chunk, double beta,
                                                            const double2* W, const double2* X1,
                                                            const double2* __restrict__ M1, const double2* X2,
                                                            const double2* __restrict__ M2, double2* out) {
  __shared__ float4 m1[kMaxK * kMaxK];
  __shared__ float4 m2[kMaxK * kMaxK];
  __shared__ float4 x1s[2 * kThreads];
  __shared__ float4 x2s[2 * kThreads];
  const int s = blockIdx.y;
  const int c = blockIdx.x;
  const int tid = threadIdx.x;
  const int kk = k * k;
  const bool two = X2 != nullptr;
  for (int e = tid; e < kk; e += kThreads) {
    m1[e] = split_c(M1[(size_t)s * kk + e]);
    if (two) m2[e] = split_c(M2[(size_t)s * kk + e]);
  }
  const int rows_per_pass = kThreads / k;
  const int tile_rows = 2 * rows_per_pass;
  const int j = tid % k;
  const int rl = tid / k;
  const bool active = rl < rows_per_pass;
  const int64_t r0 = (int64_t)c * rows_per_chunk;
  const int64_t r1 = r0 + rows_per_chunk < D ? r0 + rows_per_chunk : D;
  const size_t base = (size_t)s * D * k;
  for (int64_t rt = r0; rt < r1; rt += tile_rows) {
    const int n = (int)(r1 - rt < tile_rows ? r1 - rt : tile_rows);
    const int ne = n * k;
    __syncthreads();  // previous tile consumed (and the matrices staged, first time)
    for (int e = tid; e < ne; e += kThreads) {
      x1s[e] = split_c(X1[base + rt * k + e]);
      if (two) x2s[e] = split_c(X2[base + rt * k + e]);
    }
    __syncthreads();
    if (!active) continue;
    for (int rr = rl; rr < n; rr += rows_per_pass) {
      const size_t at = base + (size_t)(rt + rr) * k + j;
      F2 re{0.0f, 0.0f}, im{0.0f, 0.0f};
      if (beta != 0.0) {
        double2 w = W[at];
        if (beta != 1.0) w = make_double2(beta * w.x, beta * w.y);
        const float4 ws = split_c(w);
        re = F2{ws.x, ws.y};
        im = F2{ws.z, ws.w};
      }
      const float4* xr = x1s + rr * k;
      for (int i = 0; i < k; ++i) {
        const float4 x = xr[i];
        const float4 m = m1[i * k + j];
        // x m = (xr mr - xi mi) + i (xr mi + xi mr)
        mac(re, x.x, x.y, m.x, m.y);
        mac(re, -x.z, -x.w, m.z, m.w);
        mac(im, x.x, x.y, m.z, m.w);
        mac(im, x.z, x.w, m.x, m.y);
        renorm(re);
        renorm(im);
      }
      if (two) {
        const float4* xq = x2s + rr * k;
        for (int i = 0; i < k; ++i) {
          const float4 x = xq[i];
          const float4 m = m2[i * k + j];
          mac(re, x.x, x.y, m.x, m.y);
          mac(re, -x.z, -x.w, m.z, m.w);
          mac(im, x.x, x.y, m.z, m.w);
          mac(im, x.z, x.w, m.x, m.y);
          renorm(re);
          renorm(im);
        }
      }
      out[at] = make_double2(join(re), join(im));
    }
  }
}

// CTAs per sector: about 8 per SM over the whole grid, at least one tile of rows each.
int64_t chunk_rows(int64_t S, int64_t D, int tile_rows) {
  const int64_t target = std::max<int64_t>(1, ((int64_t)num_sms() * 8 + S - 1) / S);
  const int64_t max_chunks = std::max<int64_t>(1, (D + tile_rows - 1) / tile_rows);
  const int64_t chunks = std::min(target, max_chunks);
  int64_t rows = (D + chunks - 1) / chunks;
  rows = (rows + tile_rows - 1) / tile_rows * tile_rows;
  return std::max<int64_t>(rows, tile_rows);
}

bool check_shape(int64_t S, int64_t D, int k) {
  return S >= 1 && S <= 65535 && D >= 0 && k >= 1 && k <= kMaxK;
}

}  // namespace

int launch_block_gram(int64_t S, int64_t D, int k, const double* d_x, const double* d_y, double* d_g,
                      cudaStream_t s) {
  if (!check_shape(S, D, k)) return fail(LS_GPU_ERR_INVALID, "block Gram: need 1 <= S <= 65535, D >= 0, 1 <= k <= 16");
  if (d_g == nullptr || (D > 0 && (d_x == nullptr || d_y == nullptr)))
    return fail(LS_GPU_ERR_INVALID, "block Gram: NULL pointer");
  const int nout = k * k;
  if (D == 0) {
    return cuda_ok(cudaMemsetAsync(d_g, 0, (size_t)S * nout * 16, s), "block Gram (empty)") ? 0 : LS_GPU_ERR_CUDA;
  }
  const int64_t rows = chunk_rows(S, D, kTileRows);
  const int64_t chunks = (D + rows - 1) / rows;
  if (chunks > 0x7fffffff) return fail(LS_GPU_ERR_INVALID, "block Gram: too many rows");
  double2* partial = nullptr;
  if (!cuda_ok(cudaMallocAsync((void**)&partial, (size_t)S * chunks * nout * sizeof(double2), s),
               "cudaMallocAsync(block Gram partials)"))
    return LS_GPU_ERR_CUDA;
  const dim3 grid((unsigned)chunks, (unsigned)S);
  StageScope stage("lanczos.gram", s);
  k_block_gram<<<grid, kThreads, 0, s>>>(D, k, rows, (int)chunks, reinterpret_cast<const double2*>(d_x),
                                         reinterpret_cast<const double2*>(d_y), d_x == d_y, partial);
  bool ok = cuda_ok(cudaGetLastError(), "k_block_gram");
  if (ok) {
    k_block_gram_sum<<<dim3((unsigned)S, (unsigned)((nout + 31) / 32)), 1024, 0, s>>>(
        partial, (int)chunks, nout, reinterpret_cast<double2*>(d_g));
    ok = cuda_ok(cudaGetLastError(), "k_block_gram_sum");
  }
  ok = cuda_ok(cudaFreeAsync(partial, s), "cudaFreeAsync(block Gram partials)") && ok;
  return ok ? 0 : LS_GPU_ERR_CUDA;
}

int launch_gram_partial_sum(const double2* partial, int chunks, int nout, int64_t S, double2* G, cudaStream_t s) {
  k_block_gram_sum<<<dim3((unsigned)S, (unsigned)((nout + 31) / 32)), 1024, 0, s>>>(partial, chunks, nout, G);
  return cuda_ok(cudaGetLastError(), "k_block_gram_sum") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_block_update(int64_t S, int64_t D, int k, double beta, const double* d_w, const double* d_x1,
                        const double* d_m1, const double* d_x2, const double* d_m2, double* d_out,
                        cudaStream_t s) {
  if (!check_shape(S, D, k)) return fail(LS_GPU_ERR_INVALID, "block update: need 1 <= S <= 65535, D >= 0, 1 <= k <= 16");
  if (D == 0) return 0;
  if (d_out == nullptr || d_x1 == nullptr || d_m1 == nullptr || (beta != 0.0 && d_w == nullptr) ||
      ((d_x2 == nullptr) != (d_m2 == nullptr)))
    return fail(LS_GPU_ERR_INVALID, "block update: NULL pointer");
  const int tile_rows = 2 * (kThreads / k);
  const int64_t rows = chunk_rows(S, D, tile_rows);
  const int64_t chunks = (D + rows - 1) / rows;
  if (chunks > 0x7fffffff) return fail(LS_GPU_ERR_INVALID, "block update: too many rows");
  const dim3 grid((unsigned)chunks, (unsigned)S);
  StageScope stage("lanczos.update", s);
  k_block_update<<<grid, kThreads, 0, s>>>(D, k, rows, beta, reinterpret_cast<const double2*>(d_w),
                                           reinterpret_cast<const double2*>(d_x1),
                                           reinterpret_cast<const double2*>(d_m1),
                                           reinterpret_cast<const double2*>(d_x2),
                                           reinterpret_cast<const double2*>(d_m2), reinterpret_cast<double2*>(d_out));
  return cuda_ok(cudaGetLastError(), "k_block_update") ? 0 : LS_GPU_ERR_CUDA;
}

}  // namespace lsg

extern "C" int ls_gpu_block_gram(int64_t S, int64_t D, int k, double const* d_x, double const* d_y, double* d_g,
                                 void* stream) {
  return lsg::launch_block_gram(S, D, k, d_x, d_y, d_g, (cudaStream_t)stream);
}

extern "C" int ls_gpu_block_update(int64_t S, int64_t D, int k, double beta, double const* d_w, double const* d_x1,
                                   double const* d_m1, double const* d_x2, double const* d_m2, double* d_out,
                                   void* stream) {
  return lsg::launch_block_update(S, D, k, beta, d_w, d_x1, d_m1, d_x2, d_m2, d_out, (cudaStream_t)stream);
}
