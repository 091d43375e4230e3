// matvec.cu -- launch policy of the gather kernels (kernel choice, grid shape, RHS blocking).
#include <algorithm>

#include "matvec_dispatch.h"
#include "matvec_impl.cuh"

namespace lsg {

int launch_packed(bool cplx, int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L,
                  LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                  const uint64_t* binom, cudaStream_t s) {
  if (p.group.fermionic) {
    if (inv) return fail(LS_GPU_ERR_INVALID, "fermionic groups have no spin inversion");
    return launch_packed_fermi(cplx, k, gpl, p, L, sh, x, ldx, y, ldy, err, binom, s);
  }
  if (!cplx) {
    switch (k) {
      case 1: return launch_packed_real(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
      case 2: return launch_packed_real_k2(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
      case 4: return launch_packed_real_k4(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
      case 8: return launch_packed_real_k8(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
      case 16: return launch_packed_real_k16(gpl, inv, p, L, sh, x, ldx, y, ldy, err, binom, s);
      default: return LS_GPU_ERR_INVALID;
    }
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
static int g_rhs_tile = 16;  // most right-hand sides per launch (16, 8, 4 or 1)

int set_matvec_config(int threads, int blocks_per_sm) {
  // the warp-per-row kernels are compiled for at most 320 threads per block
  if (threads != 0 && (threads < 32 || threads > 320 || threads % 32 != 0)) return LS_GPU_ERR_INVALID;
  if (blocks_per_sm < 0 || blocks_per_sm > 64) return LS_GPU_ERR_INVALID;
  g_threads_override = threads;
  g_blocks_per_sm_override = blocks_per_sm;
  return 0;
}

int set_matvec_rhs_tile(int tile) {
  if (tile != 1 && tile != 4 && tile != 8 && tile != 16) return LS_GPU_ERR_INVALID;
  g_rhs_tile = tile;
  return 0;
}

void get_matvec_config(int* threads, int* waves, int* rhs_tile) {
  if (threads) *threads = g_threads_override > 0 ? g_threads_override : 320;
  if (waves) *waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : 8;
  if (rhs_tile) *rhs_tile = g_rhs_tile;
}

extern const uint64_t* device_binomials();

// xs[i][c] = x[i][c] * norms[i] for k columns of `words` doubles per element (1 real, 2 complex).
__global__ void k_prescale(const double* __restrict__ x, int64_t ldx, const double* __restrict__ norms, int64_t n,
                           int k, int words, double* __restrict__ xs) {
  const int64_t per_row = (int64_t)k * words;
  const int64_t total = n * per_row;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / per_row, r = e - i * per_row;
    xs[e] = __ldg(x + i * ldx * words + r) * __ldg(norms + i);
  }
}


constexpr size_t kMaxDynamicSmem = 200 * 1024;

LaunchShape packed_shape(int64_t n_rows) {
  // two resident CTAs per SM; `waves` grids of that size balance the uneven per-row work
  const int threads = g_threads_override > 0 ? g_threads_override : 320;
  const int waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : 8;
  const int warps_per_block = threads / 32;
  int64_t blocks = (int64_t)num_sms() * 2 * waves;
  blocks = std::min<int64_t>(blocks, (n_rows + warps_per_block - 1) / warps_per_block);
  blocks = std::max<int64_t>(blocks, 1);
  return LaunchShape{(int)blocks, threads};
}

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
    const LaunchShape sh = packed_shape(p.n_rows);
    const PackedLayout PL = make_packed_layout(p);
    const bool packed = p.group.gpl > 0 && p.group.onehot_packed != nullptr && PL.total <= kMaxDynamicSmem;
    if (packed) {
      // Gather source x_j * n_j for all k columns (one streaming pass), so that the kernels read
      // no norm per generated element.  Not when counting elements (the count needs the norms).
      MatvecProblem q = p;
      double* d_xs = nullptr;
      const size_t xs_bytes = (size_t)p.n_rows * k * scalar_words * sizeof(double);
      if (p.nnz_counter == nullptr && p.index.norms != nullptr &&
          cudaMallocAsync((void**)&d_xs, xs_bytes, s) == cudaSuccess) {
        const int64_t total = p.n_rows * k * (int64_t)scalar_words;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16));
        k_prescale<<<blocks, 256, 0, s>>>(d_x, ldx, p.index.norms, p.n_rows, k, (int)scalar_words, d_xs);
        if (!cuda_ok(cudaGetLastError(), "k_prescale")) {
          cudaFreeAsync(d_xs, s);
          return LS_GPU_ERR_CUDA;
        }
      } else {
        cudaGetLastError();  // a failed stream-ordered allocation: gather x and the norms instead
        d_xs = nullptr;
      }
      int done = 0, rc = 0;
      while (done < k && rc == 0) {
        const int left = k - done;
        const int most = std::min(left, g_rhs_tile);
        int chunk = most >= 16 ? 16 : most >= 8 ? 8 : most >= 4 ? 4 : 1;
        if (!cplx && left == 2 && g_rhs_tile >= 2) chunk = 2;
        if (p.group.fermionic && !cplx) chunk = 1;  // fermionic real path: one column per launch
        const double* xs = d_x + (size_t)done * scalar_words;
        double* ys = d_y + (size_t)done * scalar_words;
        q.xs = d_xs ? d_xs + (size_t)done * scalar_words : nullptr;
        q.ldxs = k;
        rc = launch_packed(cplx, chunk, p.group.gpl, inv, q, PL, sh, xs, ldx, ys, ldy, d_err, binom, s);
        done += chunk;
      }
      if (d_xs) cudaFreeAsync(d_xs, s);
      return rc;
    }
    if (p.group.fermionic)
      return fail(LS_GPU_ERR_INVALID, "fermionic lattice symmetries need the packed kernel (tables too large)");
    const int gpl = pick_gpl_for(p.group.n_elems);
    if (gpl < 0) return fail(LS_GPU_ERR_INVALID, "symmetry group too large for the matvec kernels");
    const SmemLayout L = make_layout(p, true);
    if (L.total > kMaxDynamicSmem) return fail(LS_GPU_ERR_INVALID, "term tables too large for shared memory");
    // the fallback kernel is compiled for at most 256 threads per block
    const LaunchShape shf{(int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sh.blocks * sh.threads / 256,
                                                                      (p.n_rows + 7) / 8)),
                          256};
    for (int c = 0; c < k; ++c) {
      const double* xs = d_x + (size_t)c * scalar_words;
      double* ys = d_y + (size_t)c * scalar_words;
      int rc = cplx ? launch_projected_cplx_k1(gpl, inv, p, L, shf, xs, ldx, ys, ldy, d_err, binom, s)
                    : launch_projected_real(gpl, inv, p, L, shf, xs, ldx, ys, ldy, d_err, binom, s);
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

// ------------------------------------------------------------------------------------------------
// Sector plans: y_s = H_s x_s for many sectors s in one persistent launch per RHS chunk.
// ------------------------------------------------------------------------------------------------
struct SectorPlan {
  int n_sectors = 0, k = 0;
  int64_t ldx = 0, ldy = 0;
  bool batched = false;
  MatvecProblem shared{};          // tables of the first sector (batched form)
  PackedLayout layout{};
  int64_t total_rows = 0;
  struct Chunk {
    int k;
    int col;
    SectorDesc* d_desc;
  };
  std::vector<Chunk> chunks;
  std::vector<MatvecProblem> problems;  // per-sector form
  std::vector<const double*> xs;
  std::vector<double*> ys;
};

int sector_plan_build(const std::vector<MatvecProblem>& problems, bool shareable, int k,
                      const std::vector<const double*>& xs, int64_t ldx, const std::vector<double*>& ys,
                      int64_t ldy, SectorPlan** out) {
  *out = nullptr;
  const int n = (int)problems.size();
  SectorPlan* plan = new SectorPlan();
  plan->n_sectors = n;
  plan->k = k;
  plan->ldx = ldx;
  plan->ldy = ldy;
  plan->problems = problems;
  plan->xs = xs;
  plan->ys = ys;
  const MatvecProblem& p0 = problems[0];
  plan->batched = shareable && n <= kMaxSectors && p0.projection == 2 && !p0.group.fermionic && p0.group.gpl >= 1 &&
                  p0.group.gpl <= kSectorMaxGpl && p0.group.onehot_packed != nullptr;
  if (plan->batched) {
    plan->shared = p0;
    plan->layout = make_packed_layout(p0, n);
    if (plan->layout.total > kMaxDynamicSmem) plan->batched = false;
  }
  if (plan->batched) {
    std::vector<SectorDesc> h(n);
    int64_t rows = 0;
    for (int i = 0; i < n; ++i) {
      h[i].index = problems[i].index;
      h[i].chars = problems[i].group.chars_packed;
      h[i].row_begin = rows;
      h[i].spin_inversion = problems[i].group.spin_inversion;
      h[i].real_elements = problems[i].real_elements;
      rows += problems[i].n_rows;
    }
    plan->total_rows = rows;
    int done = 0;
    while (done < k) {
      const int left = k - done;
      const int chunk = left >= 16 ? 16 : left >= 8 ? 8 : left >= 4 ? 4 : 1;
      for (int i = 0; i < n; ++i) {
        h[i].x = xs[i] + (size_t)done * 2;
        h[i].y = ys[i] + (size_t)done * 2;
      }
      SectorDesc* d = nullptr;
      if (!cuda_ok(cudaMalloc((void**)&d, (size_t)n * sizeof(SectorDesc)), "cudaMalloc(sector table)") ||
          !cuda_ok(cudaMemcpy(d, h.data(), (size_t)n * sizeof(SectorDesc), cudaMemcpyHostToDevice),
                   "upload sector table")) {
        sector_plan_free(plan);
        return LS_GPU_ERR_CUDA;
      }
      plan->chunks.push_back({chunk, done, d});
      done += chunk;
    }
  }
  *out = plan;
  return 0;
}

bool sector_plan_batched(const SectorPlan* plan) { return plan != nullptr && plan->batched; }

int sector_plan_run(const SectorPlan* plan, int* d_err, cudaStream_t s) {
  if (!plan->batched) {
    for (int i = 0; i < plan->n_sectors; ++i) {
      const int rc = launch_matvec(plan->problems[i], Scalar::Complex, plan->k, plan->xs[i], plan->ldx,
                                   plan->ys[i], plan->ldy, d_err, s);
      if (rc != 0) return rc;
    }
    return 0;
  }
  const uint64_t* binom = device_binomials();
  if (binom == nullptr) return LS_GPU_ERR_CUDA;
  if (plan->total_rows == 0) return 0;
  const LaunchShape sh = packed_shape(plan->total_rows);
  const bool inv = plan->shared.group.spin_inversion != 0;
  for (const SectorPlan::Chunk& c : plan->chunks) {
    const int rc = launch_sectors(c.k, plan->shared.group.gpl, inv, plan->shared, plan->layout, sh, c.d_desc,
                                  plan->n_sectors, plan->total_rows, plan->ldx, plan->ldy, d_err, binom, s);
    if (rc != 0) return rc;
  }
  return 0;
}

void sector_plan_free(SectorPlan* plan) {
  if (plan == nullptr) return;
  for (const SectorPlan::Chunk& c : plan->chunks) cudaFree(c.d_desc);
  delete plan;
}

}  // namespace lsg
