// matvec.cu -- launch policy of the gather kernels (kernel choice, grid shape, RHS blocking).
#include <algorithm>

#include "matvec_launch.cuh"

namespace lsg {

int launch_packed(bool cplx, int k, int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx,
                  double* y, int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s) {
  if (p.group.fermionic) {
    if (inv) return fail(LS_GPU_ERR_INVALID, "fermionic groups have no spin inversion");
    return launch_packed_fermi(cplx, k, gpl, p, x, ldx, y, ldy, err, binom, s);
  }
  if (!cplx) {
    switch (k) {
      case 1: return launch_packed_real(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
      case 2: return launch_packed_real_k2(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
      case 4: return launch_packed_real_k4(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
      case 8: return launch_packed_real_k8(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
      case 16: return launch_packed_real_k16(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
      default: return LS_GPU_ERR_INVALID;
    }
  }
  switch (k) {
    case 1: return launch_packed_cplx_k1(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    case 4: return launch_packed_cplx_k4(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    case 8: return launch_packed_cplx_k8(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    case 16: return launch_packed_cplx_k16(gpl, inv, p, x, ldx, y, ldy, err, binom, s);
    default: return LS_GPU_ERR_INVALID;
  }
}

static int g_threads_override = 0;
static int g_blocks_per_sm_override = 0;
static int g_rhs_tile = 16;  // most right-hand sides per launch (16, 8, 4 or 1)

int set_matvec_config(int threads, int blocks_per_sm) {
  // the warp-per-row kernels are compiled for at most 1024 threads per block (each kernel clamps
  // the setting to its own maximum)
  if (threads != 0 && (threads < 32 || threads > 1024 || threads % 32 != 0)) return LS_GPU_ERR_INVALID;
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

// Complex blocks of 8 or 16 right-hand sides: 0 = FP64 multiply-adds; 1 = FP32 pairs where the
// FP64 pipe bounds the kernel (groups of at most 64 elements: a short orbit scan per element
// against 4 FP64 FMAs per element and column); 2 = FP32 pairs for every group.  With larger
// groups the integer orbit scan is the bound and the pair form's extra instructions cost time.
// The default is FP64 (amplitudes stay FP64 unless a caller opts into pairs).
static int g_block_pairs = 0;

int set_block_arithmetic(int mode) {
  if (mode < 0 || mode > 2) return LS_GPU_ERR_INVALID;
  g_block_pairs = mode;
  return 0;
}

int get_block_arithmetic() { return g_block_pairs; }

static bool use_pairs(int gpl) { return g_block_pairs == 2 || (g_block_pairs == 1 && gpl <= 2); }

// Grid waves of the packed kernels when none is configured: several CTAs per SM slot over time
// balance the uneven per-row work of the last rows.
constexpr int kDefaultWaves = 4;

// threads 0: each kernel's own maximum; waves: grid = SMs x resident CTAs per SM x waves.
void get_matvec_config(int* threads, int* waves, int* rhs_tile) {
  if (threads) *threads = g_threads_override;
  if (waves) *waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : kDefaultWaves;
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

// xp[i][c] = x[i][c] * norms[i] as a float pair per component [re_h, re_l, im_h, im_l] for k
// complex columns (the gather source of the pair kernels).
__global__ void k_prescale_pairs(const double2* __restrict__ x, int64_t ldx, const double* __restrict__ norms,
                                 int64_t n, int k, float4* __restrict__ xp) {
  const int64_t total = n * k;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, c = e - i * k;
    const double nrm = __ldg(norms + i);
    const double2 v = __ldg(x + i * ldx + c);
    const F2 re = split_double(v.x * nrm), im = split_double(v.y * nrm);
    xp[e] = make_float4(re.h, re.l, im.h, im.l);
  }
}

int packed_launch_shape(const void* kern, int max_threads, const MatvecProblem& p, int n_sectors, int64_t rows,
                        LaunchShape* sh, PackedLayout* L) {
  const int waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : kDefaultWaves;
  int threads = g_threads_override > 0 ? std::min(g_threads_override, max_threads) : max_threads;
  for (; threads >= 64; threads -= 32) {
    *L = make_packed_layout(p, n_sectors, threads);
    if (L->total > kMaxDynamicSmem) continue;
    if (!ensure_smem_limit(kern, L->total)) return LS_GPU_ERR_CUDA;
    int resident = 0;
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, threads, L->total),
                 "occupancy of a packed kernel"))
      return LS_GPU_ERR_CUDA;
    if (resident < 1) continue;
    const int warps = threads / 32;
    int64_t blocks = (int64_t)num_sms() * resident * waves;
    blocks = std::min<int64_t>(blocks, (rows + warps - 1) / warps);
    *sh = LaunchShape{(int)std::max<int64_t>(blocks, 1), threads};
    return 0;
  }
  return fail(LS_GPU_ERR_INVALID, "packed matvec tables do not fit in shared memory");
}

// The packed tables fit in shared memory with at least two warps per CTA.
static bool packed_fits(const MatvecProblem& p, int n_sectors = 0) {
  return p.group.gpl > 0 && p.group.onehot_packed != nullptr &&
         make_packed_layout(p, n_sectors, 64).total <= kMaxDynamicSmem;
}

// Which kernel launch_matvec runs for `p`: 2 packed projected (*gpl = slots per lane), 1 the
// fallback projected kernel (*gpl = its slots per lane), 0 the thread-per-row kernel.
int matvec_kernel_form(const MatvecProblem& p, int* gpl) {
  *gpl = 0;
  if (p.projection != 2) return 0;
  if (packed_fits(p)) {
    *gpl = p.group.gpl;
    return 2;
  }
  *gpl = pick_gpl_for(p.group.n_elems);
  return 1;
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
    if (packed_fits(p)) {
      // Right-hand-side chunks of 16, 8, 4 and 1 columns; complex chunks of 8 or 16 run the
      // FP32-pair kernels (g_block_pairs).
      std::vector<int> chunks;
      for (int done = 0; done < k;) {
        const int left = k - done;
        const int most = std::min(left, g_rhs_tile);
        int chunk = most >= 16 ? 16 : most >= 8 ? 8 : most >= 4 ? 4 : 1;
        if (!cplx && left == 2 && g_rhs_tile >= 2) chunk = 2;
        if (p.group.fermionic && !cplx) chunk = 1;  // fermionic real path: one column per launch
        chunks.push_back(chunk);
        done += chunk;
      }
      // Gather sources x_j * n_j for all k columns (one streaming pass each), so that the kernels
      // read no norm per generated element: FP64 for the FP64 kernels, float pairs for the pair
      // kernels.  Not when counting elements (the count needs the norms).
      const bool can_prescale = p.nnz_counter == nullptr && p.index.norms != nullptr;
      const bool want_pairs = can_prescale && cplx && use_pairs(p.group.gpl) &&
                              std::any_of(chunks.begin(), chunks.end(), [](int c) { return c >= 8; });
      const bool want_fp64 = can_prescale && std::any_of(chunks.begin(), chunks.end(), [&](int c) {
                               return !(want_pairs && c >= 8);
                             });
      const int64_t total_elems = p.n_rows * (int64_t)k;
      const int pre_blocks = (int)std::max<int64_t>(
          1, std::min<int64_t>((total_elems * (int64_t)scalar_words + 255) / 256, (int64_t)num_sms() * 16));
      double* d_xs = nullptr;
      float4* d_xp = nullptr;
      if (want_fp64) {
        if (cudaMallocAsync((void**)&d_xs, (size_t)total_elems * scalar_words * sizeof(double), s) == cudaSuccess) {
          StageScope stage("matvec.prescale", s);
          k_prescale<<<pre_blocks, 256, 0, s>>>(d_x, ldx, p.index.norms, p.n_rows, k, (int)scalar_words, d_xs);
          if (!cuda_ok(cudaGetLastError(), "k_prescale")) {
            cudaFreeAsync(d_xs, s);
            return LS_GPU_ERR_CUDA;
          }
        } else {
          cudaGetLastError();  // a failed stream-ordered allocation: gather x and the norms instead
          d_xs = nullptr;
        }
      }
      if (want_pairs) {
        if (cudaMallocAsync((void**)&d_xp, (size_t)total_elems * sizeof(float4), s) == cudaSuccess) {
          StageScope stage("matvec.prescale", s);
          k_prescale_pairs<<<pre_blocks, 256, 0, s>>>(reinterpret_cast<const double2*>(d_x), ldx, p.index.norms,
                                                      p.n_rows, k, d_xp);
          if (!cuda_ok(cudaGetLastError(), "k_prescale_pairs")) {
            cudaFreeAsync(d_xp, s);
            if (d_xs) cudaFreeAsync(d_xs, s);
            return LS_GPU_ERR_CUDA;
          }
        } else {
          cudaGetLastError();  // no room for the pair copy: the FP64 kernels gather x and the norms
          d_xp = nullptr;
        }
      }
      MatvecProblem q = p;
      q.ldxs = k;
      int done = 0, rc = 0;
      for (const int chunk : chunks) {
        const double* xs = d_x + (size_t)done * scalar_words;
        double* ys = d_y + (size_t)done * scalar_words;
        StageScope stage("matvec.kernel", s);
        if (d_xp != nullptr && chunk >= 8) {
          q.xs = reinterpret_cast<const double*>(d_xp + done);
          rc = launch_packed_pair(chunk, p.group.gpl, inv, q, xs, ldx, ys, ldy, d_err, binom, s);
        } else {
          q.xs = d_xs ? d_xs + (size_t)done * scalar_words : nullptr;
          rc = launch_packed(cplx, chunk, p.group.gpl, inv, q, xs, ldx, ys, ldy, d_err, binom, s);
        }
        if (rc != 0) break;
        done += chunk;
      }
      if (d_xs) cudaFreeAsync(d_xs, s);
      if (d_xp) cudaFreeAsync(d_xp, s);
      return rc;
    }
    if (p.group.fermionic)
      return fail(LS_GPU_ERR_INVALID, "fermionic lattice symmetries need the packed kernel (tables too large)");
    const int gpl = pick_gpl_for(p.group.n_elems);
    if (gpl < 0) return fail(LS_GPU_ERR_INVALID, "symmetry group too large for the matvec kernels");
    const SmemLayout L = make_layout(p, true);
    if (L.total > kMaxDynamicSmem) return fail(LS_GPU_ERR_INVALID, "term tables too large for shared memory");
    // the fallback kernel is compiled for at most 256 threads per block (two CTAs per SM)
    const int waves = g_blocks_per_sm_override > 0 ? g_blocks_per_sm_override : 8;
    const LaunchShape shf{(int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms() * 2 * waves,
                                                                      (p.n_rows + 7) / 8)),
                          256};
    for (int c = 0; c < k; ++c) {
      const double* xs = d_x + (size_t)c * scalar_words;
      double* ys = d_y + (size_t)c * scalar_words;
      StageScope stage("matvec.kernel", s);
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
  StageScope stage("matvec.kernel", s);
  return launch_plain(cplx, p.projection == 1, k, p, L, sh, d_x, ldx, d_y, ldy, d_err, binom, s);
}

// ------------------------------------------------------------------------------------------------
// Sector plans: y_s = H_s x_s for many sectors s in one persistent launch per RHS chunk.
// ------------------------------------------------------------------------------------------------
struct SectorPlan {
  int n_sectors = 0, k = 0;
  int64_t ldx = 0, ldy = 0;
  bool batched = false;      // the sectors can share one launch
  bool use_batched = true;   // ... and run() does so (else one launch per sector)
  MatvecProblem shared{};          // tables of the first sector (batched form)
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
    if (!packed_fits(p0, n)) plan->batched = false;
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

bool sector_plan_batched(const SectorPlan* plan) { return plan != nullptr && plan->batched && plan->use_batched; }

int sector_plan_set_batched(SectorPlan* plan, bool batched) {
  if (plan == nullptr || (batched && !plan->batched)) return LS_GPU_ERR_INVALID;
  plan->use_batched = batched;
  return 0;
}

// Gather source of the pair kernels in a batched launch: xp[row_begin_s + i][c] = x_s[i][c] *
// n_s[i] as float pairs, for every sector s (blockIdx.y) and all k complex columns.
__global__ void k_prescale_pairs_sectors(const SectorDesc* __restrict__ desc, int n_sectors, int64_t total_rows,
                                         int k, int64_t ldx, float4* __restrict__ xp) {
  const int s = blockIdx.y;
  const int64_t begin = desc[s].row_begin;
  const int64_t n = (s + 1 < n_sectors ? desc[s + 1].row_begin : total_rows) - begin;
  const double2* __restrict__ x = reinterpret_cast<const double2*>(desc[s].x);
  const double* __restrict__ norms = desc[s].index.norms;
  float4* __restrict__ out = xp + (size_t)begin * k;
  const int64_t total = n * k;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, c = e - i * k;
    const double nrm = __ldg(norms + i);
    const double2 v = __ldg(x + i * ldx + c);
    const F2 re = split_double(v.x * nrm), im = split_double(v.y * nrm);
    out[e] = make_float4(re.h, re.l, im.h, im.l);
  }
}

int sector_plan_run(const SectorPlan* plan, int* d_err, cudaStream_t s) {
  if (!plan->batched || !plan->use_batched) {
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
  const bool inv = plan->shared.group.spin_inversion != 0;
  // chunks of 8 or 16 columns run the FP32-pair kernels from a prescaled pair copy of all
  // sectors' columns (one streaming pass); the others gather x and the norms in FP64
  float4* d_xp = nullptr;
  const bool want_pairs = use_pairs(plan->shared.group.gpl) && plan->shared.nnz_counter == nullptr &&
                          std::any_of(plan->chunks.begin(), plan->chunks.end(),
                                      [](const SectorPlan::Chunk& c) { return c.k >= 8; });
  if (want_pairs) {
    if (cudaMallocAsync((void**)&d_xp, (size_t)plan->total_rows * plan->k * sizeof(float4), s) == cudaSuccess) {
      const int n = plan->n_sectors;
      const int64_t per_sector = (plan->total_rows * plan->k + n - 1) / n;
      const int bx = (int)std::max<int64_t>(1, std::min<int64_t>((per_sector + 255) / 256,
                                                                 ((int64_t)num_sms() * 16 + n - 1) / n));
      StageScope stage("sectors.prescale", s);
      k_prescale_pairs_sectors<<<dim3((unsigned)bx, (unsigned)n), 256, 0, s>>>(
          plan->chunks[0].d_desc, n, plan->total_rows, plan->k, plan->ldx, d_xp);
      if (!cuda_ok(cudaGetLastError(), "k_prescale_pairs_sectors")) {
        cudaFreeAsync(d_xp, s);
        return LS_GPU_ERR_CUDA;
      }
    } else {
      cudaGetLastError();  // no room for the pair copy: FP64 kernels
      d_xp = nullptr;
    }
  }
  int rc = 0;
  for (const SectorPlan::Chunk& c : plan->chunks) {
    StageScope stage("sectors.kernel", s);
    if (d_xp != nullptr && c.k >= 8)
      rc = launch_sectors_pair(c.k, plan->shared.group.gpl, inv, plan->shared, plan->n_sectors, c.d_desc,
                               plan->n_sectors, plan->total_rows, plan->ldx, plan->ldy, d_err, binom,
                               reinterpret_cast<const double*>(d_xp), plan->k, c.col, s);
    else
      rc = launch_sectors(c.k, plan->shared.group.gpl, inv, plan->shared, plan->n_sectors, c.d_desc,
                          plan->n_sectors, plan->total_rows, plan->ldx, plan->ldy, d_err, binom, nullptr, 0, 0, s);
    if (rc != 0) break;
  }
  if (d_xp) cudaFreeAsync(d_xp, s);
  return rc;
}

void sector_plan_free(SectorPlan* plan) {
  if (plan == nullptr) return;
  for (const SectorPlan::Chunk& c : plan->chunks) cudaFree(c.d_desc);
  delete plan;
}

}  // namespace lsg
