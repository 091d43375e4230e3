// basis.cu -- orbit scan, basis enumeration and state index on sm_103a.
//
// Orbit scan (kernels/generator.cpp:10-272 of the reference, Halide on x86): for a state x and
// every group element g, g.x is computed by the element's Benes network (bit_permute_step,
// generator.cpp:5-8) and the candidates g.x (and g.x ^ flip under spin inversion) are reduced
// to the representative, its character and the stabiliser sum.
//
//  * state_info: thread per state, uniform loop over g (masks are warp-broadcast loads).  The
//    winner among equal minima follows the reference's Halide reduction order: lanes
//    j = e mod W over chunks e / W, lanes combined in order, tail elements last, the initial
//    candidate (x, character 1) first (generator.cpp:77-128).  The stabiliser sum is exact:
//    |Stab| when every stabiliser character has real part exactly 1, else 0.
//  * is_representative: thread per state, reproduces the reference's float summation order
//    and early exit (generator.cpp:181-253), so flags and norms are bit-identical to the
//    reference built with lane width W.
//  * enumeration: candidates in increasing order (combinadics unrank + Gosper steps,
//    StatesEnumeration.chpl:29-32), one tile of blockDim*K candidates per block, flags kept
//    as per-thread bit masks, block scan, a run per tile in an append buffer, an exclusive
//    scan over tile counts, and a final ordered gather; the output is sorted.
//  * state index: the prefix-bucket table of kernels/indexing.c:45-117 built on the GPU and
//    a branch-free window search (indexing.c:196-215).
#include <algorithm>
#include <cstdio>
#include <vector>

#include "lsg.h"

namespace lsg {

__constant__ uint64_t c_binom[65][65];
static bool g_binom_uploaded[64] = {false};

static void host_binomials(uint64_t (*b)[65]) {
  for (int n = 0; n <= 64; ++n)
    for (int k = 0; k <= 64; ++k) b[n][k] = 0;
  b[0][0] = 1;
  for (int n = 1; n <= 64; ++n) {
    b[n][0] = 1;
    for (int k = 1; k <= n; ++k) b[n][k] = b[n - 1][k - 1] + b[n - 1][k];
  }
}

static int ensure_binomials() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && g_binom_uploaded[dev]) return 0;
  static uint64_t table[65][65];
  host_binomials(table);
  if (!cuda_ok(cudaMemcpyToSymbol(c_binom, table, sizeof(table)), "upload binomials")) return -1;
  if (dev < 64) g_binom_uploaded[dev] = true;
  return 0;
}

// binomial n k = 0 when n <= 0 or k > n (Basis.hs:506-509)
__host__ __device__ inline uint64_t binom_rule(const uint64_t (*b)[65], int n, int k) {
  if (n <= 0 || k > n) return 0;
  return b[n][k];
}

int64_t fixed_hamming_state_to_index(uint64_t a) {
  static uint64_t table[65][65];
  static bool ready = false;
  if (!ready) {
    host_binomials(table);
    ready = true;
  }
  int64_t i = 0;
  for (int k = 1; a != 0; ++k) {
    int c = __builtin_ctzll(a);
    a &= a - 1;
    i += (int64_t)binom_rule(table, c, k);
  }
  return i;
}

uint64_t fixed_hamming_index_to_state(int64_t index, int h) {
  static uint64_t table[65][65];
  static bool ready = false;
  if (!ready) {
    host_binomials(table);
    ready = true;
  }
  uint64_t state = 0;
  for (int i = h; i > 0; --i) {
    int c = i - 1;
    uint64_t contribution = binom_rule(table, c, i);
    while (c < 64) {
      uint64_t nc = binom_rule(table, c + 1, i);
      if ((int64_t)nc > index) break;
      ++c;
      contribution = nc;
    }
    state |= (uint64_t)1 << c;
    index -= (int64_t)contribution;
  }
  return state;
}

__device__ inline uint64_t d_binom(int n, int k) {
  if (n <= 0 || k > n) return 0;
  return c_binom[n][k];
}

// Unrank with a downward scan: the bit positions decrease with i, so the total work is
// O(n_bits + h) instead of O(n_bits * h).
__device__ inline uint64_t d_unrank(int64_t index, int h, int n_bits) {
  uint64_t state = 0;
  int c = n_bits - 1;
  for (int i = h; i > 0; --i) {
    while (c >= i && (int64_t)d_binom(c, i) > index) --c;
    if (c < i - 1) c = i - 1;
    uint64_t contribution = d_binom(c, i);
    state |= (uint64_t)1 << c;
    index -= (int64_t)contribution;
    --c;
  }
  return state;
}

__device__ inline int64_t d_rank(uint64_t a) {
  int64_t i = 0;
  for (int k = 1; a != 0; ++k) {
    int c = __ffsll((long long)a) - 1;
    a &= a - 1;
    i += (int64_t)d_binom(c, k);
  }
  return i;
}

__device__ inline uint64_t next_fixed_hamming(uint64_t v) {
  uint64_t t = v | (v - 1);
  return (t + 1) | (((~t & (t + 1)) - 1) >> (__ffsll((long long)v)));
}

// ------------------------------------------------------------------------------------------------
// Benes network application.  DEPTH > 0: stage distances 1,2,..,2^(h-1),..,2,1 known at compile
// time; DEPTH < 0: runtime distances.
// ------------------------------------------------------------------------------------------------
template <int DEPTH>
__device__ __forceinline__ uint64_t benes(uint64_t x, const uint64_t* __restrict__ m,
                                          const uint32_t* __restrict__ shifts, int depth) {
  if constexpr (DEPTH > 0) {
    constexpr int half = (DEPTH + 1) / 2;
#pragma unroll
    for (int k = 0; k < DEPTH; ++k) {
      const int d = (k < half) ? (1 << k) : (1 << (DEPTH - 1 - k));
      const uint64_t mk = __ldg(m + k);
      const uint64_t y = ((x >> d) ^ x) & mk;
      x = x ^ y ^ (y << d);
    }
    return x;
  } else if constexpr (DEPTH == 0) {
    return x;
  } else {
    for (int k = 0; k < depth; ++k) {
      const uint32_t d = __ldg(shifts + k);
      const uint64_t mk = __ldg(m + k);
      const uint64_t y = ((x >> d) ^ x) & mk;
      x = x ^ y ^ (y << d);
    }
    return x;
  }
}

// ------------------------------------------------------------------------------------------------
// state_info
// ------------------------------------------------------------------------------------------------
template <int DEPTH>
__global__ void k_state_info(DeviceGroup g, int64_t n, const uint64_t* __restrict__ xs,
                             uint64_t* __restrict__ reps, double2* __restrict__ chars,
                             double* __restrict__ norms) {
  const int G = g.n_elems;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = xs[i];
    uint64_t best = a;
    uint32_t bestkey = 0;  // the initial candidate (a, character 1) has the smallest key
    int bestg = -1, bestf = 0;
    int count = 0;
    bool trivial = true;
    for (int e = 0; e < G; ++e) {
      const uint64_t y = benes<DEPTH>(a, g.masks_t + (int64_t)e * g.depth, g.shifts, g.depth);
      const uint32_t key = 2u * (uint32_t)__ldg(g.prio + e);
      const double cre = __ldg(&g.chars[e].x);
      if (y < best || (y == best && key < bestkey)) {
        best = y; bestkey = key; bestg = e; bestf = 0;
      }
      if (y == a) {
        ++count;
        const double sg = (g.fermionic && fermion_parity(g.fsign + (int64_t)e * g.n_bits, 1, a)) ? -1.0 : 1.0;
        if (sg * cre != 1.0) trivial = false;
      }
      if (g.spin_inversion != 0) {
        const uint64_t yf = y ^ g.flip;
        if (yf < best || (yf == best && key + 1 < bestkey)) {
          best = yf; bestkey = key + 1; bestg = e; bestf = 1;
        }
        if (yf == a) {
          ++count;
          if ((double)g.spin_inversion * cre != 1.0) trivial = false;
        }
      }
    }
    double2 ch = make_double2(1.0, 0.0);
    if (bestg >= 0) {
      ch = g.chars[bestg];
      if (bestf && g.spin_inversion == -1) ch = make_double2(-ch.x, -ch.y);
      if (g.fermionic && fermion_parity(g.fsign + (int64_t)bestg * g.n_bits, 1, a)) ch = make_double2(-ch.x, -ch.y);
    }
    reps[i] = best;
    chars[i] = ch;
    const double denom = (double)(g.spin_inversion == 0 ? G : 2 * G);
    norms[i] = sqrt((trivial ? (double)count : 0.0) / denom);
  }
}

// Norms sqrt(S/|G|) of representatives (exact stabiliser rule).
template <int DEPTH>
__global__ void k_orbit_norms(DeviceGroup g, int64_t n, const uint64_t* __restrict__ xs,
                              double* __restrict__ norms) {
  const int G = g.n_elems;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = xs[i];
    int count = 0;
    bool trivial = true;
    for (int e = 0; e < G; ++e) {
      const uint64_t y = benes<DEPTH>(a, g.masks_t + (int64_t)e * g.depth, g.shifts, g.depth);
      const double cre = __ldg(&g.chars[e].x);
      if (y == a) {
        ++count;
        const double sg = (g.fermionic && fermion_parity(g.fsign + (int64_t)e * g.n_bits, 1, a)) ? -1.0 : 1.0;
        if (sg * cre != 1.0) trivial = false;
      }
      if (g.spin_inversion != 0 && (y ^ g.flip) == a) {
        ++count;
        if ((double)g.spin_inversion * cre != 1.0) trivial = false;
      }
    }
    const double denom = (double)(g.spin_inversion == 0 ? G : 2 * G);
    norms[i] = sqrt((trivial ? (double)count : 0.0) / denom);
  }
}

// ------------------------------------------------------------------------------------------------
// is_representative (reference float order, lane width W)
// ------------------------------------------------------------------------------------------------
struct IsRepResult {
  double sum;       // the reference's floating stabiliser sum (partial for non-representatives)
  bool ok;          // no smaller image
  int exact_count;  // exact stabiliser count
  bool trivial;     // every stabiliser character has real part 1
};

template <int DEPTH>
__device__ __forceinline__ void ir_term(const DeviceGroup& g, uint64_t a, int e, double& s,
                                        bool& ge, int& cnt, bool& trivial) {
  const uint64_t y = benes<DEPTH>(a, g.masks_t + (int64_t)e * g.depth, g.shifts, g.depth);
  const double cre = __ldg(&g.chars[e].x);
  if (g.spin_inversion == 0) {
    const bool eq = (y == a);
    double c = cre;
    if (eq && g.fermionic && fermion_parity(g.fsign + (int64_t)e * g.n_bits, 1, a)) c = -cre;
    s = eq ? c : 0.0;
    ge = y >= a;
    if (eq) {
      ++cnt;
      if (c != 1.0) trivial = false;
    }
  } else {
    const uint64_t yf = y ^ g.flip;
    const double p = (double)(y == a), q = (double)(yf == a);
    s = (g.spin_inversion == 1 ? p + q : p - q) * cre;
    ge = (y >= a) && (yf >= a);
    if (y == a) {
      ++cnt;
      if (cre != 1.0) trivial = false;
    }
    if (yf == a) {
      ++cnt;
      if ((double)g.spin_inversion * cre != 1.0) trivial = false;
    }
  }
}

// early_exit: stop at the first smaller image (the sum is then irrelevant for the caller).
template <int DEPTH>
__device__ IsRepResult is_rep(const DeviceGroup& g, uint64_t a, int W, bool early_exit) {
  const int G = g.n_elems;
  const int nchunks = G / W;
  IsRepResult r{0.0, true, 0, true};
  for (int m = 0; m < nchunks && r.ok; ++m) {
    double ls = 0.0;
    bool lok = true;
    for (int j = 0; j < W; ++j) {
      double s;
      bool ge;
      ir_term<DEPTH>(g, a, m * W + j, s, ge, r.exact_count, r.trivial);
      ls = ls + s;
      lok = lok && ge;
      if (early_exit && !ge) {
        r.ok = false;
        return r;
      }
    }
    r.sum = r.sum + ls;
    r.ok = r.ok && lok;
  }
  for (int e = nchunks * W; e < G; ++e) {
    double s;
    bool ge;
    ir_term<DEPTH>(g, a, e, s, ge, r.exact_count, r.trivial);
    r.sum = r.sum + s;
    r.ok = r.ok && ge;
    if (early_exit && !ge) return r;
  }
  return r;
}

template <int DEPTH>
__global__ void k_is_representative(DeviceGroup g, int64_t n, const uint64_t* __restrict__ xs,
                                    uint8_t* __restrict__ flags, double* __restrict__ norms, int W) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    IsRepResult r = is_rep<DEPTH>(g, xs[i], W, false);
    norms[i] = r.sum;
    flags[i] = (r.sum > 0) ? (uint8_t)r.ok : (uint8_t)0;
  }
}

// ------------------------------------------------------------------------------------------------
// Depth dispatch
// ------------------------------------------------------------------------------------------------
static bool standard_shifts(const DeviceGroup& g, const std::vector<uint32_t>& shifts) {
  const int D = (int)shifts.size();
  const int half = (D + 1) / 2;
  for (int k = 0; k < D; ++k) {
    const uint32_t d = (k < half) ? (1u << k) : (1u << (D - 1 - k));
    if (shifts[k] != d) return false;
  }
  (void)g;
  return true;
}

template <template <int> class F, typename... Args>
static void dispatch_depth(int depth, bool standard, Args&&... args) {
  if (!standard) {
    F<-1>::run(args...);
    return;
  }
  switch (depth) {
    case 0: F<0>::run(args...); break;
    case 1: F<1>::run(args...); break;
    case 3: F<3>::run(args...); break;
    case 5: F<5>::run(args...); break;
    case 7: F<7>::run(args...); break;
    case 9: F<9>::run(args...); break;
    case 11: F<11>::run(args...); break;
    default: F<-1>::run(args...); break;
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t blocks = (n + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms() * 32;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

template <int D>
struct RunStateInfo {
  static void run(const DeviceGroup& g, int64_t n, const uint64_t* x, uint64_t* r, double2* c,
                  double* nm, cudaStream_t s) {
    k_state_info<D><<<grid_for(n, 256), 256, 0, s>>>(g, n, x, r, c, nm);
  }
};
template <int D>
struct RunIsRep {
  static void run(const DeviceGroup& g, int64_t n, const uint64_t* x, uint8_t* f, double* nm,
                  int W, cudaStream_t s) {
    k_is_representative<D><<<grid_for(n, 256), 256, 0, s>>>(g, n, x, f, nm, W);
  }
};
template <int D>
struct RunNorms {
  static void run(const DeviceGroup& g, int64_t n, const uint64_t* x, double* nm, cudaStream_t s) {
    k_orbit_norms<D><<<grid_for(n, 256), 256, 0, s>>>(g, n, x, nm);
  }
};

static bool group_is_standard(const DeviceGroup& g) {
  // OrbitData validates the shifts when it is created; a group with non-standard distances
  // carries depth with bit 30 set (see compute_site_images).
  return (g.depth & (1 << 30)) == 0;
}

static DeviceGroup strip(const DeviceGroup& g) {
  DeviceGroup h = g;
  h.depth &= ~(1 << 30);
  return h;
}

__global__ void k_inverse_norms(const double* __restrict__ norms, int64_t n, double* __restrict__ inv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = norms[i];
    inv[i] = v == 0.0 ? 0.0 : 1.0 / v;
  }
}

int launch_inverse_norms(const double* d_norms, int64_t n, double* d_inv, cudaStream_t s) {
  if (n <= 0) return 0;
  k_inverse_norms<<<grid_for(n, 256), 256, 0, s>>>(d_norms, n, d_inv);
  return cuda_ok(cudaGetLastError(), "k_inverse_norms") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_state_info(const DeviceGroup& g0, int64_t n, const uint64_t* d_x, uint64_t* d_rep,
                      double2* d_char, double* d_norm, int lane_width, cudaStream_t s) {
  (void)lane_width;  // encoded in g.prio
  if (n <= 0) return 0;
  DeviceGroup g = strip(g0);
  dispatch_depth<RunStateInfo>(g.depth, group_is_standard(g0), g, n, d_x, d_rep, d_char, d_norm, s);
  return cuda_ok(cudaGetLastError(), "k_state_info") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_is_representative(const DeviceGroup& g0, int64_t n, const uint64_t* d_x,
                             uint8_t* d_flag, double* d_norm, int lane_width, cudaStream_t s) {
  if (n <= 0) return 0;
  DeviceGroup g = strip(g0);
  dispatch_depth<RunIsRep>(g.depth, group_is_standard(g0), g, n, d_x, d_flag, d_norm, lane_width, s);
  return cuda_ok(cudaGetLastError(), "k_is_representative") ? 0 : LS_GPU_ERR_CUDA;
}

int launch_orbit_norms(const DeviceGroup& g0, int64_t n, const uint64_t* d_reps, double* d_norms,
                       cudaStream_t s) {
  if (n <= 0) return 0;
  StageScope stage("basis.orbit_norms", s);
  DeviceGroup g = strip(g0);
  dispatch_depth<RunNorms>(g.depth, group_is_standard(g0), g, n, d_reps, d_norms, s);
  return cuda_ok(cudaGetLastError(), "k_orbit_norms") ? 0 : LS_GPU_ERR_CUDA;
}

// ------------------------------------------------------------------------------------------------
// Site images: onehot[b][e] = image of 1<<b under element e.  Host side, from the masks.
// ------------------------------------------------------------------------------------------------
int compute_site_images(OrbitData* od) {
  const int G = od->n_elems, B = od->n_bits, D = od->depth;
  std::vector<uint64_t> onehot((size_t)B * G);
  for (int e = 0; e < G; ++e) {
    for (int b = 0; b < B; ++b) {
      uint64_t x = (uint64_t)1 << b;
      for (int k = 0; k < D; ++k) {
        const uint64_t m = od->masks[(size_t)k * G + e];
        const uint32_t d = od->shifts[k];
        const uint64_t y = ((x >> d) ^ x) & m;
        x = x ^ y ^ (y << d);
      }
      onehot[(size_t)b * G + e] = x;
    }
  }
  // Priority of element e in the reference's state_info reduction with lane width 8.
  const int W = 8;
  const int nchunks = G / W;
  std::vector<uint16_t> prio(G);
  for (int e = 0; e < G; ++e) {
    prio[e] = (uint16_t)((e < nchunks * W) ? ((e % W) * nchunks + e / W + 1) : (e + 1));
  }
  std::vector<uint64_t> masks_t((size_t)G * D);
  for (int e = 0; e < G; ++e)
    for (int k = 0; k < D; ++k) masks_t[(size_t)e * D + k] = od->masks[(size_t)k * G + e];
  std::vector<double2> chars(G);
  for (int e = 0; e < G; ++e) chars[e] = make_double2(od->chars_re[e], od->chars_im[e]);

  // Packed tables of the matvec kernels (see DeviceGroup::onehot_packed).  Available when the
  // bits below the shifted state can hold the candidate index 2 * slot + flip.
  int gpl = G > 0 ? pick_gpl_for(G) : -1;
  if (gpl > 0) {
    const int idx_bits = 32 - __builtin_clz((unsigned)(2 * 32 * gpl - 1));
    if (B < 1 || 64 - B < idx_bits) gpl = -1;
  }
  const int Gp = gpl > 0 ? 32 * gpl : 0;
  std::vector<uint64_t> onehot_packed((size_t)B * Gp);
  std::vector<double2> chars_packed(Gp);
  for (int s = 0; s < Gp; ++s) {
    const int e = s < G ? s : 0;
    chars_packed[s] = chars[e];
    for (int b = 0; b < B; ++b) onehot_packed[(size_t)b * Gp + s] = onehot[(size_t)b * G + e] << (64 - B);
  }
  od->gpl = gpl > 0 ? gpl : 0;

  // Fermionic sign tables: g moves orbital k to g(k) = position of the image of 1 << k, and
  // L_g[k] holds the orbitals l < k with g(l) > g(k) (the pairs whose order g reverses).
  std::vector<uint64_t> fsign, fsign_packed;
  if (od->fermionic) {
    fsign.assign((size_t)G * B, 0);
    for (int e = 0; e < G; ++e) {
      for (int k = 0; k < B; ++k) {
        const int gk = __builtin_ctzll(onehot[(size_t)k * G + e]);
        uint64_t m = 0;
        for (int l = 0; l < k; ++l)
          if (__builtin_ctzll(onehot[(size_t)l * G + e]) > gk) m |= (uint64_t)1 << l;
        fsign[(size_t)e * B + k] = m;
      }
    }
    fsign_packed.assign((size_t)B * Gp, 0);
    for (int s = 0; s < Gp; ++s) {
      const int e = s < G ? s : 0;
      for (int k = 0; k < B; ++k) fsign_packed[(size_t)k * Gp + s] = fsign[(size_t)e * B + k];
    }
  }

  // One block: masks_t | shifts | chars | onehot | prio | onehot_packed | chars_packed
  // [| fsign | fsign_packed] (16-byte aligned pieces).
  auto align16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  od->off_masks = 0;
  od->off_shifts = align16(od->off_masks + masks_t.size() * 8);
  od->off_chars = align16(od->off_shifts + (size_t)std::max(D, 1) * 4);
  od->off_onehot = align16(od->off_chars + (size_t)std::max(G, 1) * 16);
  od->off_prio = align16(od->off_onehot + std::max<size_t>(onehot.size(), 1) * 8);
  od->off_onehot_packed = align16(od->off_prio + (size_t)std::max(G, 1) * 2);
  od->off_chars_packed = align16(od->off_onehot_packed + std::max<size_t>(onehot_packed.size(), 1) * 8);
  od->off_fsign = align16(od->off_chars_packed + (size_t)std::max(Gp, 1) * 16);
  od->off_fsign_packed = align16(od->off_fsign + fsign.size() * 8);
  const size_t total = align16(od->off_fsign_packed + fsign_packed.size() * 8) + 16;
  od->host_block.assign(total, 0);
  uint8_t* h = od->host_block.data();
  if (!masks_t.empty()) memcpy(h + od->off_masks, masks_t.data(), masks_t.size() * 8);
  if (D > 0) memcpy(h + od->off_shifts, od->shifts.data(), (size_t)D * 4);
  if (G > 0) memcpy(h + od->off_chars, chars.data(), (size_t)G * 16);
  if (!onehot.empty()) memcpy(h + od->off_onehot, onehot.data(), onehot.size() * 8);
  if (G > 0) memcpy(h + od->off_prio, prio.data(), (size_t)G * 2);
  if (!onehot_packed.empty())
    memcpy(h + od->off_onehot_packed, onehot_packed.data(), onehot_packed.size() * 8);
  if (Gp > 0) memcpy(h + od->off_chars_packed, chars_packed.data(), (size_t)Gp * 16);
  if (!fsign.empty()) memcpy(h + od->off_fsign, fsign.data(), fsign.size() * 8);
  if (!fsign_packed.empty()) memcpy(h + od->off_fsign_packed, fsign_packed.data(), fsign_packed.size() * 8);
  DeviceGroup probe;
  od->standard_shifts = standard_shifts(probe, od->shifts);
  return 0;
}

const DeviceGroup* orbit_device(const OrbitData* od) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (od->dev_block != nullptr) {
    if (od->dev_device == dev) return &od->dev;
    set_error("orbit data was uploaded to another device");
    return nullptr;
  }
  void* d = nullptr;
  const size_t total = od->host_block.size();
  if (!cuda_ok(cudaMalloc(&d, total), "cudaMalloc(orbit data)")) return nullptr;
  if (!cuda_ok(cudaMemcpy(d, od->host_block.data(), total, cudaMemcpyHostToDevice), "upload orbit data")) {
    cudaFree(d);
    return nullptr;
  }
  uint8_t* base = (uint8_t*)d;
  DeviceGroup& g = od->dev;
  g.n_bits = od->n_bits;
  g.n_elems = od->n_elems;
  g.depth = od->depth;
  if (!od->standard_shifts) g.depth |= (1 << 30);
  g.spin_inversion = od->spin_inversion;
  g.flip = od->n_bits == 0 ? 0 : (~(uint64_t)0) >> (64 - od->n_bits);
  g.masks_t = (const uint64_t*)(base + od->off_masks);
  g.shifts = (const uint32_t*)(base + od->off_shifts);
  g.chars = (const double2*)(base + od->off_chars);
  g.onehot = (const uint64_t*)(base + od->off_onehot);
  g.prio = (const uint16_t*)(base + od->off_prio);
  g.gpl = od->gpl;
  g.onehot_packed = od->gpl > 0 ? (const uint64_t*)(base + od->off_onehot_packed) : nullptr;
  g.chars_packed = od->gpl > 0 ? (const double2*)(base + od->off_chars_packed) : nullptr;
  g.fermionic = od->fermionic;
  g.fsign = od->fermionic ? (const uint64_t*)(base + od->off_fsign) : nullptr;
  g.fsign_packed = (od->fermionic && od->gpl > 0) ? (const uint64_t*)(base + od->off_fsign_packed) : nullptr;
  od->dev_block = d;
  od->dev_device = dev;
  return &od->dev;
}

// ------------------------------------------------------------------------------------------------
// Exclusive scan (int32 counts -> int64 offsets), three phases per level.
// ------------------------------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* warp_sums, int64_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += t;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int64_t w = lane < nw ? warp_sums[lane] : 0;
    int64_t winc = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, winc, d);
      if (lane >= d) winc += t;
    }
    if (lane < nw) warp_sums[lane] = winc - w;
    if (lane == nw - 1) *total = winc;
  }
  __syncthreads();
  int64_t r = inc - v + warp_sums[warp];
  __syncthreads();
  return r;
}

template <typename In>
__global__ void k_scan_tiles(const In* __restrict__ in, int64_t n, int64_t* __restrict__ out,
                             int64_t* __restrict__ tile_sums) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t vals[kScanItems];
  int64_t local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    vals[k] = (base + k < n) ? (int64_t)in[base + k] : 0;
    local += vals[k];
  }
  int64_t excl = block_exclusive_scan(local, warp_sums, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = excl;
    excl += vals[k];
  }
  if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ tile_off) {
  const int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  const int64_t add = tile_off[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t j = i + (int64_t)k * kScanThreads;
    if (j < n) out[j] += add;
  }
}

// out[i] = sum_{k<i} in[k]; out has n + 1 entries (out[n] = total).
template <typename In>
static int exclusive_scan(const In* d_in, int64_t n, int64_t* d_out, cudaStream_t s) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (n == 0) {
    return cuda_ok(cudaMemsetAsync(d_out, 0, sizeof(int64_t), s), "scan") ? 0 : LS_GPU_ERR_CUDA;
  }
  int64_t* sums = nullptr;
  int64_t* sums_scan = nullptr;
  if (!cuda_ok(cudaMallocAsync((void**)&sums, (tiles + 1) * sizeof(int64_t), s), "scan alloc") ||
      !cuda_ok(cudaMallocAsync((void**)&sums_scan, (tiles + 1) * sizeof(int64_t), s), "scan alloc"))
    return LS_GPU_ERR_CUDA;
  k_scan_tiles<In><<<(unsigned)tiles, kScanThreads, 0, s>>>(d_in, n, d_out, sums);
  int rc = 0;
  if (tiles > 1) {
    rc = exclusive_scan<int64_t>(sums, tiles, sums_scan, s);
    if (rc == 0) k_scan_add<<<(unsigned)tiles, kScanThreads, 0, s>>>(d_out, n, sums_scan);
    // total = scan of sums at position tiles
    if (rc == 0)
      rc = cuda_ok(cudaMemcpyAsync(d_out + n, sums_scan + tiles, sizeof(int64_t),
                                   cudaMemcpyDeviceToDevice, s), "scan total") ? 0 : LS_GPU_ERR_CUDA;
  } else {
    rc = cuda_ok(cudaMemcpyAsync(d_out + n, sums, sizeof(int64_t), cudaMemcpyDeviceToDevice, s),
                 "scan total") ? 0 : LS_GPU_ERR_CUDA;
  }
  cudaFreeAsync(sums, s);
  cudaFreeAsync(sums_scan, s);
  if (!cuda_ok(cudaGetLastError(), "exclusive_scan")) return LS_GPU_ERR_CUDA;
  return rc;
}

int exclusive_scan_counts(const int32_t* d_in, int64_t n, int64_t* d_out, cudaStream_t s) {
  return exclusive_scan<int32_t>(d_in, n, d_out, s);
}

// ------------------------------------------------------------------------------------------------
// Enumeration
// ------------------------------------------------------------------------------------------------
constexpr int kEnumThreads = 256;
constexpr int kEnumPerThread = 16;
constexpr int64_t kEnumTile = (int64_t)kEnumThreads * kEnumPerThread;

struct EnumArgs {
  int64_t first_rank;    // rank of the first candidate (fixed weight) / value (all states)
  int64_t n_candidates;
  int h;                 // Hamming weight, -1 for +1 stepping
  int n_bits;
  int lane_width;        // W of the reference's is_representative
  int reference_rule;
  int64_t n_tiles;
  int32_t* tile_count;
  int64_t* tile_start;
  uint64_t* append;
  int64_t capacity;
  unsigned long long* counter;
  // Spinful fermions (mode 3): candidate (iB, iA) = (idx / nA, idx % nA) is
  // unrank(rankB + iB, hB) << ns | unrank(rankA + iA, hA), ascending.
  int spinful;
  int ns, hA, hB;
  int64_t rankA, rankB, nA;
  uint64_t minA, maxA;
};

__device__ inline uint64_t candidate_at(const EnumArgs& a, int64_t idx) {
  if (a.spinful) {
    const int64_t iB = idx / a.nA, iA = idx - iB * a.nA;
    return (d_unrank(a.rankB + iB, a.hB, a.ns) << a.ns) | d_unrank(a.rankA + iA, a.hA, a.ns);
  }
  return a.h >= 0 ? d_unrank(a.first_rank + idx, a.h, a.n_bits) : (uint64_t)(a.first_rank + idx);
}
// Successor of candidate v (only called while another candidate follows in the range).
__device__ inline uint64_t candidate_next(const EnumArgs& a, uint64_t v) {
  if (a.spinful) {
    const uint64_t mask = (~0ull) >> (64 - a.ns);
    const uint64_t A = v & mask;
    if (A == a.maxA) return (next_fixed_hamming(v >> a.ns) << a.ns) | a.minA;
    return (v & ~mask) | next_fixed_hamming(A);
  }
  return a.h >= 0 ? next_fixed_hamming(v) : v + 1;
}

// Candidate range of a projected enumeration: fixed Hamming weight / all states of n_bits
// (mode 0), or the (N_up, N_down) product range of spinful fermions (mode 3).
static void projected_candidates(const EnumerateRequest& req, int n_bits, EnumArgs* a) {
  a->n_bits = n_bits;
  a->lane_width = 4;
  a->reference_rule = req.reference_norm_rule;
  if (req.mode == 3) {
    const int ns = req.number_sites;
    const uint64_t mask = (~0ull) >> (64 - ns);
    a->spinful = 1;
    a->h = -1;
    a->ns = ns;
    a->minA = req.lower & mask;
    a->maxA = req.upper & mask;
    const uint64_t minB = (req.lower >> ns) & mask, maxB = (req.upper >> ns) & mask;
    a->hA = __builtin_popcountll(a->minA);
    a->hB = __builtin_popcountll(minB);
    a->rankA = fixed_hamming_state_to_index(a->minA);
    a->nA = fixed_hamming_state_to_index(a->maxA) - a->rankA + 1;
    a->rankB = fixed_hamming_state_to_index(minB);
    const int64_t nB = fixed_hamming_state_to_index(maxB) - a->rankB + 1;
    a->n_candidates = a->nA * nB;
    a->reference_rule = 0;  // no floating rule for fermionic signs: exact stabiliser rule
  } else {
    a->spinful = 0;
    a->h = req.hamming_fixed ? __builtin_popcountll(req.lower) : -1;
    if (a->h >= 0) {
      a->first_rank = fixed_hamming_state_to_index(req.lower);
      a->n_candidates = fixed_hamming_state_to_index(req.upper) - a->first_rank + 1;
    } else {
      a->first_rank = (int64_t)req.lower;
      a->n_candidates = (int64_t)(req.upper - req.lower) + 1;
    }
  }
  a->n_tiles = (a->n_candidates + kEnumTile - 1) / kEnumTile;
}

template <int DEPTH>
__global__ void __launch_bounds__(kEnumThreads) k_enumerate_projected(DeviceGroup g, EnumArgs a) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t total;
  __shared__ unsigned long long base_slot;
  for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
    const int64_t first = tile * kEnumTile + (int64_t)threadIdx.x * kEnumPerThread;
    uint32_t bits = 0;
    int cnt = 0;
    if (first < a.n_candidates) {
      uint64_t v = candidate_at(a, first);
      const int todo = (int)min((int64_t)kEnumPerThread, a.n_candidates - first);
      for (int k = 0; k < todo; ++k) {
        IsRepResult r = is_rep<DEPTH>(g, v, a.lane_width, true);
        bool keep;
        if (!r.ok) {
          keep = false;
        } else if (a.reference_rule) {
          keep = r.sum > 0;
        } else {
          keep = r.trivial && r.exact_count > 0;
        }
        if (keep) {
          bits |= 1u << k;
          ++cnt;
        }
        if (k + 1 < todo) v = candidate_next(a, v);
      }
    }
    const int64_t excl = block_exclusive_scan((int64_t)cnt, warp_sums, &total);
    if (threadIdx.x == 0) {
      unsigned long long b = 0;
      if (total > 0) b = atomicAdd(a.counter, (unsigned long long)total);
      base_slot = b;
      a.tile_count[tile] = (int32_t)total;
      a.tile_start[tile] = (int64_t)b;
    }
    __syncthreads();
    if (cnt > 0) {
      int64_t pos = (int64_t)base_slot + excl;
      uint64_t v = candidate_at(a, first);
      for (int k = 0; bits != 0; ++k) {
        if (bits & 1u) {
          if (pos < a.capacity) a.append[pos] = v;
          ++pos;
        }
        bits >>= 1;
        if (bits) v = candidate_next(a, v);
      }
    }
    __syncthreads();
  }
}

template <int D>
struct RunEnumerate {
  static void run(const DeviceGroup& g, const EnumArgs& a, cudaStream_t s) {
    int64_t blocks = std::min<int64_t>(a.n_tiles, (int64_t)num_sms() * 8);
    if (blocks < 1) blocks = 1;
    k_enumerate_projected<D><<<(unsigned)blocks, kEnumThreads, 0, s>>>(g, a);
  }
};

__global__ void k_gather_runs(int64_t n_tiles, const int32_t* __restrict__ tile_count,
                              const int64_t* __restrict__ tile_start,
                              const int64_t* __restrict__ tile_offset,
                              const uint64_t* __restrict__ append, uint64_t* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_tiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int c = tile_count[t];
    const int64_t src = tile_start[t], dst = tile_offset[t];
    for (int k = 0; k < c; ++k) out[dst + k] = append[src + k];
  }
}

// Unprojected: out[i] = unrank(first_rank + i) (fixed weight) or first + i.
__global__ void k_enumerate_plain(int64_t first_rank, int64_t n, int h, int n_bits,
                                  uint64_t* __restrict__ out) {
  constexpr int K = 16;
  for (int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * K; c < n;
       c += (int64_t)gridDim.x * blockDim.x * K) {
    uint64_t v = h >= 0 ? d_unrank(first_rank + c, h, n_bits) : (uint64_t)(first_rank + c);
    const int todo = (int)min((int64_t)K, n - c);
    for (int k = 0; k < todo; ++k) {
      out[c + k] = v;
      v = h >= 0 ? next_fixed_hamming(v) : v + 1;
    }
  }
}

// Spinful fermions with (N_up, N_down) fixed: out[iB * nA + iA] = (stateB << ns) | stateA.
__global__ void k_enumerate_spinful(int64_t rankA, int64_t nA, int hA, int64_t rankB, int64_t nB,
                                    int hB, int ns, uint64_t* __restrict__ out) {
  constexpr int K = 16;
  const int64_t chunksA = (nA + K - 1) / K;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < chunksA * nB;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t iB = w / chunksA, cA = (w % chunksA) * K;
    const uint64_t b = d_unrank(rankB + iB, hB, ns) << ns;
    uint64_t v = d_unrank(rankA + cA, hA, ns);
    const int todo = (int)min((int64_t)K, nA - cA);
    for (int k = 0; k < todo; ++k) {
      out[iB * nA + cA + k] = b | v;
      v = next_fixed_hamming(v);
    }
  }
}

int enumerate_states(const DeviceGroup* g0, const EnumerateRequest& req, uint64_t** d_out,
                     int64_t* count, cudaStream_t s) {
  *d_out = nullptr;
  *count = 0;
  if (ensure_binomials() != 0) return LS_GPU_ERR_CUDA;
  const int n_bits = (req.mode == 2 || req.mode == 3) ? 2 * req.number_sites : req.number_sites;
  if (req.lower > req.upper) return 0;
  if (req.mode == 1) {
    uint64_t low = req.lower, high = req.upper;
    if (req.spin_inversion != 0) {
      const uint64_t mask = req.number_sites == 0 ? 0 : (~(uint64_t)0) >> (64 - req.number_sites);
      if ((high ^ mask) < high) high ^= mask;
    }
    if (low > high) return 0;
    int64_t r0, r1;
    int h = -1;
    if (req.hamming_fixed) {
      h = __builtin_popcountll(low);
      r0 = fixed_hamming_state_to_index(low);
      r1 = fixed_hamming_state_to_index(high);
    } else {
      r0 = (int64_t)low;
      r1 = (int64_t)high;
    }
    const int64_t n = r1 - r0 + 1;
    uint64_t* out = nullptr;
    if (!cuda_ok(cudaMalloc((void**)&out, std::max<int64_t>(n, 1) * 8), "cudaMalloc(states)"))
      return LS_GPU_ERR_CUDA;
    {
      StageScope stage("basis.enumerate", s);
      k_enumerate_plain<<<grid_for((n + 15) / 16, 256), 256, 0, s>>>(r0, n, h, n_bits, out);
    }
    if (!cuda_ok(cudaGetLastError(), "k_enumerate_plain")) {
      cudaFree(out);
      return LS_GPU_ERR_CUDA;
    }
    *d_out = out;
    *count = n;
    return 0;
  }
  if (req.mode == 2) {
    const int ns = req.number_sites;
    const uint64_t mask = ns == 0 ? 0 : (~(uint64_t)0) >> (64 - ns);
    const uint64_t minA = req.lower & mask, maxA = req.upper & mask;
    const uint64_t minB = (req.lower >> ns) & mask, maxB = (req.upper >> ns) & mask;
    const int hA = __builtin_popcountll(minA), hB = __builtin_popcountll(minB);
    const int64_t rA = fixed_hamming_state_to_index(minA);
    const int64_t nA = fixed_hamming_state_to_index(maxA) - rA + 1;
    const int64_t rB = fixed_hamming_state_to_index(minB);
    const int64_t nB = fixed_hamming_state_to_index(maxB) - rB + 1;
    const int64_t n = nA * nB;
    uint64_t* out = nullptr;
    if (!cuda_ok(cudaMalloc((void**)&out, std::max<int64_t>(n, 1) * 8), "cudaMalloc(states)"))
      return LS_GPU_ERR_CUDA;
    {
      StageScope stage("basis.enumerate", s);
      k_enumerate_spinful<<<grid_for(n / 16 + 1, 256), 256, 0, s>>>(rA, nA, hA, rB, nB, hB, ns, out);
    }
    if (!cuda_ok(cudaGetLastError(), "k_enumerate_spinful")) {
      cudaFree(out);
      return LS_GPU_ERR_CUDA;
    }
    *d_out = out;
    *count = n;
    return 0;
  }
  // Projected spin basis.
  if (g0 == nullptr || g0->n_elems == 0) return fail(LS_GPU_ERR_INVALID, "projected enumeration without a group");
  DeviceGroup g = strip(*g0);
  EnumArgs a{};
  projected_candidates(req, n_bits, &a);
  // Capacity guess: candidates / |G| * 2 + slack; retried with the exact count on overflow.
  int64_t capacity = std::min<int64_t>(a.n_candidates,
                                       a.n_candidates / std::max(1, g.n_elems) * 2 + 1024 * 1024);
  int32_t* tile_count = nullptr;
  int64_t* tile_start = nullptr;
  int64_t* tile_offset = nullptr;
  unsigned long long* counter = nullptr;
  uint64_t* append = nullptr;
  auto cleanup = [&]() {
    cudaFree(tile_count);
    cudaFree(tile_start);
    cudaFree(tile_offset);
    cudaFree(counter);
    cudaFree(append);
  };
  if (!cuda_ok(cudaMalloc((void**)&tile_count, a.n_tiles * 4), "alloc") ||
      !cuda_ok(cudaMalloc((void**)&tile_start, a.n_tiles * 8), "alloc") ||
      !cuda_ok(cudaMalloc((void**)&tile_offset, (a.n_tiles + 1) * 8), "alloc") ||
      !cuda_ok(cudaMalloc((void**)&counter, 8), "alloc")) {
    cleanup();
    return LS_GPU_ERR_CUDA;
  }
  unsigned long long total = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if (!cuda_ok(cudaMalloc((void**)&append, std::max<int64_t>(capacity, 1) * 8), "alloc append")) {
      cleanup();
      return LS_GPU_ERR_CUDA;
    }
    a.tile_count = tile_count;
    a.tile_start = tile_start;
    a.append = append;
    a.capacity = capacity;
    a.counter = counter;
    cudaMemsetAsync(counter, 0, 8, s);
    {
      StageScope stage("basis.enumerate", s);
      dispatch_depth<RunEnumerate>(g.depth, group_is_standard(*g0), g, a, s);
    }
    if (!cuda_ok(cudaGetLastError(), "k_enumerate_projected") ||
        !cuda_ok(cudaMemcpyAsync(&total, counter, 8, cudaMemcpyDeviceToHost, s), "read count") ||
        !cuda_ok(cudaStreamSynchronize(s), "enumerate")) {
      cleanup();
      return LS_GPU_ERR_CUDA;
    }
    if ((int64_t)total <= capacity) break;
    cudaFree(append);
    append = nullptr;
    capacity = (int64_t)total;
  }
  uint64_t* out = nullptr;
  if (!cuda_ok(cudaMalloc((void**)&out, std::max<unsigned long long>(total, 1) * 8), "alloc out")) {
    cleanup();
    return LS_GPU_ERR_CUDA;
  }
  int rc = 0;
  {
    StageScope stage("basis.enumerate_compact", s);
    rc = exclusive_scan<int32_t>(tile_count, a.n_tiles, tile_offset, s);
    if (rc == 0)
      k_gather_runs<<<grid_for(a.n_tiles, 256), 256, 0, s>>>(a.n_tiles, tile_count, tile_start,
                                                            tile_offset, append, out);
  }
  if (rc == 0) {
    if (!cuda_ok(cudaGetLastError(), "k_gather_runs") || !cuda_ok(cudaStreamSynchronize(s), "gather"))
      rc = LS_GPU_ERR_CUDA;
  }
  cleanup();
  if (rc != 0) {
    cudaFree(out);
    return rc;
  }
  *d_out = out;
  *count = (int64_t)total;
  return 0;
}

// ------------------------------------------------------------------------------------------------
// Prefix-bucket index (indexing.c:45-117 semantics, built on the device)
// ------------------------------------------------------------------------------------------------
__global__ void k_bucket_offsets(const uint64_t* __restrict__ reps, int64_t n, int shift,
                                 int64_t n_buckets, uint32_t* __restrict__ offsets) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b <= n_buckets;
       b += (int64_t)gridDim.x * blockDim.x) {
    if (b == n_buckets) {
      offsets[b] = (uint32_t)n;
      continue;
    }
    // first k with (reps[k] >> shift) >= b
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((reps[mid] >> shift) < (uint64_t)b) lo = mid + 1; else hi = mid;
    }
    offsets[b] = (uint32_t)lo;
  }
}

__global__ void k_bucket_max(const uint32_t* __restrict__ offsets, int64_t n_buckets,
                             unsigned long long* __restrict__ out) {
  unsigned long long m = 0;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < n_buckets;
       b += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long r = (unsigned long long)(offsets[b + 1] - offsets[b]);
    m = r > m ? r : m;
  }
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_down_sync(0xffffffffu, m, d);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// suffix[i] = the low `shift` bits of reps[i] (shift <= 16).
__global__ void k_key_suffixes(const uint64_t* __restrict__ reps, int64_t n, int shift, uint16_t* __restrict__ suffix) {
  const uint64_t mask = (1ull << shift) - 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    suffix[i] = (uint16_t)(reps[i] & mask);
}

// The reference buckets on the top prefix_bits of number_bits (indexing.c:94-117).  Sorted
// representatives are orbit minima and crowd towards small values, so here the buckets cover the
// bits actually used (up to the largest representative) and their count grows with the basis
// (about one state per bucket) up to 2^24 buckets of 32-bit starts (a 64 MB table, most of which
// stays in L2 while the matvec probes it once per generated element).  The answers are the same
// indices.
int build_prefix_index(const uint64_t* d_reps, int64_t n, int number_bits, int prefix_bits,
                       uint32_t** d_offsets, int64_t* range_size, int* shift, cudaStream_t s,
                       uint64_t* max_state, uint16_t** d_suffix) {
  if (n >= ((int64_t)1 << 32)) return fail(LS_GPU_ERR_INVALID, "more than 2^32 representatives");
  StageScope stage("basis.index", s);
  uint64_t max_rep = 0;
  if (n > 0 && !cuda_ok(cudaMemcpyAsync(&max_rep, d_reps + (n - 1), 8, cudaMemcpyDeviceToHost, s), "read max") )
    return LS_GPU_ERR_CUDA;
  if (!cuda_ok(cudaStreamSynchronize(s), "read max")) return LS_GPU_ERR_CUDA;
  *max_state = n > 0 ? max_rep : 0;
  const int used_bits = max_rep == 0 ? 1 : 64 - __builtin_clzll(max_rep);
  int want = 1;
  while (want < 24 && ((int64_t)1 << want) < n) ++want;
  int p = std::max(std::min(prefix_bits, number_bits), want);
  p = std::min(p, std::min(used_bits, 24));
  if (p < 0) p = 0;
  *shift = used_bits - p;
  const int64_t nb = (int64_t)1 << p;
  uint32_t* off = nullptr;
  unsigned long long* mx = nullptr;
  if (!cuda_ok(cudaMalloc((void**)&off, (nb + 1) * 4), "alloc offsets") ||
      !cuda_ok(cudaMalloc((void**)&mx, 8), "alloc")) {
    cudaFree(off);
    return LS_GPU_ERR_CUDA;
  }
  cudaMemsetAsync(mx, 0, 8, s);
  k_bucket_offsets<<<grid_for(nb + 1, 256), 256, 0, s>>>(d_reps, n, *shift, nb, off);
  k_bucket_max<<<grid_for(nb, 256), 256, 0, s>>>(off, nb, mx);
  unsigned long long r = 0;
  if (!cuda_ok(cudaGetLastError(), "bucket kernels") ||
      !cuda_ok(cudaMemcpyAsync(&r, mx, 8, cudaMemcpyDeviceToHost, s), "read range") ||
      !cuda_ok(cudaStreamSynchronize(s), "bucket sync")) {
    cudaFree(off);
    cudaFree(mx);
    return LS_GPU_ERR_CUDA;
  }
  cudaFree(mx);
  uint16_t* suf = nullptr;
  if (*shift <= 16 && n > 0) {
    if (!cuda_ok(cudaMalloc((void**)&suf, (size_t)n * 2), "alloc suffixes")) {
      cudaFree(off);
      return LS_GPU_ERR_CUDA;
    }
    k_key_suffixes<<<grid_for(n, 256), 256, 0, s>>>(d_reps, n, *shift, suf);
    if (!cuda_ok(cudaGetLastError(), "k_key_suffixes")) {
      cudaFree(off);
      cudaFree(suf);
      return LS_GPU_ERR_CUDA;
    }
  }
  *d_offsets = off;
  *d_suffix = suf;
  *range_size = (int64_t)r;
  return 0;
}

__device__ __forceinline__ int64_t index_lookup(const DeviceIndex& ix, uint64_t needle) {
  if (ix.identity) return (int64_t)needle;
  if (ix.combinadic) return d_rank(needle) - ix.rank_base;
  int64_t len = ix.range_size;
  if (len <= 0 || needle > ix.max_state) return -1;
  const uint64_t b = needle >> ix.shift;
  if (ix.suffix16 != nullptr) {
    // binary search of the needle's bucket [start, end) in its 2-byte suffixes
    const uint16_t target = (uint16_t)(needle & ((1ull << ix.shift) - 1));
    int64_t base = __ldg(ix.offsets + b);
    const int64_t end = __ldg(ix.offsets + b + 1);
    int64_t n = end - base;
    if (n <= 0) return -1;
    while (n > 1) {
      const int64_t half = n >> 1;
      base = (__ldg(ix.suffix16 + base + half) <= target) ? base + half : base;
      n -= half;
    }
    return __ldg(ix.suffix16 + base) == target ? base : -1;
  }
  // a window of the largest bucket's length starting at the bucket, moved back to end at n
  int64_t base = min((int64_t)__ldg(ix.offsets + b), ix.n_states - len);
  while (len > 1) {
    const int64_t half = len >> 1;
    base = (__ldg(ix.reps + base + half) < needle) ? base + half : base;
    len -= half;
  }
  if (base < ix.n_states && __ldg(ix.reps + base) < needle) ++base;
  return (base < ix.n_states && __ldg(ix.reps + base) == needle) ? base : -1;
}

__global__ void k_state_index(DeviceIndex ix, int64_t n, const uint64_t* __restrict__ xs,
                              int64_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    out[i] = index_lookup(ix, xs[i]);
  }
}

int launch_state_index(const DeviceIndex& ix, int64_t n, const uint64_t* d_x, int64_t* d_out,
                       cudaStream_t s) {
  if (n <= 0) return 0;
  if (ix.combinadic && ensure_binomials() != 0) return LS_GPU_ERR_CUDA;
  k_state_index<<<grid_for(n, 256), 256, 0, s>>>(ix, n, d_x, d_out);
  return cuda_ok(cudaGetLastError(), "k_state_index") ? 0 : LS_GPU_ERR_CUDA;
}

// ================================================================================================
// Allocation-free enumeration (ls_gpu_enumerate_noalloc).
//
// Some callers cannot allocate device memory: code that runs under a framework owning every
// device allocation (a custom call of an array framework, a pool that reserves all of HBM), or
// code between stream captures where cudaMalloc must not be called.  For them the enumeration runs
// in two passes (count per tile, then write straight into the caller's output at scanned offsets)
// and keeps all of its scratch in g_noalloc_scratch, a file-scope device array of
// kNoallocScratchBytes that every GPU loading the library holds until the process exits:
//   [0, kNoallocGroupBytes)   the basis' group tables, copied from the host on every call
//   [kNoallocGroupBytes, ..)  tile counts (int32), tile offsets (int64), scan block sums (int64)
// Each call overwrites everything it reads, so nothing needs clearing between calls; calls that
// overlap on the GPU (different streams, or another host thread) race on the array.
// ================================================================================================
constexpr size_t kNoallocScratchBytes = 16u << 20;  // 16 MiB per device
constexpr size_t kNoallocGroupBytes = 1u << 20;     // group tables up to 1 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];
static unsigned char* g_noalloc_scratch_addr[64];   // device address of the array, per device

// Set-up, once per device with that device current: the device address of g_noalloc_scratch (its
// name in host code is only a host-side stand-in and must never be passed to a kernel).
static int noalloc_scratch_address(unsigned char** out) {
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return LS_GPU_ERR_CUDA;
  if (dev < 0 || dev >= 64) return fail(LS_GPU_ERR_INVALID, "device ordinal out of range");
  if (g_noalloc_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(g_noalloc_scratch)"))
      return LS_GPU_ERR_CUDA;
    g_noalloc_scratch_addr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_scratch_addr[dev];
  return 0;
}

// SM count of the current device for the grid sizes of this path, read with
// cudaDeviceGetAttribute and kept per device.  The library's shared runtime (stream, error word,
// binomial table) is never touched here: setting it up allocates device memory.
static int noalloc_sms() {
  static int sms[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  if (sms[dev] <= 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
    sms[dev] = n;
  }
  return sms[dev];
}

static int noalloc_grid(int64_t n, int threads) {
  int64_t blocks = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)noalloc_sms() * 32;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

template <int DEPTH>
__device__ inline uint32_t enum_tile_flags(const DeviceGroup& g, const EnumArgs& a, int64_t first, int* cnt) {
  uint32_t bits = 0;
  *cnt = 0;
  if (first < a.n_candidates) {
    uint64_t v = candidate_at(a, first);
    const int todo = (int)min((int64_t)kEnumPerThread, a.n_candidates - first);
    for (int k = 0; k < todo; ++k) {
      IsRepResult r = is_rep<DEPTH>(g, v, a.lane_width, true);
      const bool keep = r.ok && (a.reference_rule ? (r.sum > 0) : (r.trivial && r.exact_count > 0));
      if (keep) {
        bits |= 1u << k;
        ++*cnt;
      }
      if (k + 1 < todo) v = candidate_next(a, v);
    }
  }
  return bits;
}

template <int DEPTH>
__global__ void __launch_bounds__(kEnumThreads) k_enumerate_count(DeviceGroup g, EnumArgs a,
                                                                  int32_t* __restrict__ tile_count) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t total;
  for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
    int cnt = 0;
    enum_tile_flags<DEPTH>(g, a, tile * kEnumTile + (int64_t)threadIdx.x * kEnumPerThread, &cnt);
    block_exclusive_scan((int64_t)cnt, warp_sums, &total);
    if (threadIdx.x == 0) tile_count[tile] = (int32_t)total;
    __syncthreads();
  }
}

template <int DEPTH>
__global__ void __launch_bounds__(kEnumThreads) k_enumerate_write(DeviceGroup g, EnumArgs a,
                                                                  const int64_t* __restrict__ tile_offset,
                                                                  uint64_t* __restrict__ out, int64_t capacity) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t total;
  for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
    const int64_t first = tile * kEnumTile + (int64_t)threadIdx.x * kEnumPerThread;
    int cnt = 0;
    uint32_t bits = enum_tile_flags<DEPTH>(g, a, first, &cnt);
    const int64_t excl = block_exclusive_scan((int64_t)cnt, warp_sums, &total);
    if (cnt > 0) {
      int64_t pos = tile_offset[tile] + excl;
      uint64_t v = candidate_at(a, first);
      while (bits != 0) {
        if (bits & 1u) {
          if (pos < capacity) out[pos] = v;
          ++pos;
        }
        bits >>= 1;
        if (bits) v = candidate_next(a, v);
      }
    }
    __syncthreads();
  }
}

template <int D>
struct RunEnumerateNoalloc {
  static void run(const DeviceGroup& g, const EnumArgs& a, int32_t* counts, const int64_t* offsets,
                  uint64_t* out, int64_t capacity, int pass, cudaStream_t s) {
    int64_t blocks = std::min<int64_t>(a.n_tiles, (int64_t)noalloc_sms() * 8);
    if (blocks < 1) blocks = 1;
    if (pass == 0)
      k_enumerate_count<D><<<(unsigned)blocks, kEnumThreads, 0, s>>>(g, a, counts);
    else
      k_enumerate_write<D><<<(unsigned)blocks, kEnumThreads, 0, s>>>(g, a, offsets, out, capacity);
  }
};

int enumerate_states_noalloc(const OrbitData* od, const EnumerateRequest& req, uint64_t* d_out,
                             int64_t capacity, int64_t* count, cudaStream_t s) {
  *count = 0;
  if (capacity < 0) return fail(LS_GPU_ERR_INVALID, "negative capacity");
  if (d_out == nullptr && capacity > 0) return fail(LS_GPU_ERR_INVALID, "output buffer is NULL");
  if (ensure_binomials() != 0) return LS_GPU_ERR_CUDA;
  const int n_bits = (req.mode == 2 || req.mode == 3) ? 2 * req.number_sites : req.number_sites;
  if (req.lower > req.upper) return 0;
  if (req.mode == 1 || req.mode == 2) {
    // No scratch needed: the states are generated directly from their combinadic ranks.
    int64_t n = 0, r0 = 0, rA = 0, nA = 0, rB = 0, nB = 0;
    int h = -1, hA = 0, hB = 0;
    const int ns = req.number_sites;
    if (req.mode == 1) {
      uint64_t low = req.lower, high = req.upper;
      if (req.spin_inversion != 0) {
        const uint64_t mask = ns == 0 ? 0 : (~(uint64_t)0) >> (64 - ns);
        if ((high ^ mask) < high) high ^= mask;
      }
      if (low > high) return 0;
      if (req.hamming_fixed) {
        h = __builtin_popcountll(low);
        r0 = fixed_hamming_state_to_index(low);
        n = fixed_hamming_state_to_index(high) - r0 + 1;
      } else {
        r0 = (int64_t)low;
        n = (int64_t)(high - low) + 1;
      }
    } else {
      const uint64_t mask = ns == 0 ? 0 : (~(uint64_t)0) >> (64 - ns);
      const uint64_t minA = req.lower & mask, maxA = req.upper & mask;
      const uint64_t minB = (req.lower >> ns) & mask, maxB = (req.upper >> ns) & mask;
      hA = __builtin_popcountll(minA);
      hB = __builtin_popcountll(minB);
      rA = fixed_hamming_state_to_index(minA);
      nA = fixed_hamming_state_to_index(maxA) - rA + 1;
      rB = fixed_hamming_state_to_index(minB);
      nB = fixed_hamming_state_to_index(maxB) - rB + 1;
      n = nA * nB;
    }
    *count = n;
    if (n > capacity) return fail(LS_GPU_ERR_INVALID, "output capacity is smaller than the number of states");
    if (n == 0) return 0;
    if (req.mode == 1)
      k_enumerate_plain<<<noalloc_grid((n + 15) / 16, 256), 256, 0, s>>>(r0, n, h, n_bits, d_out);
    else
      k_enumerate_spinful<<<noalloc_grid(n / 16 + 1, 256), 256, 0, s>>>(rA, nA, hA, rB, nB, hB, ns, d_out);
    if (!cuda_ok(cudaGetLastError(), "enumerate (no allocation)")) return LS_GPU_ERR_CUDA;
    return cuda_ok(cudaStreamSynchronize(s), "enumerate (no allocation)") ? 0 : LS_GPU_ERR_CUDA;
  }
  // Projected spin basis: group tables and tile arrays in the static scratch.
  if (od == nullptr || od->n_elems == 0) return fail(LS_GPU_ERR_INVALID, "projected enumeration without a group");
  unsigned char* base = nullptr;
  int rc = noalloc_scratch_address(&base);
  if (rc != 0) return rc;
  const size_t group_bytes = od->host_block.size();
  if (group_bytes > kNoallocGroupBytes)
    return fail(LS_GPU_ERR_INVALID, "symmetry group tables exceed the 1 MiB reserved for them");
  EnumArgs a{};
  projected_candidates(req, n_bits, &a);
  // tile counts | tile offsets (n + 1) | block sums | scanned block sums (+ total)
  const int64_t max_tiles =
      (int64_t)((kNoallocScratchBytes - kNoallocGroupBytes - 4 * 65536) / (4 + 8)) - 1;
  if (a.n_tiles > max_tiles)
    return fail(LS_GPU_ERR_INVALID, "basis too large for the allocation-free enumeration (more than " +
                                        std::to_string(max_tiles * kEnumTile) + " candidate states)");
  const int64_t n_blocks2 = (a.n_tiles + kScanTile - 1) / kScanTile;
  if (n_blocks2 > kScanTile) return fail(LS_GPU_ERR_INVALID, "scan too large");
  unsigned char* p = base + kNoallocGroupBytes;
  int32_t* counts = (int32_t*)p;
  p += ((size_t)a.n_tiles * 4 + 255) & ~(size_t)255;
  int64_t* offsets = (int64_t*)p;
  p += ((size_t)(a.n_tiles + 1) * 8 + 255) & ~(size_t)255;
  int64_t* sums = (int64_t*)p;
  p += ((size_t)(n_blocks2 + 1) * 8 + 255) & ~(size_t)255;
  int64_t* sums_scan = (int64_t*)p;

  // group view into the scratch (same layout as the orbit data block)
  if (!cuda_ok(cudaMemcpyAsync(base, od->host_block.data(), group_bytes, cudaMemcpyHostToDevice, s),
               "copy group tables"))
    return LS_GPU_ERR_CUDA;
  DeviceGroup g;
  g.n_bits = od->n_bits;
  g.n_elems = od->n_elems;
  g.depth = od->depth;
  g.spin_inversion = od->spin_inversion;
  g.flip = od->n_bits == 0 ? 0 : (~(uint64_t)0) >> (64 - od->n_bits);
  g.masks_t = (const uint64_t*)(base + od->off_masks);
  g.shifts = (const uint32_t*)(base + od->off_shifts);
  g.chars = (const double2*)(base + od->off_chars);
  g.onehot = (const uint64_t*)(base + od->off_onehot);
  g.prio = (const uint16_t*)(base + od->off_prio);
  g.fermionic = od->fermionic;
  g.fsign = od->fermionic ? (const uint64_t*)(base + od->off_fsign) : nullptr;

  dispatch_depth<RunEnumerateNoalloc>(g.depth, od->standard_shifts, g, a, counts, offsets, d_out, capacity, 0, s);
  if (!cuda_ok(cudaGetLastError(), "k_enumerate_count")) return LS_GPU_ERR_CUDA;
  // exclusive scan of the tile counts: per 4096-tile block, then over the block sums
  k_scan_tiles<int32_t><<<(unsigned)n_blocks2, kScanThreads, 0, s>>>(counts, a.n_tiles, offsets, sums);
  k_scan_tiles<int64_t><<<1, kScanThreads, 0, s>>>(sums, n_blocks2, sums_scan, sums_scan + n_blocks2);
  k_scan_add<<<(unsigned)n_blocks2, kScanThreads, 0, s>>>(offsets, a.n_tiles, sums_scan);
  if (!cuda_ok(cudaMemcpyAsync(offsets + a.n_tiles, sums_scan + n_blocks2, 8, cudaMemcpyDeviceToDevice, s),
               "scan total"))
    return LS_GPU_ERR_CUDA;
  int64_t total = 0;
  if (!cuda_ok(cudaMemcpyAsync(&total, offsets + a.n_tiles, 8, cudaMemcpyDeviceToHost, s), "read count") ||
      !cuda_ok(cudaStreamSynchronize(s), "count pass"))
    return LS_GPU_ERR_CUDA;
  *count = total;
  if (total > capacity) return fail(LS_GPU_ERR_INVALID, "output capacity is smaller than the number of states");
  dispatch_depth<RunEnumerateNoalloc>(g.depth, od->standard_shifts, g, a, counts, offsets, d_out, capacity, 1, s);
  if (!cuda_ok(cudaGetLastError(), "k_enumerate_write")) return LS_GPU_ERR_CUDA;
  return cuda_ok(cudaStreamSynchronize(s), "write pass") ? 0 : LS_GPU_ERR_CUDA;
}

}  // namespace lsg
