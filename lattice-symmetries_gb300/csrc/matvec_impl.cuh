// matvec_impl.cuh -- gather-form H*x kernels (included by the matvec_*.cu translation units,
// each of which instantiates a subset so that the build compiles in parallel).
//
// The reference computes y = H x by scattering: every representative alpha_j generates
// beta = alpha_j ^ x_t, projects it onto its representative and adds
// chi * v * sign * x_j * n(beta)/n(alpha_j) to y[index(rep(beta))] with atomics
// (chapel/src/BatchedOperator.chpl:207-253, DistributedMatrixVector.chpl:91-143).
//
// Here every output row gathers instead.  For a row state a = alpha_i and a term t with
// (a & m_t) == l_t, the column state is beta = a ^ x_t and
//
//     H[i, j] += v_t (-1)^popcount(beta & s_t) conj(chi(g)) n_j / n_i,   alpha_j = g.beta,
//
// the same matrix element the reference produces from column j (it is <alpha_i-bar|H|alpha_j-bar>
// in the orthonormal symmetrised basis).  No atomics, deterministic summation order.  H^dagger
// uses the same kernels with the adjoint term table.
//
// Projected bases: one warp per row.  Lane L owns group elements e = L + 32k (k < GPL) and keeps
// g.a in registers; because permuting bits is linear over XOR, g.beta = g.a ^ g.x_t, and g.x_t
// is an XOR of one-hot site images (a shared-memory table [bit][element]).  The warp reduces the
// candidates (and their spin-flipped partners) to the representative with three REDUX.MIN
// steps, and every 32 targets the lanes look up indices and gather x in parallel.
#pragma once

#include "lsg.h"
#include "pairs.cuh"

namespace lsg {

__device__ __forceinline__ bool constraint_ok(const DeviceConstraint& c, uint64_t s) {
  if (c.kind == 0) return true;
  if (c.kind == 1) return __popcll(s) == c.w0;
  const uint64_t lo = s & ((c.half_bits >= 64) ? ~0ull : ((1ull << c.half_bits) - 1));
  return __popcll(lo) == c.w0 && __popcll(s >> c.half_bits) == c.w1;
}

// Index lookup (duplicated from basis.cu as a header-local function so that each matvec
// translation unit inlines it).
__device__ __forceinline__ int64_t mv_index_lookup(const DeviceIndex& ix, uint64_t needle,
                                                   const uint64_t* __restrict__ binom /*65x65*/) {
  if (ix.identity) return (int64_t)needle;
  if (ix.combinadic) {
    int64_t i = 0;
    uint64_t a = needle;
    for (int k = 1; a != 0; ++k) {
      const int c = __ffsll((long long)a) - 1;
      a &= a - 1;
      i += (c <= 0 || k > c) ? 0 : (int64_t)__ldg(binom + c * 65 + k);
    }
    return i - ix.rank_base;
  }
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

// Re-reads an index descriptor that lives in shared memory (the batched kernel's sector table)
// through volatile loads, so that the compiler reads it where the lookup needs it instead of
// holding its fields in registers for the whole row.
__device__ __forceinline__ DeviceIndex reload_index(const DeviceIndex* p) {
  const volatile DeviceIndex* v = p;
  DeviceIndex r;
  r.n_states = v->n_states;
  r.reps = v->reps;
  r.norms = v->norms;
  r.inv_norms = v->inv_norms;
  r.offsets = v->offsets;
  r.suffix16 = v->suffix16;
  r.shift = v->shift;
  r.range_size = v->range_size;
  r.prefix_bits = v->prefix_bits;
  r.max_state = v->max_state;
  r.identity = v->identity;
  r.combinadic = v->combinadic;
  r.rank_base = v->rank_base;
  return r;
}

struct C2 {
  double re, im;
};
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ C2 cmul_conj_b(C2 a, C2 b) {  // a * conj(b)
  return {a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im};
}

// Shared-memory layout of the projected kernel.
struct SmemLayout {
  int onehot_in_smem;
  size_t off_onehot, off_chars, off_tm, off_tl, off_tx, off_ts, off_tv, off_dm, off_dr, off_ds, off_dv;
  size_t total;
};

inline SmemLayout make_layout(const MatvecProblem& p, bool with_group) {
  SmemLayout L{};
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t o = 0;
  const int G = with_group ? p.group.n_elems : 0;
  const size_t onehot_bytes = with_group ? (size_t)p.group.n_bits * G * 8 : 0;
  L.off_chars = o; o = al(o + (size_t)G * 16);
  L.off_tm = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tl = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tx = o; o = al(o + (size_t)p.off.n * 8);
  L.off_ts = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tv = o; o = al(o + (size_t)p.off.n * 16);
  L.off_dm = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_dr = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_ds = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_dv = o; o = al(o + (size_t)p.diag.n * 16);
  // One-hot table last; kept in shared memory when the whole layout stays under 112 KB
  // (two CTAs per SM), otherwise read through L1 from global memory.
  L.off_onehot = o;
  if (with_group && o + onehot_bytes <= 112 * 1024) {
    L.onehot_in_smem = 1;
    o = al(o + onehot_bytes);
  } else {
    L.onehot_in_smem = 0;
  }
  L.total = o;
  return L;
}

__device__ __forceinline__ void stage_u64(uint64_t* dst, const uint64_t* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}
__device__ __forceinline__ void stage_d2(double2* dst, const double2* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

struct Staged {
  const uint64_t* onehot;
  const double2* chars;
  const uint64_t *tm, *tl, *tx, *ts;
  const double2* tv;
  const uint64_t *dm, *dr, *ds;
  const double2* dv;
};

__device__ __forceinline__ Staged stage_problem(const MatvecProblem& p, const SmemLayout& L,
                                                unsigned char* smem, bool with_group) {
  Staged S;
  uint64_t* tm = (uint64_t*)(smem + L.off_tm);
  uint64_t* tl = (uint64_t*)(smem + L.off_tl);
  uint64_t* tx = (uint64_t*)(smem + L.off_tx);
  uint64_t* ts = (uint64_t*)(smem + L.off_ts);
  double2* tv = (double2*)(smem + L.off_tv);
  uint64_t* dm = (uint64_t*)(smem + L.off_dm);
  uint64_t* dr = (uint64_t*)(smem + L.off_dr);
  uint64_t* ds = (uint64_t*)(smem + L.off_ds);
  double2* dv = (double2*)(smem + L.off_dv);
  stage_u64(tm, p.off.m, p.off.n);
  stage_u64(tl, p.off.l, p.off.n);
  stage_u64(tx, p.off.x, p.off.n);
  stage_u64(ts, p.off.s, p.off.n);
  stage_d2(tv, p.off.v, p.off.n);
  stage_u64(dm, p.diag.m, p.diag.n);
  stage_u64(dr, p.diag.r, p.diag.n);
  stage_u64(ds, p.diag.s, p.diag.n);
  stage_d2(dv, p.diag.v, p.diag.n);
  S.tm = tm; S.tl = tl; S.tx = tx; S.ts = ts; S.tv = tv;
  S.dm = dm; S.dr = dr; S.ds = ds; S.dv = dv;
  if (with_group) {
    double2* ch = (double2*)(smem + L.off_chars);
    stage_d2(ch, p.group.chars, p.group.n_elems);
    S.chars = ch;
    if (L.onehot_in_smem) {
      uint64_t* oh = (uint64_t*)(smem + L.off_onehot);
      stage_u64(oh, p.group.onehot, p.group.n_bits * p.group.n_elems);
      S.onehot = oh;
    } else {
      S.onehot = p.group.onehot;
    }
  } else {
    S.chars = nullptr;
    S.onehot = nullptr;
  }
  __syncthreads();
  return S;
}

struct Acc {
  double re = 0.0, im = 0.0;  // the real kernels use re only
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

// ------------------------------------------------------------------------------------------------
// Projected kernel: K right-hand sides (K in {1, 4, 8, 16}), GPL group elements per lane.
// x, y: row-major [rows][ld] of double (real) or double2 (complex, CPLX).
// ------------------------------------------------------------------------------------------------
template <int GPL, bool INV, bool CPLX, int K>
__global__ void __launch_bounds__(256, 2)
    k_matvec_projected(const MatvecProblem p, const SmemLayout L, const double* __restrict__ x,
                       int64_t ldx, double* __restrict__ y, int64_t ldy, int* __restrict__ err,
                       const uint64_t* __restrict__ binom) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Staged S = stage_problem(p, L, smem, true);
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int Q = 32 / K;  // slots handled per flush round
  const int lane = threadIdx.x & 31;
  const int G = p.group.n_elems;
  const int nbits = p.group.n_bits;
  const uint64_t flip = p.group.flip;
  const int rhs = lane % K;   // my right-hand side in the flush
  const int q = lane / K;     // my slot offset in a flush round
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;

  int eidx[GPL];
  bool evalid[GPL];
#pragma unroll
  for (int k = 0; k < GPL; ++k) {
    const int e = lane + 32 * k;
    evalid[k] = e < G;
    eidx[k] = evalid[k] ? e : (G - 1);
  }

  for (int64_t row = warp_id; row < p.n_rows; row += n_warps) {
    const uint64_t a = __ldg(p.index.reps + row);
    const double inv_na = __ldg(p.index.inv_norms + row);
    if (inv_na == 0.0) {  // zero-norm representative: zero row and column (see packed_row)
      if (lane < K) {
        if constexpr (CPLX) reinterpret_cast<double2*>(y)[row * ldy + lane] = make_double2(0.0, 0.0);
        else y[row * ldy + lane] = 0.0;
      }
      continue;
    }

    // g.a for my elements
    uint64_t ga[GPL];
#pragma unroll
    for (int k = 0; k < GPL; ++k) ga[k] = 0;
    for (uint64_t bits = a; bits != 0; bits &= bits - 1) {
      const uint64_t* oh = S.onehot + (int64_t)(__ffsll((long long)bits) - 1) * G;
#pragma unroll
      for (int k = 0; k < GPL; ++k) ga[k] ^= oh[eidx[k]];
    }

    // diagonal: lanes split the terms, warp sum
    double dre = 0.0, dim = 0.0;
    for (int t = lane; t < p.diag.n; t += 32) {
      if ((a & S.dm[t]) == S.dr[t]) {
        const double2 v = S.dv[t];
        const bool neg = __popcll(a & S.ds[t]) & 1;
        dre += neg ? -v.x : v.x;
        if constexpr (CPLX) dim += neg ? -v.y : v.y;
      }
    }
    dre = warp_sum(dre);
    if constexpr (CPLX) dim = warp_sum(dim);

    Acc acc;
    unsigned found = 0;  // off-diagonal elements located by this lane (row total via warp sum)
    uint64_t my_rep = ~0ull;
    uint32_t my_idx = 0;
    double2 my_c = make_double2(0.0, 0.0);
    int nslot = 0;

    auto flush = [&]() {
      // every lane with a slot: index, character, norm ratio -> complex factor
      int64_t j = -1;
      double fre = 0.0, fim = 0.0;
      if (lane < nslot) {
        j = mv_index_lookup(p.index, my_rep, binom);
        const double nj = j >= 0 ? __ldg(p.index.norms + j) : 0.0;
        if (nj == 0.0) j = -1;  // zero-norm column
        found += (j >= 0);
        if (j >= 0) {
          double2 chi = S.chars[my_idx >> 1];
          if (INV && (my_idx & 1) && p.group.spin_inversion == -1) chi = make_double2(-chi.x, -chi.y);
          const double ratio = nj * inv_na;
          const C2 f = cmul_conj_b(C2{my_c.x, my_c.y}, C2{chi.x, chi.y});
          fre = f.re * ratio;
          fim = f.im * ratio;
        }
      }
      for (int s0 = 0; s0 < nslot; s0 += Q) {
        const int s = s0 + q;
        const int src = s & 31;
        const int64_t js = (K == 1) ? j : __shfl_sync(FULL, j, src);
        const double sre = (K == 1) ? fre : __shfl_sync(FULL, fre, src);
        const double sim = (K == 1) ? fim : __shfl_sync(FULL, fim, src);
        if (s < nslot && js >= 0) {
          if constexpr (CPLX) {
            const double2 xv = __ldg(reinterpret_cast<const double2*>(x) + js * ldx + rhs);
            acc.re += sre * xv.x - sim * xv.y;
            acc.im += sre * xv.y + sim * xv.x;
          } else {
            const double xv = __ldg(x + js * ldx + rhs);
            acc.re += sre * xv;
          }
        }
        if (K == 1) break;
      }
    };

    for (int t = 0; t < p.off.n; ++t) {
      if ((a & S.tm[t]) != S.tl[t]) continue;
      const uint64_t xt = S.tx[t];
      const uint64_t beta = a ^ xt;
      if (!constraint_ok(p.constraint, beta)) {
        if (lane == 0) atomicOr(err, 1);
        continue;
      }
      double2 c = S.tv[t];
      if (__popcll(beta & S.ts[t]) & 1) c = make_double2(-c.x, -c.y);

      uint64_t gx[GPL];
#pragma unroll
      for (int k = 0; k < GPL; ++k) gx[k] = ga[k];
      for (uint64_t bits = xt; bits != 0; bits &= bits - 1) {
        const uint64_t* oh = S.onehot + (int64_t)(__ffsll((long long)bits) - 1) * G;
#pragma unroll
        for (int k = 0; k < GPL; ++k) gx[k] ^= oh[eidx[k]];
      }
      uint64_t best = ~0ull;
      uint32_t bidx = 0xffffffffu;
#pragma unroll
      for (int k = 0; k < GPL; ++k) {
        uint64_t cand = gx[k];
        uint32_t id = 2u * (uint32_t)(lane + 32 * k);
        if (INV) {
          const uint64_t top = (cand >> (nbits - 1)) & 1ull;
          cand ^= flip & (0ull - top);
          id += (uint32_t)top;
        }
        if (evalid[k] && cand < best) {
          best = cand;
          bidx = id;
        }
      }
      const uint32_t hi = (uint32_t)(best >> 32), lo = (uint32_t)best;
      const uint32_t mhi = __reduce_min_sync(FULL, hi);
      const uint32_t mlo = __reduce_min_sync(FULL, hi == mhi ? lo : 0xffffffffu);
      const uint32_t midx = __reduce_min_sync(FULL, (hi == mhi && lo == mlo) ? bidx : 0xffffffffu);
      if (lane == nslot) {
        my_rep = ((uint64_t)mhi << 32) | mlo;
        my_idx = midx;
        my_c = c;
      }
      if (++nslot == 32) {
        flush();
        nslot = 0;
      }
    }
    if (nslot > 0) flush();
    if (p.nnz_counter != nullptr) {
      const unsigned total = __reduce_add_sync(FULL, found);
      if (lane == 0 && total) atomicAdd(p.nnz_counter, (unsigned long long)total);
    }

    // reduce lanes holding the same right-hand side, add the diagonal, store
    if constexpr (CPLX) {
#pragma unroll
      for (int d = 16; d >= K; d >>= 1) {
        acc.re += __shfl_xor_sync(FULL, acc.re, d);
        acc.im += __shfl_xor_sync(FULL, acc.im, d);
      }
      if (lane < K) {
        const double2 xi = __ldg(reinterpret_cast<const double2*>(x) + row * ldx + lane);
        double2 out;
        out.x = acc.re + (dre * xi.x - dim * xi.y);
        out.y = acc.im + (dre * xi.y + dim * xi.x);
        reinterpret_cast<double2*>(y)[row * ldy + lane] = out;
      }
    } else {
#pragma unroll
      for (int d = 16; d >= K; d >>= 1) acc.re += __shfl_xor_sync(FULL, acc.re, d);
      if (lane < K) y[row * ldy + lane] = acc.re + dre * __ldg(x + row * ldx + lane);
    }
  }
}

// ------------------------------------------------------------------------------------------------
// Packed projected kernel (default for projected bases).
//
// Same gather as k_matvec_projected, with a cheaper orbit scan:
//  * the site-image table is pre-shifted to the top bits and padded to GPL*32 slots, and the low
//    bits of every lane's g.a carry the candidate index 2*slot, so the minimum of the 64-bit keys
//    gives the representative and its group element together, and the spin flip is a sign-mask
//    XOR that also sets the flip bit of the index;
//  * the minimum is found in two passes (scan_two_site): the high 32 bits of every candidate
//    first (one three-input XOR and a min -- with spin inversion also a max -- per slot), then the
//    exact 64-bit keys of the few candidates whose high word ties the warp minimum;
//  * the terms matching the row are found with one ballot per 32 terms.
// The row sum is divided by n_i once at the end.
//
// Site images in shared memory are kept as lane records: slot j of lane L (group element
// e = L + 32 j) of site r is stored as its (lo, hi) 32-bit words at
// rec[(r * 32 + L) * S + 2 j + {0, 1}].  For more than 4 slots S = 2 GPL + 1 is odd, so the 32
// lanes reading one 32-bit word of their own records hit 32 distinct banks, and lanes j < GPL
// reading the slots of one lane's record read consecutive words.  Each warp also keeps the images
// of its current row state (g.a, with the candidate index in the low bits) in a record area of the
// same layout.  Up to 4 slots the scan is a plain 64-bit minimum (RowScan below) and S is even
// with S / 2 odd, so that slots load as 8-byte words without bank conflicts in either half-warp.
// ------------------------------------------------------------------------------------------------
__host__ __device__ constexpr int rec_stride(int gpl) {
  return gpl > 4 ? 2 * gpl + 1 : (gpl % 2 == 1 ? 2 * gpl : 2 * gpl + 2);
}

struct PackedLayout {
  size_t off_rec, off_ga, off_chars, off_tm, off_tl, off_tx, off_ts, off_tv, off_ti, off_dm, off_dr, off_ds, off_dv;
  size_t off_sectors;  // sector table of the batched kernel (n_sectors > 0)
  size_t off_fsign;    // fermionic sign tables [n_bits][gpl * 32] (fermionic groups)
  size_t total;
};

// One symmetry sector of a batched launch: its states, index, norms, characters and vectors.
// All sectors of a batch share the group's site images, the operator's terms and the basis
// constraint; they differ in the representatives (sector) and the characters.
struct SectorDesc {
  DeviceIndex index;
  const double2* chars;  // packed characters [gpl * 32] (device)
  const double* x;       // first column of this launch's right-hand sides
  double* y;
  int64_t row_begin;     // first row of the sector in the batch's concatenated row space
  int64_t spin_inversion;
  int64_t real_elements; // every matrix element of this sector is real
};
static_assert(sizeof(SectorDesc) % 8 == 0, "sector descriptors are staged as 64-bit words");

// Shared-memory layout of a packed kernel launched with `threads` threads per block.
inline PackedLayout make_packed_layout(const MatvecProblem& p, int n_sectors, int threads) {
  PackedLayout L{};
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  const size_t Gp = 32 * (size_t)p.group.gpl;
  const size_t S = (size_t)rec_stride(p.group.gpl);
  const size_t warps = (size_t)(threads + 31) / 32;
  size_t o = 0;
  L.off_rec = o; o = al(o + (size_t)p.group.n_bits * 32 * S * 4);
  L.off_ga = o; o = al(o + warps * 32 * S * 4);
  L.off_chars = o; o = al(o + (n_sectors > 0 ? 0 : Gp * 16));
  L.off_tm = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tl = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tx = o; o = al(o + (size_t)p.off.n * 8);
  L.off_ts = o; o = al(o + (size_t)p.off.n * 8);
  L.off_tv = o; o = al(o + (size_t)p.off.n * 16);
  L.off_ti = o; o = al(o + (size_t)p.off.n * 4);
  L.off_dm = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_dr = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_ds = o; o = al(o + (size_t)p.diag.n * 8);
  L.off_dv = o; o = al(o + (size_t)p.diag.n * 16);
  L.off_sectors = o; o = al(o + (size_t)n_sectors * sizeof(SectorDesc));
  L.off_fsign = o; o = al(o + (p.group.fermionic ? (size_t)p.group.n_bits * Gp * 8 : 0));
  L.total = o;
  return L;
}

// Shared-memory tables of the packed kernels.
struct PackedTables {
  const uint32_t* rec; // site images as lane records [n_bits][32][S]
  uint32_t* ga;        // per-warp records of g.a [warps][32][S]
  const double2* ch;   // characters (single-sector kernel only)
  const uint64_t *tm, *tl, *tx, *ts;
  const double2* tv;
  const uint32_t* ti;
  const uint64_t *dm, *dr, *ds;
  const double2* dv;
  const uint64_t* fs;  // fermionic sign tables (fermionic groups)
  int nt, nd;
  int all2;            // every off-diagonal term flips two sites and needs no constraint check
};

// Copies the group's site images (as lane records), the term tables and (with_chars) the
// characters into shared memory; the caller synchronises the block afterwards.
__device__ __forceinline__ PackedTables stage_packed(const MatvecProblem& p, const PackedLayout& L,
                                                     unsigned char* smem, bool with_chars) {
  PackedTables T;
  const int gpl = p.group.gpl;
  const int Gp = 32 * gpl;
  const int S = rec_stride(gpl);
  uint32_t* rec = (uint32_t*)(smem + L.off_rec);
  double2* ch = (double2*)(smem + L.off_chars);
  uint64_t* tm = (uint64_t*)(smem + L.off_tm);
  uint64_t* tl = (uint64_t*)(smem + L.off_tl);
  uint64_t* tx = (uint64_t*)(smem + L.off_tx);
  uint64_t* ts = (uint64_t*)(smem + L.off_ts);
  double2* tv = (double2*)(smem + L.off_tv);
  uint32_t* ti = (uint32_t*)(smem + L.off_ti);
  uint64_t* dm = (uint64_t*)(smem + L.off_dm);
  uint64_t* dr = (uint64_t*)(smem + L.off_dr);
  uint64_t* ds = (uint64_t*)(smem + L.off_ds);
  double2* dv = (double2*)(smem + L.off_dv);
  const int n_img = p.group.n_bits * Gp;
  for (int i = threadIdx.x; i < n_img; i += blockDim.x) {
    const int r = i / Gp, e = i - r * Gp;
    const uint64_t v = __ldg(p.group.onehot_packed + i);
    uint32_t* dst = rec + (r * 32 + (e & 31)) * S + 2 * (e >> 5);
    dst[0] = (uint32_t)v;
    dst[1] = (uint32_t)(v >> 32);
  }
  if (with_chars) stage_d2(ch, p.group.chars_packed, Gp);
  stage_u64(tm, p.off.m, p.off.n);
  stage_u64(tl, p.off.l, p.off.n);
  stage_u64(tx, p.off.x, p.off.n);
  stage_u64(ts, p.off.s, p.off.n);
  stage_d2(tv, p.off.v, p.off.n);
  for (int i = threadIdx.x; i < p.off.n; i += blockDim.x) ti[i] = p.off.xinfo[i];
  stage_u64(dm, p.diag.m, p.diag.n);
  stage_u64(dr, p.diag.r, p.diag.n);
  stage_u64(ds, p.diag.s, p.diag.n);
  stage_d2(dv, p.diag.v, p.diag.n);
  uint64_t* fs = (uint64_t*)(smem + L.off_fsign);
  if (p.group.fermionic) stage_u64(fs, p.group.fsign_packed, p.group.n_bits * Gp);
  T.fs = fs;
  T.rec = rec;
  T.ga = (uint32_t*)(smem + L.off_ga);
  T.ch = ch; T.tm = tm; T.tl = tl; T.tx = tx; T.ts = ts; T.tv = tv; T.ti = ti;
  T.dm = dm; T.dr = dr; T.ds = ds; T.dv = dv;
  T.nt = p.off.n;
  T.nd = p.diag.n;
  T.all2 = p.off.all_two_site;
  return T;
}

// Keys of the orbit scan for states of nbits bits (stored in the top bits of a 64-bit word):
// the state bits of the high word, and the flip key (all state bits and the flip bit of the
// candidate index) as its two words.
struct ScanKeys {
  uint32_t hmask, fk_lo, fk_hi;
};
__device__ __forceinline__ ScanKeys scan_keys(int nbits) {
  const int SH = 64 - nbits;
  const uint64_t flipkey = ((~0ull >> SH) << SH) | 1ull;
  return ScanKeys{(uint32_t)(flipkey >> 32), (uint32_t)flipkey, (uint32_t)(flipkey >> 32)};
}

// 32-bit shared-memory loads at explicit shared-window addresses (the record tables are written
// before the block's first barrier and read-only afterwards; the per-warp g.a records use the
// volatile form, ordered with the warp's record stores and __syncwarp).
__device__ __forceinline__ uint32_t lds_u32(uint32_t addr) {
  uint32_t v;
  asm("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ uint32_t lds_u32_volatile(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t lds_u64(uint32_t addr) {
  uint64_t v;
  asm("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ void sts_u32_volatile(uint32_t addr, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" : : "r"(addr), "r"(v) : "memory");
}

// g.a for this lane's slots (XOR of the images of a's set bits, two sites at a time), with the
// candidate index 2 * (lane + 32 k) in the low bits: the high words are returned in gh, both
// words go to this lane's record of the warp's area gw (read by the tie pass of scan_two_site).
template <int GPL>
__device__ __forceinline__ void row_images(const uint32_t* __restrict__ rec, uint32_t* __restrict__ gw, uint64_t a,
                                           int lane, uint32_t (&gh)[GPL]) {
  constexpr int S = rec_stride(GPL);
  constexpr uint32_t ROW = 32u * S * 4u;  // bytes per site
  const uint32_t recl = (uint32_t)__cvta_generic_to_shared(rec) + (uint32_t)(lane * S * 4);
  uint32_t gl[GPL];
#pragma unroll
  for (int k = 0; k < GPL; ++k) gl[k] = gh[k] = 0u;
  uint64_t bits = a;
  while (bits != 0) {
    const uint32_t r0 = recl + (uint32_t)(__ffsll((long long)bits) - 1) * ROW;
    bits &= bits - 1;
    if (bits == 0) {
#pragma unroll
      for (int k = 0; k < GPL; ++k) {
        gl[k] ^= lds_u32(r0 + 8 * k);
        gh[k] ^= lds_u32(r0 + 8 * k + 4);
      }
      break;
    }
    const uint32_t r1 = recl + (uint32_t)(__ffsll((long long)bits) - 1) * ROW;
    bits &= bits - 1;
#pragma unroll
    for (int k = 0; k < GPL; ++k) {
      gl[k] ^= lds_u32(r0 + 8 * k) ^ lds_u32(r1 + 8 * k);
      gh[k] ^= lds_u32(r0 + 8 * k + 4) ^ lds_u32(r1 + 8 * k + 4);
    }
  }
  const uint32_t mine = (uint32_t)__cvta_generic_to_shared(gw) + (uint32_t)(lane * S * 4);
#pragma unroll
  for (int k = 0; k < GPL; ++k) {
    sts_u32_volatile(mine + 8 * k, gl[k] | (uint32_t)(2 * (lane + 32 * k)));
    sts_u32_volatile(mine + 8 * k + 4, gh[k]);
  }
  __syncwarp();
}

// Orbit scan of beta = a ^ (sites s0, s1): the smallest 64-bit key over all slots (and their spin
// flips), i.e. (representative << SH) | (2 * element + flipped), the same key as a full 64-bit
// minimum.  Pass 1: per slot the high word h = g.a ^ image(s0) ^ image(s1); with spin inversion
// the candidate is min(h, flip(h)) and min over slots of that is min(min h, flip(max h)), so one
// min and one max per slot.  Pass 2: only lanes whose pass-1 minimum ties the warp's take part;
// for each, lanes j < GPL rebuild the exact key of its slot j and keep the lowest low word among
// the keys whose high word is the minimum.
template <int GPL, bool INV>
__device__ __forceinline__ uint64_t scan_two_site(const uint32_t* __restrict__ rec, const uint32_t* __restrict__ gw,
                                                  const uint32_t (&gh)[GPL], int s0, int s1, int lane,
                                                  const ScanKeys& K) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int S = rec_stride(GPL);
  constexpr uint32_t ROW = 32u * S * 4u;  // bytes per site
  const uint32_t rec_s = (uint32_t)__cvta_generic_to_shared(rec);
  const uint32_t gw_s = (uint32_t)__cvta_generic_to_shared(gw);
  const uint32_t r0 = rec_s + (uint32_t)s0 * ROW, r1 = rec_s + (uint32_t)s1 * ROW;
  const uint32_t p0 = r0 + (uint32_t)(lane * S * 4 + 4), p1 = r1 + (uint32_t)(lane * S * 4 + 4);
  uint32_t mn = 0xffffffffu, mx = 0u;
#pragma unroll
  for (int k = 0; k < GPL; ++k) {
    const uint32_t h = gh[k] ^ lds_u32(p0 + 8 * k) ^ lds_u32(p1 + 8 * k);
    mn = min(mn, h);
    if (INV) mx = max(mx, h);
  }
  const uint32_t lm = INV ? min(mn, ~mx & K.hmask) : mn;
  const uint32_t mhi = __reduce_min_sync(FULL, lm);
  unsigned M = __ballot_sync(FULL, lm == mhi);
  // lanes beyond the slots repeat the last slot (same candidate): no divergent branch
  const uint32_t jj8 = (uint32_t)((lane < GPL ? lane : GPL - 1) * 8);
  const uint32_t q0 = r0 + jj8, q1 = r1 + jj8, qg = gw_s + jj8;
  uint32_t blo = 0xffffffffu;
  do {
    const uint32_t o = (uint32_t)(__ffs(M) - 1) * (uint32_t)(S * 4);
    M &= M - 1;
    uint32_t lo = lds_u32_volatile(qg + o) ^ lds_u32(q0 + o) ^ lds_u32(q1 + o);
    uint32_t hi = lds_u32_volatile(qg + o + 4) ^ lds_u32(q0 + o + 4) ^ lds_u32(q1 + o + 4);
    if (INV) {  // flip when the top state bit is set: all-ones mask from the sign bit
      const uint32_t f = (uint32_t)((int32_t)hi >> 31);
      lo ^= K.fk_lo & f;
      hi ^= K.fk_hi & f;
    }
    blo = (hi == mhi) ? min(blo, lo) : blo;
  } while (M != 0);
  const uint32_t mlo = __reduce_min_sync(FULL, blo);
  return ((uint64_t)mhi << 32) | mlo;
}

// Orbit scan of beta = a ^ xt for any number of flipped sites: full 64-bit keys per slot.
// (Groups of more than 4 slots per lane; the warp's records hold the low words of g.a.)
template <int GPL, bool INV>
__device__ __forceinline__ uint64_t scan_general(const uint32_t* __restrict__ rec, const uint32_t* __restrict__ gw,
                                                 const uint32_t (&gh)[GPL], uint64_t xt, int lane,
                                                 const ScanKeys& K) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int S = rec_stride(GPL);
  const uint32_t* recl = rec + lane * S;
  const uint32_t* mine = gw + lane * S;
  const uint64_t fk = ((uint64_t)K.fk_hi << 32) | K.fk_lo;
  uint64_t cand[GPL];
#pragma unroll
  for (int k = 0; k < GPL; ++k) {
    uint32_t lo = mine[2 * k], hi = gh[k];
    for (uint64_t bits = xt; bits != 0; bits &= bits - 1) {
      const uint32_t* r = recl + (__ffsll((long long)bits) - 1) * 32 * S + 2 * k;
      lo ^= r[0];
      hi ^= r[1];
    }
    const uint64_t v = ((uint64_t)hi << 32) | lo;
    cand[k] = (INV && (int32_t)hi < 0) ? (v ^ fk) : v;
  }
#pragma unroll
  for (int w = 1; w < GPL; w *= 2) {
#pragma unroll
    for (int k = 0; k + w < GPL; k += 2 * w) cand[k] = cand[k + w] < cand[k] ? cand[k + w] : cand[k];
  }
  const uint32_t hi = (uint32_t)(cand[0] >> 32), lo = (uint32_t)cand[0];
  const uint32_t mhi = __reduce_min_sync(FULL, hi);
  const uint32_t mlo = __reduce_min_sync(FULL, hi == mhi ? lo : 0xffffffffu);
  return ((uint64_t)mhi << 32) | mlo;
}

// The orbit scan of one warp's row: init(a) computes g.a for the lane's slots, two_site / general
// return the packed key of a generated state.  More than 4 slots per lane: the two-pass scan
// (high words in registers, both words in the warp's records).  Up to 4: every slot's 64-bit key
// directly (a short scan, where the tie pass would cost more than it saves).
template <int GPL, bool INV, bool SMALL = (GPL <= 4)>
struct RowScan {
  const uint32_t* rec;
  uint32_t* gw;
  ScanKeys keys;
  int lane;
  uint32_t gh[GPL];
  __device__ __forceinline__ void init(uint64_t a) {
    __syncwarp();  // the previous row's scans have read the records
    row_images<GPL>(rec, gw, a, lane, gh);
  }
  __device__ __forceinline__ uint64_t two_site(int s0, int s1) const {
    return scan_two_site<GPL, INV>(rec, gw, gh, s0, s1, lane, keys);
  }
  __device__ __forceinline__ uint64_t general(uint64_t xt) const {
    return scan_general<GPL, INV>(rec, gw, gh, xt, lane, keys);
  }
};

template <int GPL, bool INV>
struct RowScan<GPL, INV, true> {
  static constexpr int S = rec_stride(GPL);
  const uint32_t* rec;
  uint32_t* gw;  // unused: no tie pass
  ScanKeys keys;
  int lane;
  uint64_t ga[GPL];
  __device__ __forceinline__ const uint2* row(int site) const {
    return reinterpret_cast<const uint2*>(rec + (site * 32 + lane) * S);
  }
  __device__ __forceinline__ static uint64_t word(uint2 v) { return ((uint64_t)v.y << 32) | v.x; }
  __device__ __forceinline__ void init(uint64_t a) {
#pragma unroll
    for (int k = 0; k < GPL; ++k) ga[k] = 0;
    for (uint64_t bits = a; bits != 0; bits &= bits - 1) {
      const uint2* r = row(__ffsll((long long)bits) - 1);
#pragma unroll
      for (int k = 0; k < GPL; ++k) ga[k] ^= word(r[k]);
    }
#pragma unroll
    for (int k = 0; k < GPL; ++k) ga[k] |= (uint64_t)(2 * (lane + 32 * k));
  }
  __device__ __forceinline__ uint64_t reduce(uint64_t (&cand)[GPL]) const {
    constexpr unsigned FULL = 0xffffffffu;
    if (INV) {
      const uint64_t fk = ((uint64_t)keys.fk_hi << 32) | keys.fk_lo;
#pragma unroll
      for (int k = 0; k < GPL; ++k) {
        const uint32_t m = (uint32_t)((int32_t)(uint32_t)(cand[k] >> 32) >> 31);
        cand[k] ^= fk & (((uint64_t)m << 32) | m);
      }
    }
#pragma unroll
    for (int w = 1; w < GPL; w *= 2) {
#pragma unroll
      for (int k = 0; k + w < GPL; k += 2 * w) cand[k] = cand[k + w] < cand[k] ? cand[k + w] : cand[k];
    }
    const uint32_t hi = (uint32_t)(cand[0] >> 32), lo = (uint32_t)cand[0];
    const uint32_t mhi = __reduce_min_sync(FULL, hi);
    const uint32_t mlo = __reduce_min_sync(FULL, hi == mhi ? lo : 0xffffffffu);
    return ((uint64_t)mhi << 32) | mlo;
  }
  __device__ __forceinline__ uint64_t two_site(int s0, int s1) const {
    const uint2* r0 = row(s0);
    const uint2* r1 = row(s1);
    uint64_t cand[GPL];
#pragma unroll
    for (int k = 0; k < GPL; ++k) cand[k] = ga[k] ^ word(r0[k]) ^ word(r1[k]);
    return reduce(cand);
  }
  __device__ __forceinline__ uint64_t general(uint64_t xt) const {
    uint64_t cand[GPL];
#pragma unroll
    for (int k = 0; k < GPL; ++k) cand[k] = ga[k];
    for (uint64_t bits = xt; bits != 0; bits &= bits - 1) {
      const uint2* r = row(__ffsll((long long)bits) - 1);
#pragma unroll
      for (int k = 0; k < GPL; ++k) cand[k] ^= word(r[k]);
    }
    return reduce(cand);
  }
};

// One output row of the packed kernels (executed by a whole warp): y[row, 0..K) for the sector
// described by (ix, chars, spin_inversion, x, y).
//
// PAIR (complex blocks): xs holds x_j * n_j as (hi, lo) float pairs [re_h, re_l, im_h, im_l]
// (16 bytes per element, like complex128) and the multiply-adds run in FP32-pair arithmetic
// (pairs.cuh): the coefficient is formed in FP64 and split once per element; each lane's pair
// sums are converted to FP64 before the cross-lane reduction.  With 16 right-hand sides the FP64
// form is bound by GB300's narrow FP64 pipe (4 FP64 FMAs per element and column).
template <int GPL, bool INV, bool CPLX, int K, bool FERMI = false, bool PAIR = false, bool SMEM_IX = false>
__device__ __forceinline__ void packed_row(const PackedTables& T, const int nbits, const DeviceIndex& ix,
                                           const double2* __restrict__ chars, const int spin_inversion,
                                           const DeviceConstraint& cons, const double* __restrict__ x,
                                           const int64_t ldx, double* __restrict__ y, const int64_t ldy,
                                           const int64_t row, int* __restrict__ err,
                                           const uint64_t* __restrict__ binom,
                                           unsigned long long* nnz_counter, const bool real_elements,
                                           const double* __restrict__ xs = nullptr, const int64_t ldxs = 0,
                                           const DeviceIndex* ix_smem = nullptr,
                                           const double2* const* chars_smem = nullptr) {
  // gather source: x_j * n_j when prescaled (xs), else x_j with the norm applied per element
  const bool prescaled = xs != nullptr;
  const double* __restrict__ xg = prescaled ? xs : x;
  const int64_t ldg = prescaled ? ldxs : ldx;
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int Gp = 32 * GPL;
  constexpr int Q = 32 / K;
  const int lane = threadIdx.x & 31;
  const int SH = 64 - nbits;
  const uint64_t lowmask = (1ull << SH) - 1;
  const int rhs = lane % K;
  const int q = lane / K;
  const int nt = T.nt;
  RowScan<GPL, INV> scan;
  scan.rec = T.rec;
  scan.gw = T.ga + (threadIdx.x >> 5) * 32 * rec_stride(GPL);  // this warp's g.a records
  scan.keys = scan_keys(nbits);
  scan.lane = lane;

  const uint64_t a = __ldg(ix.reps + row);
  const double inv_na = __ldg(ix.inv_norms + row);
  if (inv_na == 0.0) {
    // A representative whose orbit norm is zero spans no state of the sector (the reference's
    // floating stabiliser sum can keep such states as rounding residue in complex sectors): its
    // row and column of H are zero.  The value is the same on every lane: the warp stays converged.
    if (lane < K) {
      if constexpr (CPLX) reinterpret_cast<double2*>(y)[row * ldy + lane] = make_double2(0.0, 0.0);
      else y[row * ldy + lane] = 0.0;
    }
    return;
  }
  // g.a for this lane's slots
  scan.init(a);

  Acc acc;
  F2 pre{0.0f, 0.0f}, pim{0.0f, 0.0f};  // PAIR: this lane's pair sums
  unsigned found = 0;
  // Lane s of the warp owns the s-th generated element since the last flush: the winning key
  // (representative + group slot) and the term that generated it.  The element's coefficient,
  // its sign and the state beta are only needed by the owning lane, at the flush.
  uint64_t my_key = ~0ull;
  int my_t = 0;
  int nslot = 0;

  auto flush = [&]() {
    int64_t j = -1;
    double fre = 0.0, fim = 0.0;
    if (lane < nslot) {
      const uint64_t rep = my_key >> SH;
      const uint32_t idx = (uint32_t)(my_key & lowmask);
      // SMEM_IX (batched kernel): the sector's index and characters are re-read from the shared
      // sector table here, once per 32 elements
      const DeviceIndex ixl = SMEM_IX ? reload_index(ix_smem) : ix;
      j = mv_index_lookup(ixl, rep, binom);
      // a zero-norm column contributes nothing (prescaled: its x_j * n_j is already zero)
      const double nj = prescaled ? 1.0 : (j >= 0 ? __ldg(ixl.norms + j) : 0.0);
      if (nj == 0.0) j = -1;
      found += (j >= 0);
      if (j >= 0) {
        const uint64_t beta = a ^ T.tx[my_t];
        // coefficient v_t (-1)^popcount(beta & s_t), the sign applied to the sign bits
        double2 c = T.tv[my_t];
        const long long sbit = (long long)(__popcll(beta & T.ts[my_t]) & 1) << 63;
        c.x = __longlong_as_double(__double_as_longlong(c.x) ^ sbit);
        c.y = __longlong_as_double(__double_as_longlong(c.y) ^ sbit);
        const double2* chs = chars;
        if constexpr (SMEM_IX) chs = *(const double2* const volatile*)chars_smem;
        double2 chi = chs[idx >> 1];
        if (INV && (idx & 1) && spin_inversion == -1) chi = make_double2(-chi.x, -chi.y);
        if constexpr (FERMI) {
          // g moves the fermions of beta onto the representative with the sign of the
          // permutation it induces on the occupied orbitals (one lane per element)
          if (fermion_parity(T.fs + (idx >> 1), Gp, beta)) chi = make_double2(-chi.x, -chi.y);
        }
        const C2 f = cmul_conj_b(C2{c.x, c.y}, C2{chi.x, chi.y});
        fre = prescaled ? f.re : f.re * nj;
        fim = prescaled ? f.im : f.im * nj;
      }
    }
    if constexpr (PAIR) {
      static_assert(CPLX && K >= 2, "pair accumulation is for complex blocks");
      const F2 cr = split_double(fre), ci = split_double(fim);
      // U passes at a time: their gathers are issued before the multiply-adds, so that U loads
      // per lane are in flight (the pair arithmetic leaves the kernel latency-bound otherwise)
      constexpr int U = SMEM_IX ? 2 : 4;  // the batched kernel holds more live state per row
      const float4* __restrict__ xp = reinterpret_cast<const float4*>(xg);
      for (int s0 = 0; s0 < nslot; s0 += U * Q) {
        float4 xv[U];
        unsigned ok = 0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = s0 + u * Q + q;
          const int64_t js = __shfl_sync(FULL, j, s & 31);
          const bool valid = s < nslot && js >= 0;
          ok |= valid ? 1u << u : 0u;
          xv[u] = valid ? __ldg(xp + js * ldg + rhs) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int src = (s0 + u * Q + q) & 31;
          const float crh = __shfl_sync(FULL, cr.h, src), crl = __shfl_sync(FULL, cr.l, src);
          const float cih = __shfl_sync(FULL, ci.h, src), cil = __shfl_sync(FULL, ci.l, src);
          if (ok & (1u << u)) {
            // (cr + i ci)(xr + i xi); real elements (warp-uniform) have ci = 0
            mac(pre, crh, crl, xv[u].x, xv[u].y);
            mac(pim, crh, crl, xv[u].z, xv[u].w);
            if (!real_elements) {
              mac(pre, -cih, -cil, xv[u].z, xv[u].w);
              mac(pim, cih, cil, xv[u].x, xv[u].y);
            }
            renorm(pre);
            renorm(pim);
          }
        }
      }
      return;
    }
    if (CPLX && real_elements) {
      // real matrix elements (warp-uniform branch): complex x times a real factor
      for (int s0 = 0; s0 < nslot; s0 += Q) {
        const int s = s0 + q;
        const int src = s & 31;
        const int64_t js = (K == 1) ? j : __shfl_sync(FULL, j, src);
        const double sre = (K == 1) ? fre : __shfl_sync(FULL, fre, src);
        if (s < nslot && js >= 0) {
          const double2 xv = __ldg(reinterpret_cast<const double2*>(xg) + js * ldg + rhs);
          acc.re += sre * xv.x;
          acc.im += sre * xv.y;
        }
        if (K == 1) break;
      }
      return;
    }
    for (int s0 = 0; s0 < nslot; s0 += Q) {
      const int s = s0 + q;
      const int src = s & 31;
      const int64_t js = (K == 1) ? j : __shfl_sync(FULL, j, src);
      const double sre = (K == 1) ? fre : __shfl_sync(FULL, fre, src);
      const double sim = (K == 1) ? fim : __shfl_sync(FULL, fim, src);
      if (s < nslot && js >= 0) {
        if constexpr (CPLX) {
          const double2 xv = __ldg(reinterpret_cast<const double2*>(xg) + js * ldg + rhs);
          acc.re += sre * xv.x - sim * xv.y;
          acc.im += sre * xv.y + sim * xv.x;
        } else {
          acc.re += sre * __ldg(xg + js * ldg + rhs);
        }
      }
      if (K == 1) break;
    }
  };

  if (T.all2) {
    // Every term flips two sites and keeps the conserved numbers (warp-uniform): batches of up
    // to 32 elements are scanned in a tight loop, each batch then flushed.
    const uint32_t tm_s = (uint32_t)__cvta_generic_to_shared(T.tm);
    const uint32_t tl_s = (uint32_t)__cvta_generic_to_shared(T.tl);
    const uint32_t ti_s = (uint32_t)__cvta_generic_to_shared(T.ti);
    int t0 = 0;
    // lanes past the last term read term 0 (inside the table) and do not match
    unsigned mask = __ballot_sync(FULL, lane < nt && (a & lds_u64(tm_s + (lane < nt ? 8u * lane : 0u))) ==
                                                         lds_u64(tl_s + (lane < nt ? 8u * lane : 0u)));
    for (;;) {
      nslot = 0;
      while (nslot < 32) {
        while (mask == 0 && t0 + 32 < nt) {
          t0 += 32;
          const bool in = t0 + lane < nt;
          const uint32_t o = in ? 8u * (uint32_t)(t0 + lane) : 0u;  // lanes past the terms read term 0
          mask = __ballot_sync(FULL, in && (a & lds_u64(tm_s + o)) == lds_u64(tl_s + o));
        }
        if (mask == 0) break;
        const int t = t0 + __ffs(mask) - 1;
        mask &= mask - 1;
        const uint32_t info = lds_u32(ti_s + 4u * (uint32_t)t);
        const uint64_t key = scan.two_site((int)(info & 0xffu), (int)((info >> 8) & 0xffu));
        my_key = lane == nslot ? key : my_key;
        my_t = lane == nslot ? t : my_t;
        ++nslot;
      }
      if (nslot > 0) flush();
      if (nslot < 32) break;
    }
    nslot = 0;
  }
  for (int t0 = 0; !T.all2 && t0 < nt; t0 += 32) {
    const int tt = t0 + lane;
    const bool hit = tt < nt && (a & T.tm[tt]) == T.tl[tt];
    unsigned mask = __ballot_sync(FULL, hit);
    while (mask != 0) {
      const int t = t0 + __ffs(mask) - 1;
      mask &= mask - 1;
      const uint64_t xt = T.tx[t];
      const uint32_t info = T.ti[t];
      if (info & kTermNeedsCheck) {
        if (!constraint_ok(cons, a ^ xt)) {
          if (lane == 0) atomicOr(err, 1);
          continue;
        }
      }
      const uint64_t key = (((info >> 16) & 0xffu) == 2u)
                               ? scan.two_site((int)(info & 0xffu), (int)((info >> 8) & 0xffu))
                               : scan.general(xt);
      if (lane == nslot) {
        my_key = key;
        my_t = t;
      }
      if (++nslot == 32) {
        flush();
        nslot = 0;
      }
    }
  }
  if (nslot > 0) flush();

  // the diagonal element, after the off-diagonal scan (its sums are not live across the scan)
  double dre = 0.0, dim = 0.0;
  F2 dpr{0.0f, 0.0f}, dpi{0.0f, 0.0f};  // PAIR: the diagonal element as pairs
  if constexpr (PAIR) {
    for (int t = lane; t < T.nd; t += 32) {
      if ((a & T.dm[t]) == T.dr[t]) {
        const double2 v = T.dv[t];
        const bool neg = __popcll(a & T.ds[t]) & 1;
        const F2 vr = split_double(v.x), vi = split_double(v.y);
        dpr = pair_add(dpr, neg ? pair_neg(vr) : vr);
        dpi = pair_add(dpi, neg ? pair_neg(vi) : vi);
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      dpr = pair_add(dpr, pair_shfl_xor(dpr, d));
      dpi = pair_add(dpi, pair_shfl_xor(dpi, d));
    }
  } else {
    for (int t = lane; t < T.nd; t += 32) {
      if ((a & T.dm[t]) == T.dr[t]) {
        const double2 v = T.dv[t];
        const bool neg = __popcll(a & T.ds[t]) & 1;
        dre += neg ? -v.x : v.x;
        if constexpr (CPLX) dim += neg ? -v.y : v.y;
      }
    }
    dre = warp_sum(dre);
    if constexpr (CPLX) dim = warp_sum(dim);
  }

  if constexpr (PAIR) {
    // FP32-pair epilogue: lanes with the same column combine, then
    // y = acc / n_a + diag x_a, all in pairs; two FP64 adds per output
#pragma unroll
    for (int d = 16; d >= K; d >>= 1) {
      pre = pair_add(pre, pair_shfl_xor(pre, d));
      pim = pair_add(pim, pair_shfl_xor(pim, d));
    }
    if (lane < K) {
      const double2 xi = __ldg(reinterpret_cast<const double2*>(x) + row * ldx + lane);
      const F2 inv = split_double(inv_na), xr = split_double(xi.x), xm = split_double(xi.y);
      F2 orr{0.0f, 0.0f}, oim{0.0f, 0.0f};
      mac(orr, pre, inv);
      mac(orr, dpr, xr);
      mac(orr, pair_neg(dpi), xm);
      mac(oim, pim, inv);
      mac(oim, dpr, xm);
      mac(oim, dpi, xr);
      reinterpret_cast<double2*>(y)[row * ldy + lane] = make_double2(join(orr), join(oim));
    }
    if (nnz_counter != nullptr) {
      const unsigned total = __reduce_add_sync(FULL, found);
      if (lane == 0 && total) atomicAdd(nnz_counter, (unsigned long long)total);
    }
    return;
  }
  if (nnz_counter != nullptr) {
    const unsigned total = __reduce_add_sync(FULL, found);
    if (lane == 0 && total) atomicAdd(nnz_counter, (unsigned long long)total);
  }

  if constexpr (CPLX) {
#pragma unroll
    for (int d = 16; d >= K; d >>= 1) {
      acc.re += __shfl_xor_sync(FULL, acc.re, d);
      acc.im += __shfl_xor_sync(FULL, acc.im, d);
    }
    if (lane < K) {
      const double2 xi = __ldg(reinterpret_cast<const double2*>(x) + row * ldx + lane);
      double2 out;
      out.x = acc.re * inv_na + (dre * xi.x - dim * xi.y);
      out.y = acc.im * inv_na + (dre * xi.y + dim * xi.x);
      reinterpret_cast<double2*>(y)[row * ldy + lane] = out;
    }
  } else {
#pragma unroll
    for (int d = 16; d >= K; d >>= 1) acc.re += __shfl_xor_sync(FULL, acc.re, d);
    if (lane < K) y[row * ldy + lane] = acc.re * inv_na + dre * __ldg(x + row * ldx + lane);
  }
}

// Launch bounds of the packed single-sector kernels.  Kernels with at most two FP64 accumulators
// per lane (one complex or up to two real right-hand sides) run CTAs of up to 1024 threads (at
// most 64 registers per thread; 768 threads and 85 registers for groups of more than 288
// elements): one CTA per SM, whose 32 warps share one copy of the tables; wider FP64 blocks up to
// 640 threads (102 registers); the pair kernels keep 320-thread CTAs, three per SM on small
// groups (more warps to hide the gathers' latency).
template <int GPL, int K, bool PAIR, bool CPLX = true>
struct PackedBounds {
  static constexpr int threads = PAIR ? 320 : (K * (CPLX ? 2 : 1) <= 2 ? (GPL <= 9 ? 1024 : 768) : 640);
  static constexpr int min_blocks = PAIR ? ((GPL <= 2) ? 3 : 2) : 1;
};

template <int GPL, bool INV, bool CPLX, int K, bool FERMI = false, bool PAIR = false>
__global__ void __launch_bounds__(PackedBounds<GPL, K, PAIR, CPLX>::threads, PackedBounds<GPL, K, PAIR, CPLX>::min_blocks)
    k_matvec_packed(const MatvecProblem p, const PackedLayout L, const double* __restrict__ x, int64_t ldx,
                    double* __restrict__ y, int64_t ldy, int* __restrict__ err,
                    const uint64_t* __restrict__ binom) {
  extern __shared__ __align__(16) unsigned char smem[];
  const PackedTables T = stage_packed(p, L, smem, true);
  __syncthreads();
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp_id; row < p.n_rows; row += n_warps)
    packed_row<GPL, INV, CPLX, K, FERMI, PAIR>(T, p.group.n_bits, p.index, T.ch, p.group.spin_inversion, p.constraint,
                                               x, ldx, y, ldy, row, err, binom, p.nnz_counter,
                                               p.real_elements != 0, p.xs, p.ldxs);
}

// Batched kernel: the rows of all sectors form one row space that a persistent grid walks; each
// warp looks up the sector of its row in the shared sector table.  `p` carries the shared
// tables (site images, terms, constraint) of the first sector.
template <int GPL, bool INV, int K, bool PAIR = false>
__global__ void __launch_bounds__(320, (PAIR && GPL <= 2) ? 3 : 2)
    k_matvec_sectors(const MatvecProblem p, const PackedLayout L, const SectorDesc* __restrict__ sectors,
                     int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy, int* __restrict__ err,
                     const uint64_t* __restrict__ binom, const double* __restrict__ xs_all, int64_t ldxs,
                     int col) {
  extern __shared__ __align__(16) unsigned char smem[];
  const PackedTables T = stage_packed(p, L, smem, false);
  SectorDesc* sd = (SectorDesc*)(smem + L.off_sectors);
  {
    const uint64_t* src = reinterpret_cast<const uint64_t*>(sectors);
    uint64_t* dst = reinterpret_cast<uint64_t*>(sd);
    const int words = n_sectors * (int)(sizeof(SectorDesc) / 8);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int cur = 0;  // sector of the previous row: a warp's rows stay in one sector for many steps
  for (int64_t row = warp_id; row < total_rows; row += n_warps) {
    if (row < sd[cur].row_begin || (cur + 1 < n_sectors && row >= sd[cur + 1].row_begin)) {
      int lo = 0, hi = n_sectors - 1;  // last sector with row_begin <= row
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sd[mid].row_begin <= row) lo = mid; else hi = mid - 1;
      }
      cur = lo;
    }
    const SectorDesc& S = sd[cur];
    // gather source: the sector's rows of the prescaled copy of all columns (x_j * n_j, FP64 or
    // pairs), if the launch made one
    const double* xs = xs_all != nullptr ? xs_all + ((size_t)S.row_begin * ldxs + col) * 2 : nullptr;
    packed_row<GPL, INV, true, K, false, PAIR, true>(T, p.group.n_bits, S.index, S.chars, (int)S.spin_inversion,
                                                     p.constraint, S.x, ldx, S.y, ldy, row - S.row_begin, err,
                                                     binom, p.nnz_counter, S.real_elements != 0, xs, ldxs,
                                                     &S.index, &S.chars);
  }
}

// ------------------------------------------------------------------------------------------------
// Unprojected / spin-inversion-only kernel: one thread per row.
// ------------------------------------------------------------------------------------------------
template <bool CPLX, bool INV>
__global__ void __launch_bounds__(256)
    k_matvec_plain(const MatvecProblem p, const SmemLayout L, const double* __restrict__ x,
                   int64_t ldx, double* __restrict__ y, int64_t ldy, int k_rhs,
                   int* __restrict__ err, const uint64_t* __restrict__ binom) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Staged S = stage_problem(p, L, smem, false);
  const uint64_t flip = p.group.flip;
  const double chi_flip = (double)p.group.spin_inversion;
  unsigned long long found = 0;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < p.n_rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = (p.index.identity) ? (uint64_t)row : __ldg(p.index.reps + row);
    double dre = 0.0, dim = 0.0;
    for (int t = 0; t < p.diag.n; ++t) {
      if ((a & S.dm[t]) == S.dr[t]) {
        const double2 v = S.dv[t];
        const bool neg = __popcll(a & S.ds[t]) & 1;
        dre += neg ? -v.x : v.x;
        dim += neg ? -v.y : v.y;
      }
    }
    for (int r = 0; r < k_rhs; ++r) {
      double are = 0.0, aim = 0.0;
      if constexpr (CPLX) {
        const double2 xi = reinterpret_cast<const double2*>(x)[row * ldx + r];
        are = dre * xi.x - dim * xi.y;
        aim = dre * xi.y + dim * xi.x;
      } else {
        are = dre * x[row * ldx + r];
      }
      for (int t = 0; t < p.off.n; ++t) {
        if ((a & S.tm[t]) != S.tl[t]) continue;
        uint64_t beta = a ^ S.tx[t];
        if (!constraint_ok(p.constraint, beta)) {
          atomicOr(err, 1);
          continue;
        }
        double2 c = S.tv[t];
        if (__popcll(beta & S.ts[t]) & 1) c = make_double2(-c.x, -c.y);
        if (INV) {
          const uint64_t inv = beta ^ flip;
          if (inv < beta) {
            beta = inv;
            c = make_double2(c.x * chi_flip, c.y * chi_flip);
          }
        }
        const int64_t j = mv_index_lookup(p.index, beta, binom);
        if (j < 0) continue;
        if (r == 0) ++found;
        if constexpr (CPLX) {
          const double2 xv = reinterpret_cast<const double2*>(x)[j * ldx + r];
          are += c.x * xv.x - c.y * xv.y;
          aim += c.x * xv.y + c.y * xv.x;
        } else {
          are += c.x * x[j * ldx + r];
        }
      }
      if constexpr (CPLX) {
        reinterpret_cast<double2*>(y)[row * ldy + r] = make_double2(are, aim);
      } else {
        y[row * ldy + r] = are;
      }
    }
  }
  if (p.nnz_counter != nullptr && found) atomicAdd(p.nnz_counter, found);
}

}  // namespace lsg
