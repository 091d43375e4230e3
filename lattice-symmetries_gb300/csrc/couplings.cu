// couplings.cu -- per-coupling inner products out[c] = <g, H_c x> = sum_i conj(g_i) (H_c x)_i for an
// operator H = sum_c H_c whose terms carry coupling ids (the backward pass of H(theta) x with
// respect to the coupling constants theta_c, since d/dtheta_c Re<g, H(theta) x> = Re out[c]).
//
// One pass over the rows, the same orbit scan as the packed matvec (one warp per row): every
// element's contribution conj(g_i) / n_i * v_t (-1)^popcount(beta & s_t) conj(chi) n_j x_j goes to
// the accumulator of its term's coupling instead of to y_i.  Per-lane sums are reduced per block,
// the block partials by one more small kernel in a fixed order (deterministic).
#include <type_traits>

#include "matvec_launch.cuh"

namespace lsg {

extern const uint64_t* device_binomials();
constexpr int kMaxCouplings = 4;

template <int GPL, bool INV>
__global__ void __launch_bounds__(256, 2)
    k_coupling_products(const MatvecProblem p, const PackedLayout L, size_t off_cpl, int nc,
                        const double* __restrict__ g, const double* __restrict__ x,
                        double2* __restrict__ partial, int* __restrict__ err,
                        const uint64_t* __restrict__ binom) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr unsigned FULL = 0xffffffffu;
  const PackedTables T = stage_packed(p, L, smem, true);
  int32_t* cpl_off = (int32_t*)(smem + off_cpl);
  int32_t* cpl_diag = cpl_off + p.off.n;
  for (int i = threadIdx.x; i < p.off.n + p.diag.n; i += blockDim.x) cpl_off[i] = p.off.coupling[i];
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int nbits = p.group.n_bits;
  const int SH = 64 - nbits;
  const uint64_t lowmask = (1ull << SH) - 1;
  RowScan<GPL, INV> scan;
  scan.rec = T.rec;
  scan.gw = T.ga + (threadIdx.x >> 5) * 32 * rec_stride(GPL);  // this warp's g.a records
  scan.keys = scan_keys(nbits);
  scan.lane = lane;
  const double2* X = reinterpret_cast<const double2*>(x);
  const double2* Gv = reinterpret_cast<const double2*>(g);
  const DeviceIndex& ix = p.index;

  double2 tot[kMaxCouplings];
#pragma unroll
  for (int c = 0; c < kMaxCouplings; ++c) tot[c] = make_double2(0.0, 0.0);
  auto add = [&](int cid, double re, double im) {
#pragma unroll
    for (int c = 0; c < kMaxCouplings; ++c)
      if (c == cid) {
        tot[c].x += re;
        tot[c].y += im;
      }
  };

  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp_id; row < p.n_rows; row += n_warps) {
    const uint64_t a = __ldg(ix.reps + row);
    const double inv_na = __ldg(ix.inv_norms + row);
    if (inv_na == 0.0) continue;  // zero-norm representative: zero row
    const double2 gi = __ldg(Gv + row);
    const double2 xi = __ldg(X + row);
    const C2 gx = cmul_conj_b(C2{xi.x, xi.y}, C2{gi.x, gi.y});  // conj(g_i) x_i
    const C2 w{gi.x * inv_na, -gi.y * inv_na};                   // conj(g_i) / n_i

    for (int t = lane; t < T.nd; t += 32) {
      if ((a & T.dm[t]) == T.dr[t]) {
        double2 v = T.dv[t];
        if (__popcll(a & T.ds[t]) & 1) v = make_double2(-v.x, -v.y);
        const C2 val = cmul(C2{v.x, v.y}, gx);
        add(cpl_diag[t], val.re, val.im);
      }
    }

    scan.init(a);

    // the owning lane of each element keeps its key and term; coefficient, sign and coupling
    // are read at the flush
    uint64_t my_key = ~0ull;
    int my_t = 0;
    int nslot = 0;
    auto flush = [&]() {
      if (lane < nslot) {
        const uint64_t rep = my_key >> SH;
        const uint32_t idx = (uint32_t)(my_key & lowmask);
        const int64_t j = mv_index_lookup(ix, rep, binom);
        const double nj = j >= 0 ? __ldg(ix.norms + j) : 0.0;
        if (nj != 0.0) {
          double2 my_c = T.tv[my_t];
          if (__popcll((a ^ T.tx[my_t]) & T.ts[my_t]) & 1) my_c = make_double2(-my_c.x, -my_c.y);
          const int my_cid = cpl_off[my_t];
          double2 chi = T.ch[idx >> 1];
          if (INV && (idx & 1) && p.group.spin_inversion == -1) chi = make_double2(-chi.x, -chi.y);
          const C2 f = cmul_conj_b(C2{my_c.x * nj, my_c.y * nj}, C2{chi.x, chi.y});
          const double2 xv = __ldg(X + j);
          const C2 val = cmul(w, cmul(f, C2{xv.x, xv.y}));
          add(my_cid, val.re, val.im);
        }
      }
    };

    const int nt = T.nt;
    for (int t0 = 0; t0 < nt; t0 += 32) {
      const int tt = t0 + lane;
      const bool hit = tt < nt && (a & T.tm[tt]) == T.tl[tt];
      unsigned mask = __ballot_sync(FULL, hit);
      while (mask != 0) {
        const int t = t0 + __ffs(mask) - 1;
        mask &= mask - 1;
        const uint64_t xt = T.tx[t];
        const uint32_t info = T.ti[t];
        if (info & kTermNeedsCheck) {
          if (!constraint_ok(p.constraint, a ^ xt)) {
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
  }

  // block reduction: lanes -> warps (shuffles) -> block (shared memory, fixed order)
  __shared__ double2 wsum[32][kMaxCouplings];
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < kMaxCouplings; ++c) {
    double re = tot[c].x, im = tot[c].y;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      re += __shfl_xor_sync(FULL, re, d);
      im += __shfl_xor_sync(FULL, im, d);
    }
    if (lane == 0) wsum[warp][c] = make_double2(re, im);
  }
  __syncthreads();
  if (threadIdx.x < nc) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      s.x += wsum[w][threadIdx.x].x;
      s.y += wsum[w][threadIdx.x].y;
    }
    partial[(size_t)blockIdx.x * nc + threadIdx.x] = s;
  }
}

__global__ void k_sum_partials(const double2* __restrict__ partial, int n_blocks, int nc, double2* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= nc) return;
  double2 s = make_double2(0.0, 0.0);
  for (int b = 0; b < n_blocks; ++b) {
    s.x += partial[(size_t)b * nc + c].x;
    s.y += partial[(size_t)b * nc + c].y;
  }
  out[c] = s;
}

int launch_coupling_products(const MatvecProblem& p, int nc, const double* d_g, const double* d_x, double* d_out,
                             int* d_err, cudaStream_t s) {
  if (nc < 1 || nc > kMaxCouplings)
    return fail(LS_GPU_ERR_INVALID, "the fused coupling kernel handles 1 to 4 couplings");
  if (p.projection != 2 || p.group.gpl < 1 || p.group.gpl > 4 || p.group.onehot_packed == nullptr)
    return fail(LS_GPU_ERR_INVALID, "the fused coupling kernel needs a basis with lattice symmetries of at most "
                                    "128 elements");
  if (p.group.fermionic) return fail(LS_GPU_ERR_INVALID, "the fused coupling kernel has no fermionic signs");
  if (p.off.coupling == nullptr) return fail(LS_GPU_ERR_INVALID, "operator terms carry no coupling ids");
  const uint64_t* binom = device_binomials();
  if (binom == nullptr) return LS_GPU_ERR_CUDA;
  const PackedLayout L = make_packed_layout(p, 0, 256);
  const size_t off_cpl = (L.total + 15) & ~(size_t)15;
  const size_t smem = off_cpl + (size_t)(p.off.n + p.diag.n) * 4;
  if (smem > kMaxDynamicSmem) return fail(LS_GPU_ERR_INVALID, "term tables too large for shared memory");
  const int blocks = std::max(1, std::min(num_sms() * 8, (int)((p.n_rows + 7) / 8)));
  double2* partial = (double2*)scratch((size_t)blocks * nc * sizeof(double2), 6);
  if (partial == nullptr) return LS_GPU_ERR_CUDA;
  auto go = [&](auto kern) -> int {
    StageScope stage("couplings.kernel", s);
    if (!ensure_smem_limit((const void*)kern, smem)) return LS_GPU_ERR_CUDA;
    kern<<<blocks, 256, smem, s>>>(p, L, off_cpl, nc, d_g, d_x, partial, d_err, binom);
    if (!cuda_ok(cudaGetLastError(), "k_coupling_products")) return LS_GPU_ERR_CUDA;
    k_sum_partials<<<1, 32, 0, s>>>(partial, blocks, nc, reinterpret_cast<double2*>(d_out));
    return cuda_ok(cudaGetLastError(), "k_sum_partials") ? 0 : LS_GPU_ERR_CUDA;
  };
  const bool inv = p.group.spin_inversion != 0;
  switch (p.group.gpl) {
    case 1: return inv ? go(k_coupling_products<1, true>) : go(k_coupling_products<1, false>);
    case 2: return inv ? go(k_coupling_products<2, true>) : go(k_coupling_products<2, false>);
    case 3: return inv ? go(k_coupling_products<3, true>) : go(k_coupling_products<3, false>);
    case 4: return inv ? go(k_coupling_products<4, true>) : go(k_coupling_products<4, false>);
    default: return LS_GPU_ERR_INVALID;
  }
}

}  // namespace lsg
