// blockops_tc.cu -- the block eigensolver's tall-skinny products on the fifth-generation tensor
// cores (tcgen05.mma, bf16 operands, FP32 accumulators in tensor memory), to FP64 working
// precision by an error-free fixed-point splitting.
//
//     out[s] = beta W[s] + X1[s] M1[s] + X2[s] M2[s]      (complex, k <= 16 columns)
//
// Method: an error-free splitting in the manner of Ozaki, Ogita, Oishi & Rump (Numer. Algorithms
// 59, 2012) with fixed-point frames as in the integer variant of Ootomo, Ozaki & Yokota (2024),
// evaluated with bf16 digits on FP32-accumulating tensor cores:
//
//  * [X1 | X2] is a real D x K matrix (K = 4 kp reals; kp = 8 or 16 complex columns, zero
//    padded) and [M1; M2] the real K x 2kp matrix with the 2 x 2 block [[Re m, Im m],
//    [-Im m, Re m]] per complex entry m, so that the interleaved (re, im) row of X times it is
//    the interleaved row of X M.
//  * Row r of X gets the frame 2^E_r above its largest magnitude, column c of M the frame 2^E_c.
//    A value v becomes the integer F = trunc(|v| 2^(56 - E)) < 2^56, written as 8 signed
//    base-2^7 digits: v = sign(v) sum_i d_i 2^(E - 7 - 7i), |d_i| <= 128 for i = 0, 3, 6 and
//    <= 64 otherwise; every digit is an exact bf16.
//  * Digit products with i + j = t (t = 0..7) are summed by the tensor cores into accumulator
//    group t.  Every partial sum stays within K * max_t sum_{i+j=t} |d_i| |d_j| <= 64 * 2^16 =
//    2^22, so the FP32 accumulation is exact.
//  * An output's 8 groups are combined in 64-bit integers (Horner in base 2^7, at most 2^62.1;
//    group 7 is truncated to the unit 2^(E_r + E_c - 56)), converted to FP64 by integer
//    instructions (round to nearest even), and beta W is added with one FP64 FMA.
//
// Error per output: the dropped digit products (t >= 8), the truncation of F and of group 7 sum
// to below (K + 2) 2^-54 2^(E_r + E_c), i.e. within the rounding-error bound of an FP64 dot
// product of length K over values of the frames' magnitudes.  Non-finite inputs are not
// supported (the frame of a row or column holding inf or NaN is undefined).
//
// Work division: one persistent CTA of 512 threads (16 warps) per SM walks a contiguous range of
// 128-row tiles (tiles never straddle sectors).  Per tile all warps load the rows (one tile
// ahead, in registers) and write the bf16 digits of A (8 digit planes of 128 x K) into shared
// memory; one thread issues 8 MMAs per K step (plane i against the digit planes j = 0..7-i of M
// at once, N = 2kp (8 - i), into the accumulator columns of groups i..7) and commits them to an
// mbarrier; while those run, the warps combine the previous tile from the other tensor-memory
// buffer (two buffers of 16 kp columns).  Only that thread polls the mbarrier; the others wait at
// the CTA barrier.  M's digit image is built once per call by k_update_tc_prep.  The Gram kernel
// below shares the digit code and the tile loop.
#include "lsg.h"
#include "tc.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

namespace lsg {
namespace {

constexpr int kDigits = 8;
constexpr int kRows = 128;  // rows per tile: the MMA's M
constexpr int kThreads = 512;  // 16 warps: 4 per SM sub-partition
constexpr int kWarps = kThreads / 32;
constexpr int kParts = kThreads / 128;  // epilogue: column parts per lane quarter
constexpr uint32_t kRowCore = 128;      // bytes between core matrices adjacent in rows
constexpr long long kWaitCycles = 4000000000ll;  // about 2 s at GB300 clocks

template <int KP>
struct UpdShape {
  static constexpr int K = 4 * KP;   // reals per row of [X1 | X2]
  static constexpr int NC = 2 * KP;  // real output columns
  static constexpr int G = K / 8;    // 8-real groups per row (one 16-byte core row each)
  // A: 8 digit planes of kRows x K.  Core matrices adjacent in K are 129 * 16 bytes apart, so
  // that the 32 lanes of a producer store (4 or 8 rows x G groups) hit distinct bank quads.
  static constexpr uint32_t a_kstride = 129 * 16;
  static constexpr uint32_t a_plane = G * a_kstride;
  static constexpr uint32_t a_bytes = kDigits * a_plane;
  // B: the digit planes of M stacked in rows: row n = j * NC + c, K columns.
  static constexpr uint32_t b_rows = kDigits * NC;
  static constexpr uint32_t b_kstride = b_rows * 16;
  static constexpr uint32_t b_bytes = G * b_kstride;
  static constexpr uint32_t tmem_cols = 2 * kDigits * NC;  // two accumulator buffers
  static constexpr uint32_t smem = a_bytes + b_bytes;
};

// Raises a kernel's dynamic shared-memory limit once per device (the attribute is per device).
bool smem_attribute_set(const void* kern, uint32_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, uint32_t> done;
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find({kern, dev});
  if (it != done.end() && it->second >= bytes) return true;
  if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
               "cudaFuncSetAttribute(tensor-core block kernel)"))
    return false;
  done[{kern, dev}] = bytes;
  return true;
}

// ---- digits ---------------------------------------------------------------------------------

// The biased FP64 exponent field of v (0 for zeros and subnormals).
__device__ __forceinline__ int exp_field(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }

// 56-bit fixed-point magnitude of v in the frame whose biased exponent is `emax` (>= v's).
__device__ __forceinline__ uint64_t fixed56(double v, int emax) {
  const uint64_t u = (uint64_t)__double_as_longlong(v);
  const int e = (int)((u >> 52) & 0x7ff);
  if (e == 0) return 0;  // zero or subnormal: below every frame's resolution
  const uint64_t m = ((u & 0xfffffffffffffull) | (1ull << 52)) << 3;
  const int d = emax - e;
  return d < 56 ? m >> d : 0;
}

// The 8 digits of sign * F as bf16 bit patterns in the upper halves of 32-bit words.
__device__ __forceinline__ void digits8(uint64_t F, bool neg, uint32_t (&b)[kDigits]) {
  const float R = 12582912.0f;  // 1.5 * 2^23: fmaf(x, s, R) - R rounds x * s to an integer
  const float sg = neg ? -1.0f : 1.0f;
  const float off = neg ? 8388608.0f : -8388608.0f;
  const uint32_t chunk[3] = {(uint32_t)(F >> 35), (uint32_t)(F >> 14) & 0x1fffffu, (uint32_t)F & 0x3fffu};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // y = sign * chunk, exactly (chunk < 2^21)
    const float y = __fmaf_rn(__uint_as_float(0x4b000000u | chunk[c]), sg, off);
    if (c < 2) {  // 21 bits: y = d0 2^14 + d1 2^7 + d2
      const float d0 = __fsub_rn(__fmaf_rn(y, 0x1p-14f, R), R);
      const float r = __fmaf_rn(-d0, 16384.0f, y);
      const float d1 = __fsub_rn(__fmaf_rn(r, 0x1p-7f, R), R);
      const float d2 = __fmaf_rn(-d1, 128.0f, r);
      b[3 * c] = __float_as_uint(d0);
      b[3 * c + 1] = __float_as_uint(d1);
      b[3 * c + 2] = __float_as_uint(d2);
    } else {  // 14 bits: y = d6 2^7 + d7
      const float d6 = __fsub_rn(__fmaf_rn(y, 0x1p-7f, R), R);
      b[6] = __float_as_uint(d6);
      b[7] = __float_as_uint(__fmaf_rn(-d6, 128.0f, y));
    }
  }
}

// sign * H * 2^(scale), H a non-negative-magnitude 64-bit integer (|H| < 2^63), rounded to the
// nearest FP64 (ties to even), by integer instructions.
__device__ __forceinline__ double int64_scaled_to_double(long long H, int scale) {
  if (H == 0) return 0.0;
  const bool neg = H < 0;
  const uint64_t a = neg ? (uint64_t)(-H) : (uint64_t)H;
  const int lz = __clzll((long long)a);
  const uint64_t n = a << lz;  // leading one at bit 63
  uint64_t mant = n >> 11;     // 53 bits
  const uint32_t rem = (uint32_t)n & 0x7ffu;
  mant += (rem > 0x400u || (rem == 0x400u && (mant & 1))) ? 1 : 0;
  const int be = 63 - lz + scale + 1023;  // biased exponent of the leading bit
  uint64_t bits;
  if (be <= 0) bits = 0;                                   // below the normal range: flush
  else if (be >= 2047) bits = 0x7ff0000000000000ull;       // overflow
  else bits = ((uint64_t)(be - 1) << 52) + mant;           // a rounding carry bumps the exponent
  return __longlong_as_double((long long)(bits | (neg ? 0x8000000000000000ull : 0)));
}

// ---- M's digit image --------------------------------------------------------------------------

// One CTA per sector: the real K x NC matrix of [M1; M2], its column frames (biased exponents,
// written to col_exp[s][c]) and the digit planes in the B layout (written to image[s]).
template <int KP>
__global__ void __launch_bounds__(kThreads) k_update_tc_prep(int k, const double2* __restrict__ M1,
                                                              const double2* __restrict__ M2,
                                                              uint8_t* __restrict__ image,
                                                              int* __restrict__ col_exp) {
  using Sh = UpdShape<KP>;
  __shared__ int cmax[Sh::NC];
  const int s = blockIdx.x;
  const int tid = threadIdx.x;
  const size_t kk2 = (size_t)k * k;
  auto entry = [&](int kr, int c) -> double {
    const double2* M = kr < 2 * KP ? M1 : M2;
    const int i = (kr % (2 * KP)) >> 1, ri = kr & 1;
    const int j = c >> 1, rc = c & 1;
    if (M == nullptr || i >= k || j >= k) return 0.0;
    const double2 m = M[(size_t)s * kk2 + (size_t)i * k + j];
    // [[Re, Im], [-Im, Re]]
    return ri == 0 ? (rc == 0 ? m.x : m.y) : (rc == 0 ? -m.y : m.x);
  };
  if (tid < Sh::NC) cmax[tid] = 0;
  __syncthreads();
  for (int e = tid; e < Sh::K * Sh::NC; e += kThreads) atomicMax(&cmax[e % Sh::NC], exp_field(entry(e / Sh::NC, e % Sh::NC)));
  __syncthreads();
  uint8_t* img = image + (size_t)s * Sh::b_bytes;
  for (int e = tid; e < Sh::K * Sh::NC; e += kThreads) {
    const int kr = e / Sh::NC, c = e % Sh::NC;
    const double v = entry(kr, c);
    uint32_t b[kDigits];
    digits8(fixed56(v, cmax[c]), v < 0.0, b);
#pragma unroll
    for (int j = 0; j < kDigits; ++j)
      *reinterpret_cast<uint16_t*>(img + tc::kmajor_offset(j * Sh::NC + c, kr, Sh::b_kstride, kRowCore)) =
          (uint16_t)(b[j] >> 16);
  }
  if (tid < Sh::NC) col_exp[(size_t)s * Sh::NC + tid] = cmax[tid];
}

// ---- the product kernel -----------------------------------------------------------------------

// TWO: two terms (X1 M1 + X2 M2, K = 4 kp reals per row of A); one term uses the first 2 kp reals
// only (half the digits and MMAs).
template <int KP, bool TWO>
struct UpdTile {
  static constexpr int G = TWO ? UpdShape<KP>::G : UpdShape<KP>::G / 2;  // 8-real groups per row
  static constexpr int RPW = 32 / G;                                      // rows per warp and pass
  static constexpr int PASSES = (kRows * G + kThreads - 1) / kThreads;    // 2 or 1
  double2 v[PASSES][4];                                                   // 8 reals per pass
};

template <int KP, bool TWO>
__device__ __forceinline__ void update_load(UpdTile<KP, TWO>& t, int64_t tile_row0, int64_t D, int k,
                                            int64_t sec_base, const double2* X1, const double2* X2) {
  using T = UpdTile<KP, TWO>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane % T::G;
  const double2* X = (TWO && g >= T::G / 2) ? X2 : X1;
  const int c0 = (TWO ? g % (T::G / 2) : g) * 4;
#pragma unroll
  for (int p = 0; p < T::PASSES; ++p) {
    const int r = (p * kWarps + warp) * T::RPW + lane / T::G;
    const int64_t row = tile_row0 + r;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool in = r < kRows && row < D && c0 + q < k;
      t.v[p][q] = in ? X[(sec_base + row) * k + c0 + q] : make_double2(0.0, 0.0);
    }
  }
}

template <int KP, bool TWO>
__device__ __forceinline__ void update_produce(const UpdTile<KP, TWO>& t, uint8_t* A, int* rowexp) {
  using Sh = UpdShape<KP>;
  using T = UpdTile<KP, TWO>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane % T::G;
#pragma unroll
  for (int p = 0; p < T::PASSES; ++p) {
    const int r = (p * kWarps + warp) * T::RPW + lane / T::G;
    if ((p * kWarps + warp) * T::RPW >= kRows) break;  // this warp has no rows left (warp-uniform)
    int e = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) e = max(e, max(exp_field(t.v[p][q].x), exp_field(t.v[p][q].y)));
#pragma unroll
    for (int o = 1; o < T::G; o <<= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if (g == 0) rowexp[r] = e;
    uint32_t w[kDigits][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t br[kDigits], bi[kDigits];
      // signs from the high words (integer test: no FP64 comparison)
      digits8(fixed56(t.v[p][q].x, e), __double2hiint(t.v[p][q].x) < 0, br);
      digits8(fixed56(t.v[p][q].y, e), __double2hiint(t.v[p][q].y) < 0, bi);
#pragma unroll
      for (int j = 0; j < kDigits; ++j) w[j][q] = __byte_perm(br[j], bi[j], 0x7632);
    }
    const uint32_t off = (uint32_t)g * Sh::a_kstride + (uint32_t)(r >> 3) * kRowCore + (uint32_t)(r & 7) * 16;
#pragma unroll
    for (int j = 0; j < kDigits; ++j)
      *reinterpret_cast<uint4*>(A + j * Sh::a_plane + off) = make_uint4(w[j][0], w[j][1], w[j][2], w[j][3]);
  }
}

// Combines the accumulator groups of one finished tile and writes its rows.  Warp w reads lane
// quarter w % 4 (rows 32 (w % 4) ..) and real columns [(w / 4) KP, (w / 4 + 1) KP).
template <int KP>
__device__ __forceinline__ void update_epilogue(uint32_t tmem_buf, const int* rowexp, const int* colexp,
                                                int64_t tile_row0, int64_t D, int k, int64_t sec_base, double beta,
                                                const double2* W, double2* out) {
  using Sh = UpdShape<KP>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int quarter = warp & 3, part = warp >> 2;
  constexpr int RC = Sh::NC / kParts;  // real columns of this thread
  constexpr int KC = RC / 2;           // complex columns
  const int r = quarter * 32 + lane;
  const int64_t row = tile_row0 + r;
  const uint32_t taddr = tmem_buf + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(part * RC);
  // W's part of this row first, so that its latency overlaps the tensor-memory loads and the
  // integer combination
  const int j0 = part * KC;
  const bool live = row < D;
  double2 w[KC];
#pragma unroll
  for (int c = 0; c < KC; ++c)
    w[c] = (beta != 0.0 && live && j0 + c < k) ? W[(sec_base + row) * k + j0 + c] : make_double2(0.0, 0.0);
  long long H[RC];
  uint32_t a[kDigits][RC];
  // all groups in flight at once, one wait
#pragma unroll
  for (int t = 0; t < kDigits; ++t) tc::tmem_ld<RC>(taddr + t * Sh::NC, a[t]);
  tc::tmem_ld_wait();
  // groups 0 .. 6: Horner in base 2^7
#pragma unroll
  for (int t = 0; t < kDigits; ++t) {
#pragma unroll
    for (int c = 0; c < RC; ++c) {
      // |group sum| <= 2^22: adding 1.5 * 2^23 puts the integer in the low mantissa bits (FP32
      // pipe, exact), instead of a float-to-integer conversion
      const long long g = (long long)(__float_as_int(__fadd_rn(__uint_as_float(a[t][c]), 12582912.0f)) - 0x4b400000);
      if (t == 0) H[c] = g;
      else if (t < kDigits - 1) H[c] = H[c] * 128 + g;
      else H[c] += g >> 7;  // group 7, truncated to the unit of group 6
    }
  }
  if (!live) return;
  const int er = rowexp[r];
  double2* orow = out + (sec_base + row) * k;
#pragma unroll
  for (int c = 0; c < KC; ++c) {
    const int j = j0 + c;  // complex column
    if (j >= k) break;
    double re = int64_scaled_to_double(H[2 * c], er + colexp[2 * j] - 2100);
    double im = int64_scaled_to_double(H[2 * c + 1], er + colexp[2 * j + 1] - 2100);
    if (beta != 0.0) {
      re = fma(beta, w[c].x, re);
      im = fma(beta, w[c].y, im);
    }
    orow[j] = make_double2(re, im);
  }
}

template <int KP, bool TWO>
__global__ void __launch_bounds__(kThreads, 1)
    k_block_update_tc(int64_t D, int k, int64_t tiles_per_sector, int64_t total_tiles, double beta,
                      const double2* W, const double2* X1, const double2* X2, const uint8_t* __restrict__ image,
                      const int* __restrict__ col_exp, double2* out, int* err) {
  using Sh = UpdShape<KP>;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* A = smem;
  uint8_t* B = smem + Sh::a_bytes;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int rowexp[2][kRows];
  __shared__ int colexp[2][Sh::NC];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t t_begin = (int64_t)blockIdx.x * total_tiles / gridDim.x;
  const int64_t t_end = (int64_t)(blockIdx.x + 1) * total_tiles / gridDim.x;
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_u32(&tmem_slot), Sh::tmem_cols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_u32(&mbar[0]), 1);
    tc::mbar_init(tc::smem_u32(&mbar[1]), 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
  int64_t loaded_sector = -1;
  int64_t prev_row0 = 0, prev_base = 0;
  bool failed = false;
  UpdTile<KP, TWO> regs;
  if (t_begin < t_end) {
    const int64_t s = t_begin / tiles_per_sector;
    update_load<KP, TWO>(regs, (t_begin % tiles_per_sector) * kRows, D, k, s * D, X1, X2);
  }
  for (int64_t tile = t_begin; tile < t_end; ++tile) {
    const int it = (int)(tile - t_begin);
    const int buf = it & 1;
    const int64_t s = tile / tiles_per_sector;
    const int64_t row0 = (tile % tiles_per_sector) * kRows;
    if (it >= 1) {
      // the previous tile's MMAs are done (A and B free, its accumulators final) and every
      // thread has finished the epilogue before it (rowexp / colexp of this buffer free)
      const bool ok = tid != 0 || tc::mbar_wait(tc::smem_u32(&mbar[buf ^ 1]), ((it - 1) >> 1) & 1, kWaitCycles);
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
    }
    if (s != loaded_sector) {
      const uint4* src = reinterpret_cast<const uint4*>(image + (size_t)s * Sh::b_bytes);
      for (uint32_t e = tid; e < Sh::b_bytes / 16; e += kThreads) reinterpret_cast<uint4*>(B)[e] = src[e];
      loaded_sector = s;
    }
    if (tid < Sh::NC) colexp[buf][tid] = col_exp[s * Sh::NC + tid];
    update_produce<KP, TWO>(regs, A, rowexp[buf]);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint64_t ad0 = tc::smem_desc(a0, Sh::a_kstride, kRowCore);
      const uint64_t bd0 = tc::smem_desc(b0, Sh::b_kstride, kRowCore);
      const uint32_t d0 = tmem + buf * (kDigits * Sh::NC);
#pragma unroll
      for (int i = 0; i < kDigits; ++i) {
#pragma unroll
        for (int ks = 0; ks < (TWO ? Sh::K : Sh::K / 2) / 16; ++ks) {
          // start addresses advance in the descriptors' low field (units of 16 bytes)
          tc::mma_bf16(d0 + i * Sh::NC, ad0 + ((i * Sh::a_plane + ks * 2 * Sh::a_kstride) >> 4),
                       bd0 + ((ks * 2 * Sh::b_kstride) >> 4), tc::idesc_bf16_f32(kRows, Sh::NC * (kDigits - i)),
                       (i > 0 || ks > 0) ? 1u : 0u);
        }
      }
      tc::commit(tc::smem_u32(&mbar[buf]));
    }
    if (tile + 1 < t_end) {
      const int64_t sn = (tile + 1) / tiles_per_sector;
      update_load<KP, TWO>(regs, ((tile + 1) % tiles_per_sector) * kRows, D, k, sn * D, X1, X2);
    }
    if (it >= 1)
      update_epilogue<KP>(tmem + (buf ^ 1) * (kDigits * Sh::NC), rowexp[buf ^ 1], colexp[buf ^ 1], prev_row0, D, k,
                          prev_base, beta, W, out);
    tc::fence_before_sync();
    prev_row0 = row0;
    prev_base = s * D;
  }
  const int n = (int)(t_end - t_begin);
  if (!failed && n >= 1) {
    const int lb = (n - 1) & 1;
    const bool ok = tid != 0 || tc::mbar_wait(tc::smem_u32(&mbar[lb]), ((n - 1) >> 1) & 1, kWaitCycles);
    if (__syncthreads_or(!ok)) {
      failed = true;
    } else {
      tc::fence_after_sync();
      update_epilogue<KP>(tmem + lb * (kDigits * Sh::NC), rowexp[lb], colexp[lb], prev_row0, D, k, prev_base, beta,
                          W, out);
    }
  }
  if (failed && threadIdx.x == 0) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, Sh::tmem_cols);
}

template <int KP>
int run_update_tc(int64_t S, int64_t D, int k, double beta, const double* d_w, const double* d_x1,
                  const double* d_m1, const double* d_x2, const double* d_m2, double* d_out, cudaStream_t st) {
  using Sh = UpdShape<KP>;
  const bool two = d_x2 != nullptr;
  const void* kern = two ? (const void*)k_block_update_tc<KP, true> : (const void*)k_block_update_tc<KP, false>;
  if (!smem_attribute_set(kern, Sh::smem)) return LS_GPU_ERR_CUDA;
  const int64_t tiles_per_sector = (D + kRows - 1) / kRows;
  const int64_t total = S * tiles_per_sector;
  const int grid = (int)std::min<int64_t>(total, (int64_t)num_sms());
  uint8_t* image = nullptr;
  const size_t img_bytes = (size_t)S * Sh::b_bytes;
  const size_t ce_bytes = (size_t)S * Sh::NC * sizeof(int);
  if (!cuda_ok(cudaMallocAsync((void**)&image, img_bytes + ce_bytes, st), "cudaMallocAsync(update digits)"))
    return LS_GPU_ERR_CUDA;
  int* col_exp = reinterpret_cast<int*>(image + img_bytes);
  // a timed-out wait is reported through the shared device error word (read after the next
  // matvec or by ls_gpu_check_device_errors), so that the call stays graph-capturable
  int* err = device_error_word() + 1;
  bool ok = true;
  {
    k_update_tc_prep<KP><<<(unsigned)S, kThreads, 0, st>>>(k, reinterpret_cast<const double2*>(d_m1),
                                                           reinterpret_cast<const double2*>(d_m2), image, col_exp);
    ok = cuda_ok(cudaGetLastError(), "k_update_tc_prep");
  }
  if (ok) {
    if (two)
      k_block_update_tc<KP, true><<<grid, kThreads, Sh::smem, st>>>(
          D, k, tiles_per_sector, total, beta, reinterpret_cast<const double2*>(d_w),
          reinterpret_cast<const double2*>(d_x1), reinterpret_cast<const double2*>(d_x2), image, col_exp,
          reinterpret_cast<double2*>(d_out), err);
    else
      k_block_update_tc<KP, false><<<grid, kThreads, Sh::smem, st>>>(
          D, k, tiles_per_sector, total, beta, reinterpret_cast<const double2*>(d_w),
          reinterpret_cast<const double2*>(d_x1), nullptr, image, col_exp, reinterpret_cast<double2*>(d_out), err);
    ok = cuda_ok(cudaGetLastError(), "k_block_update_tc");
  }
  ok = cuda_ok(cudaFreeAsync(image, st), "cudaFreeAsync(update digits)") && ok;
  return ok ? 0 : LS_GPU_ERR_CUDA;
}

// ---- the Gram kernel --------------------------------------------------------------------------
//
//     G[s] = X[s]^H Y[s]      (the contraction runs over the D rows)
//
// A tile of 128 rows is the K extent of one round of MMAs (8 K steps of 16 rows).  Every complex
// column of X and of Y gets a frame over the tile's rows (its re and im parts share it, so that
// the complex combination stays exact), and the digit planes are written transposed: element
// (plane * NR + c, row) of a K-major operand, NR = 2 kp real columns.  One MMA with M = 128 covers
// Q = 128 / NR consecutive planes a .. a + Q - 1 of X (lane block q = plane a + q; planes below 0
// are zero planes stacked in front) and two planes j, j + 1 of Y (N = 2 NR).  Its first column
// block then holds digit pairs of weight t = a + j + q, its second t = a + j + 1 + q.  With
// MMAs (a = s - j, j) for s in {0, Q, ..} and even j, the two column blocks of region s are the
// weights t = s + q (even j) and t = s + q + 1 (odd j) of lane block q, and every digit pair
// (i, j) lands in exactly one cell.  A cell sums at most 4 pairs x 128 rows of digit products,
// |cell| <= 2^23 (exact in FP32).  After a tile the epilogue joins a lane's cells into one 64-bit
// integer per column (weights t = q .. q + 5 span 35 bits above a 2^23 cell: below 2^58),
// converts it to FP64 with the tile's frames and adds it to per-thread FP64 sums; at the end of a
// sector's rows the sums are reduced over lane blocks and complex pairs into this CTA's partial
// Gram, and the partials are added over CTAs in a fixed order by a second kernel (deterministic).

template <int KP>
struct GramShape {
  static constexpr int NR = 2 * KP;        // real columns
  static constexpr int Q = kRows / NR;     // X digit planes per MMA: 4 (kp = 16) or 8 (kp = 8)
  static constexpr int REG = kDigits / Q;  // accumulator regions (pairs of column blocks): 2 or 1
  static constexpr int Z = Q == 4 ? 2 : 6; // zero planes in front of X's planes (lowest a = -Z)
  static constexpr int x_rows = (Z + kDigits) * NR;
  static constexpr int y_rows = kDigits * NR;
  static constexpr uint32_t x_kstride = x_rows * 16;
  static constexpr uint32_t y_kstride = y_rows * 16;
  static constexpr uint32_t x_bytes = (kRows / 8) * x_kstride;
  static constexpr uint32_t y_bytes = (kRows / 8) * y_kstride;
  static constexpr uint32_t p_bytes = kRows * NR * 8;  // flush buffer: 128 lanes x NR doubles
  static constexpr uint32_t smem = x_bytes + y_bytes + p_bytes;
  static constexpr uint32_t buf_cols = REG * 2 * NR;   // tensor-memory columns per tile
  static constexpr uint32_t tmem_cols = 2 * buf_cols < 32 ? 32 : 2 * buf_cols;
  static constexpr int units = NR * (kRows / 8);       // (column, 8-row group) units per operand
  static constexpr int PASSES = 2 * units / kThreads;  // units of X and Y per thread
  static constexpr int DC = NR / kParts;               // epilogue: columns of Y per thread
  static constexpr int TOP = (REG - 1) * Q + 1;        // a lane's highest weight offset
};

template <int KP>
struct GramTile {
  double v[GramShape<KP>::PASSES][8];
};

template <int KP>
__device__ __forceinline__ void gram_load(GramTile<KP>& t, int64_t row0, int64_t D, int k, int64_t sec_base,
                                          const double* X, const double* Y, bool same) {
  using Sh = GramShape<KP>;
#pragma unroll
  for (int p = 0; p < Sh::PASSES; ++p) {
    const int u = threadIdx.x + p * kThreads;
    const int which = u / Sh::units, v = u % Sh::units;
    const int c = v % Sh::NR, g = v / Sh::NR;
    const double* P = which == 0 ? X : Y;
    const bool active = !(same && which == 1) && c < 2 * k;
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const int64_t row = row0 + 8 * g + rr;
      t.v[p][rr] = (active && row < D) ? P[((sec_base + row) * k) * 2 + c] : 0.0;
    }
  }
}

// Frames (per complex column, into colmax[2][16] by atomicMax), then the digit planes.
template <int KP>
__device__ __forceinline__ void gram_produce(const GramTile<KP>& t, uint8_t* XD, uint8_t* YD, int (*colmax)[16],
                                             bool same) {
  using Sh = GramShape<KP>;
#pragma unroll
  for (int p = 0; p < Sh::PASSES; ++p) {
    const int u = threadIdx.x + p * kThreads;
    const int which = u / Sh::units, c = (u % Sh::units) % Sh::NR;
    int e = 0;
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) e = max(e, exp_field(t.v[p][rr]));
    e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));  // re and im of one complex column
    if (!(same && which == 1) && (c & 1) == 0 && e > 0) atomicMax(&colmax[which][c >> 1], e);
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < Sh::PASSES; ++p) {
    const int u = threadIdx.x + p * kThreads;
    const int which = u / Sh::units, v = u % Sh::units;
    const int c = v % Sh::NR, g = v / Sh::NR;
    if (same && which == 1) continue;
    const int e = colmax[which][c >> 1];
    uint32_t w[kDigits][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t b0[kDigits], b1[kDigits];
      const double x0 = t.v[p][2 * q], x1 = t.v[p][2 * q + 1];
      digits8(fixed56(x0, e), __double2hiint(x0) < 0, b0);
      digits8(fixed56(x1, e), __double2hiint(x1) < 0, b1);
#pragma unroll
      for (int j = 0; j < kDigits; ++j) w[j][q] = __byte_perm(b0[j], b1[j], 0x7632);
    }
    uint8_t* base = which == 0 ? XD : YD;
    const uint32_t ks = which == 0 ? Sh::x_kstride : Sh::y_kstride;
    const int plane0 = which == 0 ? Sh::Z : 0;
#pragma unroll
    for (int j = 0; j < kDigits; ++j) {
      const int m = (plane0 + j) * Sh::NR + c;
      *reinterpret_cast<uint4*>(base + g * ks + (m >> 3) * kRowCore + (m & 7) * 16) =
          make_uint4(w[j][0], w[j][1], w[j][2], w[j][3]);
    }
  }
}

// Adds one finished tile to the per-thread FP64 sums acc[d] (this thread: lane (quarter, lane),
// i.e. lane block q = lane / NR and column c = lane % NR of X; columns d of Y in its part).
template <int KP>
__device__ __forceinline__ void gram_epilogue(uint32_t tmem_buf, const int (*colmax)[16], bool same,
                                              double (&acc)[GramShape<KP>::DC]) {
  using Sh = GramShape<KP>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int quarter = warp & 3, part = warp >> 2;
  const int l = quarter * 32 + lane;
  const int q = l / Sh::NR, c = l % Sh::NR;
  const uint32_t taddr = tmem_buf + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(part * Sh::DC);
  uint32_t cell[Sh::REG][2][Sh::DC];
#pragma unroll
  for (int r = 0; r < Sh::REG; ++r)
#pragma unroll
    for (int b = 0; b < 2; ++b) tc::tmem_ld<Sh::DC>(taddr + (r * 2 + b) * Sh::NR, cell[r][b]);
  tc::tmem_ld_wait();
  const int ec = colmax[0][c >> 1];
  const int* ey = colmax[same ? 0 : 1];
#pragma unroll
  for (int dd = 0; dd < Sh::DC; ++dd) {
    // weights t = r Q + b + q; unit = the weight of t = q + TOP
    long long v = 0;
#pragma unroll
    for (int r = 0; r < Sh::REG; ++r) {
      if (r > 0) v *= 1ll << (7 * (Sh::Q - 1));
#pragma unroll
      for (int b = 0; b < 2; ++b) v = v * (b == 0 ? 1ll : 128ll) + (long long)__float2int_rn(__uint_as_float(cell[r][b][dd]));
    }
    const int ed = ey[(part * Sh::DC + dd) >> 1];
    // v counts units of 2^(E_c + E_d - 14 - 7 (q + TOP)), E = biased exponent - 1022
    acc[dd] += int64_scaled_to_double(v, ec + ed - 2058 - 7 * (q + Sh::TOP));
  }
}

// Reduces the per-thread sums over lane blocks and complex pairs into partial[s][blockIdx.x]
// (k x k complex), then clears them.
template <int KP>
__device__ __forceinline__ void gram_flush(double (&acc)[GramShape<KP>::DC], double* P, int k, int64_t s,
                                           double2* partial) {
  using Sh = GramShape<KP>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int quarter = warp & 3, part = warp >> 2;
  const int l = quarter * 32 + lane;
#pragma unroll
  for (int dd = 0; dd < Sh::DC; ++dd) {
    P[l * Sh::NR + part * Sh::DC + dd] = acc[dd];
    acc[dd] = 0.0;
  }
  __syncthreads();
  const int nout = k * k;
  for (int o = threadIdx.x; o < nout; o += kThreads) {
    const int a = o / k, b = o % k;
    double re = 0.0, im = 0.0;
    for (int q = 0; q < Sh::Q; ++q) {
      const double* Pq = P + (size_t)q * Sh::NR * Sh::NR;
      // conj(x) y = (xr yr + xi yi) + i (xr yi - xi yr)
      re += Pq[(2 * a) * Sh::NR + 2 * b] + Pq[(2 * a + 1) * Sh::NR + 2 * b + 1];
      im += Pq[(2 * a) * Sh::NR + 2 * b + 1] - Pq[(2 * a + 1) * Sh::NR + 2 * b];
    }
    partial[((size_t)s * gridDim.x + blockIdx.x) * nout + o] = make_double2(re, im);
  }
  __syncthreads();
}

template <int KP>
__global__ void __launch_bounds__(kThreads, 1)
    k_block_gram_tc(int64_t D, int k, int64_t tiles_per_sector, int64_t total_tiles, const double* X,
                    const double* Y, bool same, double2* partial, int* err) {
  using Sh = GramShape<KP>;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* XD = smem;
  uint8_t* YD = smem + Sh::x_bytes;
  double* P = reinterpret_cast<double*>(smem + Sh::x_bytes + Sh::y_bytes);
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int colmax[3][2][16];  // frames of three tiles in flight (reset one tile ahead)
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t t_begin = (int64_t)blockIdx.x * total_tiles / gridDim.x;
  const int64_t t_end = (int64_t)(blockIdx.x + 1) * total_tiles / gridDim.x;
  // zero planes of X (never written again)
  for (uint32_t g = 0; g < kRows / 8; ++g)
    for (uint32_t e = tid; e < (uint32_t)(Sh::Z * Sh::NR * 16 / 16); e += kThreads)
      reinterpret_cast<uint4*>(XD + g * Sh::x_kstride)[e] = make_uint4(0, 0, 0, 0);
  if (tid < 3 * 2 * 16) (&colmax[0][0][0])[tid] = 0;
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_u32(&tmem_slot), Sh::tmem_cols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_u32(&mbar[0]), 1);
    tc::mbar_init(tc::smem_u32(&mbar[1]), 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t x0 = tc::smem_u32(XD), y0 = same ? x0 + (Sh::Z * Sh::NR / 8) * kRowCore : tc::smem_u32(YD);
  const uint32_t yks = same ? Sh::x_kstride : Sh::y_kstride;
  double acc[Sh::DC];
#pragma unroll
  for (int dd = 0; dd < Sh::DC; ++dd) acc[dd] = 0.0;
  bool failed = false;
  GramTile<KP> regs;
  if (t_begin < t_end)
    gram_load<KP>(regs, (t_begin % tiles_per_sector) * kRows, D, k, (t_begin / tiles_per_sector) * D, X, Y, same);
  for (int64_t tile = t_begin; tile < t_end; ++tile) {
    const int it = (int)(tile - t_begin);
    const int buf = it & 1;
    const int64_t s = tile / tiles_per_sector;
    if (it >= 1) {
      const bool ok = tid != 0 || tc::mbar_wait(tc::smem_u32(&mbar[buf ^ 1]), ((it - 1) >> 1) & 1, kWaitCycles);
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      tc::fence_after_sync();
    }
    gram_produce<KP>(regs, XD, YD, colmax[it % 3], same);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t d0 = tmem + buf * Sh::buf_cols;
      const uint64_t ad0 = tc::smem_desc(x0, Sh::x_kstride, kRowCore);
      const uint64_t bd0 = tc::smem_desc(y0, yks, kRowCore);
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kRows, 2 * Sh::NR);
#pragma unroll
      for (int ks = 0; ks < kRows / 16; ++ks) {
#pragma unroll
        for (int r = 0; r < Sh::REG; ++r) {
#pragma unroll
          for (int j = 0; j < kDigits; j += 2) {
            const int a = r * Sh::Q - j;  // lowest X plane of this MMA
            if (a + Sh::Q - 1 < 0) continue;  // only zero planes
            // start addresses advance in the descriptors' low field (units of 16 bytes)
            const uint32_t arow = (uint32_t)(Sh::Z + a) * Sh::NR;
            tc::mma_bf16(d0 + r * 2 * Sh::NR, ad0 + (((arow / 8) * kRowCore + ks * 2 * Sh::x_kstride) >> 4),
                         bd0 + (((uint32_t)(j * Sh::NR / 8) * kRowCore + ks * 2 * yks) >> 4), idesc,
                         (ks > 0 || j > 0) ? 1u : 0u);
          }
        }
      }
      tc::commit(tc::smem_u32(&mbar[buf]));
    }
    if (tid < 2 * 16) (&colmax[(it + 1) % 3][0][0])[tid] = 0;  // frames of the next tile
    if (tile + 1 < t_end)
      gram_load<KP>(regs, ((tile + 1) % tiles_per_sector) * kRows, D, k, ((tile + 1) / tiles_per_sector) * D, X, Y,
                    same);
    if (it >= 1) {
      gram_epilogue<KP>(tmem + (buf ^ 1) * Sh::buf_cols, colmax[(it - 1) % 3], same, acc);
      if ((tile - 1) / tiles_per_sector != s) gram_flush<KP>(acc, P, k, (tile - 1) / tiles_per_sector, partial);
    }
    tc::fence_before_sync();
  }
  const int n = (int)(t_end - t_begin);
  if (!failed && n >= 1) {
    const int lb = (n - 1) & 1;
    const bool ok = tid != 0 || tc::mbar_wait(tc::smem_u32(&mbar[lb]), ((n - 1) >> 1) & 1, kWaitCycles);
    if (__syncthreads_or(!ok)) {
      failed = true;
    } else {
      tc::fence_after_sync();
      gram_epilogue<KP>(tmem + lb * Sh::buf_cols, colmax[(n - 1) % 3], same, acc);
      gram_flush<KP>(acc, P, k, (t_end - 1) / tiles_per_sector, partial);
    }
  }
  if (failed && threadIdx.x == 0) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, Sh::tmem_cols);
}

template <int KP>
int run_gram_tc(int64_t S, int64_t D, int k, const double* d_x, const double* d_y, double* d_g, cudaStream_t st) {
  using Sh = GramShape<KP>;
  if (!smem_attribute_set((const void*)k_block_gram_tc<KP>, Sh::smem)) return LS_GPU_ERR_CUDA;
  const int64_t tiles_per_sector = (D + kRows - 1) / kRows;
  const int64_t total = S * tiles_per_sector;
  const int grid = (int)std::min<int64_t>(total, (int64_t)num_sms());
  const int nout = k * k;
  const size_t pbytes = (size_t)S * grid * nout * sizeof(double2);
  double2* partial = nullptr;
  if (!cuda_ok(cudaMallocAsync((void**)&partial, pbytes, st), "cudaMallocAsync(Gram partials)")) return LS_GPU_ERR_CUDA;
  // a CTA writes the partials of the sectors its rows touch; the others stay zero
  bool ok = cuda_ok(cudaMemsetAsync(partial, 0, pbytes, st), "cudaMemsetAsync(Gram partials)");
  if (ok) {
    k_block_gram_tc<KP><<<grid, kThreads, Sh::smem, st>>>(D, k, tiles_per_sector, total, d_x, d_y, d_x == d_y,
                                                          partial, device_error_word() + 1);
    ok = cuda_ok(cudaGetLastError(), "k_block_gram_tc");
  }
  if (ok) ok = launch_gram_partial_sum(partial, grid, nout, S, reinterpret_cast<double2*>(d_g), st) == 0;
  ok = cuda_ok(cudaFreeAsync(partial, st), "cudaFreeAsync(Gram partials)") && ok;
  return ok ? 0 : LS_GPU_ERR_CUDA;
}

}  // namespace

int launch_block_update_tc(int64_t S, int64_t D, int k, double beta, const double* d_w, const double* d_x1,
                           const double* d_m1, const double* d_x2, const double* d_m2, double* d_out,
                           cudaStream_t s) {
  if (S < 1 || S > 65535 || D < 0 || k < 1 || k > 16)
    return fail(LS_GPU_ERR_INVALID, "block update: need 1 <= S <= 65535, D >= 0, 1 <= k <= 16");
  if (D == 0) return 0;
  if (d_out == nullptr || d_x1 == nullptr || d_m1 == nullptr || (beta != 0.0 && d_w == nullptr) ||
      ((d_x2 == nullptr) != (d_m2 == nullptr)))
    return fail(LS_GPU_ERR_INVALID, "block update: NULL pointer");
  StageScope stage("lanczos.update", s);
  return k <= 8 ? run_update_tc<8>(S, D, k, beta, d_w, d_x1, d_m1, d_x2, d_m2, d_out, s)
                : run_update_tc<16>(S, D, k, beta, d_w, d_x1, d_m1, d_x2, d_m2, d_out, s);
}

int launch_block_gram_tc(int64_t S, int64_t D, int k, const double* d_x, const double* d_y, double* d_g,
                         cudaStream_t s) {
  if (S < 1 || S > 65535 || D < 0 || k < 1 || k > 16)
    return fail(LS_GPU_ERR_INVALID, "block Gram: need 1 <= S <= 65535, D >= 0, 1 <= k <= 16");
  if (d_g == nullptr || (D > 0 && (d_x == nullptr || d_y == nullptr)))
    return fail(LS_GPU_ERR_INVALID, "block Gram: NULL pointer");
  if (D == 0)
    return cuda_ok(cudaMemsetAsync(d_g, 0, (size_t)S * k * k * 16, s), "block Gram (empty)") ? 0 : LS_GPU_ERR_CUDA;
  StageScope stage("lanczos.gram", s);
  return k <= 8 ? run_gram_tc<8>(S, D, k, d_x, d_y, d_g, s) : run_gram_tc<16>(S, D, k, d_x, d_y, d_g, s);
}

}  // namespace lsg

extern "C" int ls_gpu_block_gram_tc(int64_t S, int64_t D, int k, double const* d_x, double const* d_y, double* d_g,
                                    void* stream) {
  return lsg::launch_block_gram_tc(S, D, k, d_x, d_y, d_g, (cudaStream_t)stream);
}

extern "C" int ls_gpu_block_update_tc(int64_t S, int64_t D, int k, double beta, double const* d_w,
                                      double const* d_x1, double const* d_m1, double const* d_x2,
                                      double const* d_m2, double* d_out, void* stream) {
  return lsg::launch_block_update_tc(S, D, k, beta, d_w, d_x1, d_m1, d_x2, d_m2, d_out, (cudaStream_t)stream);
}
