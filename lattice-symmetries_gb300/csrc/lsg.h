// lsg.h -- internal declarations shared by the CUDA kernels and the C-ABI layer of
// libls_gb300.so.  Nothing here is part of the public ABI (see include/ls_gb300.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ls_gb300.h"
#include "trace.h"

namespace lsg {

constexpr int kMaxGroupElements = 2048;  // |G| handled by the device orbit scan
constexpr int kWarp = 32;

// Device view of a permutation group (all pointers are device memory).
struct DeviceGroup {
  int n_bits = 0;          // bits of a basis state
  int n_elems = 0;         // |G| (0: spin inversion only / no projection)
  int depth = 0;           // Benes stages
  int spin_inversion = 0;  // 0, +1, -1
  uint64_t flip = 0;       // all n_bits set
  const uint64_t* masks_t = nullptr;  // [n_elems][depth] (transposed reference layout)
  const uint32_t* shifts = nullptr;   // [depth]
  const double2* chars = nullptr;     // [n_elems] characters
  const uint64_t* onehot = nullptr;   // [n_bits][n_elems]: image of the one-bit state 1<<b under g
  const uint16_t* prio = nullptr;     // [n_elems] tie-break priority of state_info (lane order)
  // Packed tables of the matvec kernels: the group padded to gpl * 32 slots (slot s holds element
  // s, or element 0 for s >= n_elems), images shifted to the top bits (<< (64 - n_bits)) so that
  // the low bits can carry the candidate index 2 * slot + flip.
  int gpl = 0;                              // slots per lane (0: packed tables unavailable)
  const uint64_t* onehot_packed = nullptr;  // [n_bits][gpl * 32]
  const double2* chars_packed = nullptr;    // [gpl * 32]
  // Fermionic groups (spinful fermions with lattice symmetries): g acts on Fock states with the
  // sign of the permutation it induces on the occupied orbitals.  inv_g(x) = sum over occupied k
  // of popcount(x & L_g[k]), L_g[k] = orbitals l < k that g moves past k; the sign is
  // (-1)^inv_g(x).
  int fermionic = 0;
  const uint64_t* fsign = nullptr;          // [n_elems][n_bits]: L_g[k]
  const uint64_t* fsign_packed = nullptr;   // [n_bits][gpl * 32], slot-padded like onehot_packed
};

// (-1)^inv parity of a fermionic group element on `state`: L points to L_g[0] and consecutive
// orbitals are `stride` words apart.
__host__ __device__ inline int fermion_parity(const uint64_t* L, int stride, uint64_t state) {
  int inv = 0;
  for (uint64_t bits = state; bits != 0; bits &= bits - 1) {
#ifdef __CUDA_ARCH__
    const int k = __ffsll((long long)bits) - 1;
    inv += __popcll(state & L[(size_t)k * stride]);
#else
    const int k = __builtin_ctzll(bits);
    inv += __builtin_popcountll(state & L[(size_t)k * stride]);
#endif
  }
  return inv & 1;
}

// Slots per lane of the matvec kernels for a group of n elements (ascending choices).
constexpr int kGplSet[] = {1, 2, 3, 4, 6, 9, 12, 16};
inline int pick_gpl_for(int n_elems) {
  const int need = (n_elems + 31) / 32;
  for (int g : kGplSet)
    if (g >= need) return g;
  return -1;
}

// Device view of a sorted representative array and its prefix-bucket index.
struct DeviceIndex {
  int64_t n_states = 0;
  const uint64_t* reps = nullptr;
  const double* norms = nullptr;      // state_info norms of the representatives
  const double* inv_norms = nullptr;  // 1 / norm (0 for a zero norm): no division per row
  const uint32_t* offsets = nullptr;  // [2^prefix_bits + 1] bucket starts, or null
  // Low `shift` bits of every representative (shift <= 16), or null: a lookup then scans the
  // needle's bucket [offsets[b], offsets[b + 1]) in these 2-byte suffixes instead of searching
  // a window of 8-byte representatives.
  const uint16_t* suffix16 = nullptr;
  int shift = 0;                      // bucket = state >> shift
  int64_t range_size = 0;             // largest bucket (window length of the search without suffixes)
  int prefix_bits = 0;
  uint64_t max_state = ~0ull;         // largest representative (larger needles are absent)
  int identity = 0;                   // index(state) = state
  // combinadics ranking (fixed Hamming weight, no projection): index = rank(state) - rank_base
  int combinadic = 0;
  int64_t rank_base = 0;
};

// Basis-level constraints checked on every generated state (fixed particle numbers).
struct DeviceConstraint {
  int kind = 0;            // 0 none, 1 popcount(state) == w0, 2 popcount(low half)==w0 && popcount(high half)==w1
  int half_bits = 0;
  int w0 = 0, w1 = 0;
};

// Off-diagonal / diagonal term tables on the device.
struct DeviceTerms {
  int n = 0;
  const uint64_t* m = nullptr;
  const uint64_t* l = nullptr;  // pattern matched by the row state (the bra side)
  const uint64_t* r = nullptr;
  const uint64_t* x = nullptr;
  const uint64_t* s = nullptr;
  const double2* v = nullptr;
  const int32_t* coupling = nullptr;  // optional coupling id per term
  // Per term: bits 0-7 lowest flipped site, 8-15 highest flipped site, 16-23 number of flipped
  // sites, bit 24 set when the term can change a conserved particle number of the basis.
  const uint32_t* xinfo = nullptr;
  int all_two_site = 0;               // every term flips exactly two sites and keeps the basis'
                                      // conserved numbers (no term needs a constraint check)
};
constexpr uint32_t kTermNeedsCheck = 1u << 24;

// Host-side records behind the opaque kernel-data pointers of the plugin tables.
struct OrbitData {
  uint32_t magic;
  int n_bits, n_elems, depth, spin_inversion;
  std::vector<uint64_t> masks;        // reference layout [depth][n_elems]
  std::vector<uint32_t> shifts;
  std::vector<double> chars_re, chars_im;
  // Host image of the device block (masks_t | shifts | chars | onehot | prio) and its offsets;
  // uploaded on first use so that kernel data can be created on a machine without a GPU.
  std::vector<uint8_t> host_block;
  size_t off_masks = 0, off_shifts = 0, off_chars = 0, off_onehot = 0, off_prio = 0;
  size_t off_onehot_packed = 0, off_chars_packed = 0;
  size_t off_fsign = 0, off_fsign_packed = 0;  // fermionic groups only
  int gpl = 0;  // packed tables present when > 0
  int fermionic = 0;
  bool standard_shifts = true;
  mutable DeviceGroup dev;
  mutable void* dev_block = nullptr;  // one allocation holding all device arrays
  mutable int dev_device = -1;
};

struct IndexData {
  uint32_t magic;
  int64_t n_states;
  const uint64_t* host_reps;          // borrowed from the basis (chpl_external_array)
  int number_bits;
  int prefix_bits;
  DeviceIndex dev;
  uint64_t* d_reps = nullptr;
  uint32_t* d_offsets = nullptr;
  uint16_t* d_suffix = nullptr;       // 2-byte key suffixes (shift <= 16)
  double* d_norms = nullptr;          // filled lazily when a projected matvec needs them
  const OrbitData* norms_for = nullptr;
};

constexpr uint32_t kOrbitMagic = 0x4f524249u;  // "ORBI"
constexpr uint32_t kIndexMagic = 0x494e4458u;  // "INDX"

// ---- runtime (abi.cu) --------------------------------------------------------------------------
cudaStream_t default_stream();
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);  // records msg, returns code
bool cuda_ok(cudaError_t e, const char* what);
int* device_error_word();                     // 4 ints of device scratch for kernel error reports
void* scratch(size_t bytes, int slot);        // cached device scratch buffers
void* pinned_scratch(size_t bytes, int slot); // cached pinned host buffers
int num_sms();

// ---- orbit scan + enumeration + index (basis.cu) -----------------------------------------------
int launch_state_info(const DeviceGroup& g, int64_t n, const uint64_t* d_x, uint64_t* d_rep,
                      double2* d_char, double* d_norm, int lane_width, cudaStream_t s);
int launch_is_representative(const DeviceGroup& g, int64_t n, const uint64_t* d_x,
                             uint8_t* d_flag, double* d_norm, int lane_width, cudaStream_t s);
int launch_orbit_norms(const DeviceGroup& g, int64_t n, const uint64_t* d_reps, double* d_norms,
                       cudaStream_t s);
// inv[i] = 1 / norms[i], or 0 where norms[i] == 0.
int launch_inverse_norms(const double* d_norms, int64_t n, double* d_inv, cudaStream_t s);
int compute_site_images(OrbitData* od);          // host tables (no GPU needed)
const DeviceGroup* orbit_device(const OrbitData* od);  // uploads on first use; null on failure

struct EnumerateRequest {
  int mode;              // 0 projected spin, 1 unprojected (fixed weight or all), 2 spinful per
                         // sector, 3 projected spinful fermions (fixed N_up, N_down)
  int hamming_fixed;
  int number_sites;
  int spin_inversion;
  uint64_t lower, upper;
  int reference_norm_rule;  // 1: keep a state iff the reference's floating stabiliser sum > 0
};
// Enumerates into device memory; *d_out is allocated with cudaMalloc (caller frees).
int enumerate_states(const DeviceGroup* g, const EnumerateRequest& req, uint64_t** d_out,
                     int64_t* count, cudaStream_t s);
// Enumerates into the caller's d_out (capacity entries) without allocating: all scratch lives in
// a static device array (see basis.cu).  *count receives the number of states.
int enumerate_states_noalloc(const OrbitData* od, const EnumerateRequest& req, uint64_t* d_out,
                             int64_t capacity, int64_t* count, cudaStream_t s);

// out[i] = sum_{k<i} in[k] for i <= n (out has n + 1 entries); stream-ordered.
int exclusive_scan_counts(const int32_t* d_in, int64_t n, int64_t* d_out, cudaStream_t s);

// Bucket starts over the top bits actually used (unclamped: bucket b is [off[b], off[b + 1])),
// the largest bucket, and, where the bucket shift is at most 16 bits, the 2-byte key suffixes
// (*d_suffix, else null).
int build_prefix_index(const uint64_t* d_reps, int64_t n, int number_bits, int prefix_bits,
                       uint32_t** d_offsets, int64_t* range_size, int* shift, cudaStream_t s,
                       uint64_t* max_state, uint16_t** d_suffix);
int launch_state_index(const DeviceIndex& ix, int64_t n, const uint64_t* d_x, int64_t* d_out,
                       cudaStream_t s);

// combinadics on the host (Basis.hs:519-550)
int64_t fixed_hamming_state_to_index(uint64_t a);
uint64_t fixed_hamming_index_to_state(int64_t index, int h);

// ---- matvec (matvec.cu) ------------------------------------------------------------------------
enum class Scalar { Real, Complex };

struct MatvecProblem {
  int projection;            // 0 none, 1 spin inversion only, 2 full group
  DeviceGroup group;
  DeviceIndex index;
  DeviceConstraint constraint;
  DeviceTerms off;           // terms applied to the row state through their l pattern
  DeviceTerms diag;
  int64_t n_rows;
  unsigned long long* nnz_counter = nullptr;  // optional: counts off-diagonal elements found
  // Every off-diagonal matrix element is real (real term coefficients and real characters): a
  // complex right-hand side then needs 2 FP64 FMAs per element instead of 4.
  int real_elements = 0;
  // Optional gather source x_j * n_j (x scaled by the orbit norms, leading dimension ldxs in
  // elements): the gathers then need no norm per element.  FP64 for the FP64 kernels; for the
  // FP32-pair kernels each complex element is four floats [re_h, re_l, im_h, im_l] (the same 16
  // bytes).  The diagonal still reads the caller's x.
  const double* xs = nullptr;
  int64_t ldxs = 0;
};

int launch_matvec(const MatvecProblem& p, Scalar sc, int k, const double* d_x, int64_t ldx,
                  double* d_y, int64_t ldy, int* d_err, cudaStream_t s);
// The kernel launch_matvec picks for p: 2 packed (*gpl slots per lane), 1 fallback, 0 plain.
int matvec_kernel_form(const MatvecProblem& p, int* gpl);

// Sector plans (matvec.cu): y_s = H_s x_s (complex, k right-hand sides, leading dimensions
// ldx/ldy) for many sectors.  When the sectors share the group's site images, the terms and the
// constraint (`shareable`), each RHS chunk is ONE persistent launch over all sectors' rows;
// otherwise the plan launches the sectors one after the other.  Running a plan allocates only
// stream-ordered and does not synchronise, so it can be captured in a CUDA graph.
struct SectorPlan;
int sector_plan_build(const std::vector<MatvecProblem>& problems, bool shareable, int k,
                      const std::vector<const double*>& xs, int64_t ldx, const std::vector<double*>& ys,
                      int64_t ldy, SectorPlan** out);
int sector_plan_run(const SectorPlan* plan, int* d_err, cudaStream_t s);
bool sector_plan_batched(const SectorPlan* plan);            // runs as one launch per RHS chunk
int sector_plan_set_batched(SectorPlan* plan, bool batched);  // LS_GPU_ERR_INVALID if it cannot
void sector_plan_free(SectorPlan* plan);

// Per-state term application on device batches (apply.cu), the semantics of
// ls_internal_operator_apply_{diag,off_diag}_x1 (reference.c:67-135).
int launch_apply_diag(const DeviceTerms& diag, int64_t count, const uint64_t* d_alphas, double* d_ys,
                      cudaStream_t s);
int launch_apply_off_diag(const DeviceTerms& off, int64_t count, const uint64_t* d_alphas, uint64_t* d_betas,
                          double* d_coeffs, int64_t* d_offsets, cudaStream_t s);

// out = in^T for a row-major rows x cols matrix of doubles (apply.cu).
int launch_transpose(const double* d_in, double* d_out, int64_t rows, int64_t cols, cudaStream_t s);

int launch_coupling_products(const MatvecProblem& p, int n_couplings, const double* d_g,
                             const double* d_x, double* d_out, int* d_err, cudaStream_t s);

// Dense products of the block eigensolver in FP32-pair arithmetic (blockops.cu).
int launch_block_gram(int64_t S, int64_t D, int k, const double* d_x, const double* d_y, double* d_g,
                      cudaStream_t s);
int launch_block_update(int64_t S, int64_t D, int k, double beta, const double* d_w, const double* d_x1,
                        const double* d_m1, const double* d_x2, const double* d_m2, double* d_out,
                        cudaStream_t s);
// G[s][o] = sum over c < chunks of partial[s][c][o] (o < nout), in a fixed order (blockops.cu)
int launch_gram_partial_sum(const double2* partial, int chunks, int nout, int64_t S, double2* G, cudaStream_t s);
// tensor-core forms (blockops_tc.cu): same contracts as launch_block_gram / launch_block_update
int launch_block_gram_tc(int64_t S, int64_t D, int k, const double* d_x, const double* d_y, double* d_g,
                         cudaStream_t s);
int launch_block_update_tc(int64_t S, int64_t D, int k, double beta, const double* d_w, const double* d_x1,
                           const double* d_m1, const double* d_x2, const double* d_m2, double* d_out,
                           cudaStream_t s);

}  // namespace lsg
