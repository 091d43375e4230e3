/*
 * ls_gb300.h -- C ABI of the GB300 (sm_103a) exact-diagonalization hot path.
 *
 * Two groups of entry points live in libls_gb300.so:
 *
 *  1. Drop-in symbols.  Same names, signatures and error behaviour as the symbols that
 *     lattice-symmetries' Haskell foreign library, its Chapel library and its Python cffi
 *     module bind for the hot path (orbit scan, enumeration, state index, matvec).  Linking
 *     the Haskell library against libls_gb300.so instead of kernels/libkernels.a and the
 *     Chapel library moves basis construction and H*x onto the GPU with no source change
 *     on the host side.  Each declaration cites the reference declaration it replaces.
 *
 *  2. Additive symbols (prefix ls_gpu_).  Device-pointer, stream-ordered, complex128,
 *     multi-right-hand-side, adjoint, multi-sector and per-coupling-gradient entry points
 *     that the reference does not have.  Nothing in group 1 depends on them.
 *
 * The struct layouts below restate kernels/lattice_symmetries_types.h:27-180 field by
 * field: the Haskell host fills these structs and passes pointers across the boundary,
 * so the byte layout must be identical.
 */
#pragma once

#if defined(__cplusplus)
#include <complex>
#include <cstddef>
#include <cstdint>
#else
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#endif

#if defined(__cplusplus)
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------
 * Types shared with the reference (lattice_symmetries_types.h).
 * ------------------------------------------------------------------------------------------- */

/* types.h:27-32: a Chapel-owned or foreign-owned array; `freer(elts)` releases it. */
typedef struct {
  void *elts;
  uint64_t num_elts;
  void *freer;
} chpl_external_array;

/* types.h:43-56: complex128 scalar. */
#if defined(__cplusplus)
typedef std::complex<double> ls_hs_scalar;
#elif defined(LS_NO_STD_COMPLEX)
typedef struct ls_hs_scalar {
  double _real;
  double _imag;
} ls_hs_scalar;
#else
typedef _Complex double ls_hs_scalar;
#endif

/* The reference declares refcounts as `_Atomic int`; the representation is a plain int. */
typedef int ls_gb300_refcount;

/* types.h:81-85 */
typedef enum ls_hs_particle_type {
  LS_HS_SPIN,
  LS_HS_SPINFUL_FERMION,
  LS_HS_SPINLESS_FERMION
} ls_hs_particle_type;

/* types.h:87-98: the three basis kernel function-pointer types. */
typedef void (*ls_hs_internal_state_index_kernel_type)(
    ptrdiff_t batch_size, uint64_t const *alphas, ptrdiff_t alphas_stride,
    ptrdiff_t *indices, ptrdiff_t indices_stride, void const *private_data);

typedef void (*ls_hs_internal_is_representative_kernel_type)(
    ptrdiff_t batch_size, uint64_t const *alphas, ptrdiff_t alphas_stride,
    uint8_t *are_representatives, double *norms, void const *private_data);

typedef void (*ls_hs_internal_state_info_kernel_type)(
    ptrdiff_t batch_size, uint64_t const *alphas, ptrdiff_t alphas_stride,
    uint64_t *betas, ptrdiff_t betas_stride, ls_hs_scalar *characters,
    double *norms, void const *private_data);

/* types.h:100-107: the basis kernel plugin table. */
typedef struct ls_hs_basis_kernels {
  ls_hs_internal_state_info_kernel_type state_info_kernel;
  void *state_info_data;
  ls_hs_internal_is_representative_kernel_type is_representative_kernel;
  void *is_representative_data;
  ls_hs_internal_state_index_kernel_type state_index_kernel;
  void *state_index_data;
} ls_hs_basis_kernels;

/* types.h:109-119: a permutation group as a batched Benes network.
 * masks: [number_shifts][number_masks] row-major, shifts: [number_shifts],
 * eigvals_re/im: [number_masks] characters of the group elements. */
typedef struct ls_hs_permutation_group {
  ls_gb300_refcount refcount;
  int number_bits;
  int number_shifts;
  int number_masks;
  uint64_t *masks;
  uint64_t *shifts;
  double *eigvals_re;
  double *eigvals_im;
  void *haskell_payload;
} ls_hs_permutation_group;

/* types.h:121-133 */
typedef struct ls_hs_basis {
  ls_gb300_refcount refcount;
  int number_sites;
  int number_particles;
  int number_up;
  ls_hs_particle_type particle_type;
  int spin_inversion;
  bool state_index_is_identity;
  bool requires_projection;
  ls_hs_basis_kernels *kernels;
  chpl_external_array representatives;
  void *haskell_payload;
} ls_hs_basis;

/* types.h:140-151: non-branching terms (v, m, l, r, x, s), one 64-bit word per term. */
typedef struct ls_hs_nonbranching_terms {
  int number_terms;
  int number_bits;
  ls_hs_scalar const *v;
  uint64_t const *m;
  uint64_t const *l;
  uint64_t const *r;
  uint64_t const *x;
  uint64_t const *s;
} ls_hs_nonbranching_terms;

/* types.h:153-161 */
typedef struct ls_hs_operator {
  ls_gb300_refcount refcount;
  ls_hs_basis const *basis;
  ls_hs_nonbranching_terms const *off_diag_terms;
  ls_hs_nonbranching_terms const *diag_terms;
  void *haskell_payload;
} ls_hs_operator;

/* types.h:170-180: the driver plugin table (installed by Chapel in the reference). */
typedef struct ls_chpl_kernels {
  void (*enumerate_states)(ls_hs_basis const *, uint64_t, uint64_t, chpl_external_array *);
  void (*operator_apply_off_diag)(ls_hs_operator *, int64_t, uint64_t *, chpl_external_array *,
                                  chpl_external_array *, chpl_external_array *, int64_t);
  void (*operator_apply_diag)(ls_hs_operator *, int64_t, uint64_t *, chpl_external_array *,
                              int64_t);
  void (*matrix_vector_product)(ls_hs_operator *, int, double const *, double *);
} ls_chpl_kernels;

/* ---------------------------------------------------------------------------------------------
 * 1. Drop-in symbols.
 * ------------------------------------------------------------------------------------------- */

/* Error handling: reference.c:11-36, types.h:61-74. */
void ls_hs_set_exception_handler(void (*handler)(char const *message));
void ls_hs_error(char const *message);
void ls_hs_fatal_error(char const *func, int line, char const *message);

/* External arrays and refcounts: reference.c:40-64, types.h:193-195. */
void ls_hs_internal_destroy_external_array(chpl_external_array *arr);
int ls_hs_internal_read_refcount(ls_gb300_refcount const *refcount);
void ls_hs_internal_write_refcount(ls_gb300_refcount *refcount, int value);
int ls_hs_internal_inc_refcount(ls_gb300_refcount *refcount);
int ls_hs_internal_dec_refcount(ls_gb300_refcount *refcount);

/* Driver plugin table: reference.c:213-225, types.h:193-194. libls_gb300.so installs its GPU
 * drivers into the table when it is loaded and again on ls_chpl_init(). */
ls_chpl_kernels const *ls_hs_internal_get_chpl_kernels(void);
void ls_hs_internal_set_chpl_kernels(ls_chpl_kernels const *kernels);
/* chapel/src/library.c:19-34 (runtime start-up / shutdown; here: install tables, create the
 * CUDA stream / release device memory). */
void ls_chpl_init(void);
void ls_chpl_finalize(void);
/* LatticeSymmetries.chpl:28-30 (declared at chapel/lib/lattice_symmetries_chapel.h:35):
 * installs this library's drivers into the plugin table again (after a host replaced them). */
void ls_chpl_init_kernels(void);
/* Module initialisers of the Chapel library (chapel/lib/lattice_symmetries_chapel.h:5-42,
 * called by chapel/src/library.c:23-31).  This library has no module state to initialise:
 * chpl__init_LatticeSymmetries installs the drivers (the module body of LatticeSymmetries.chpl:32),
 * the others do nothing.  The arguments (line and file of the call) are ignored.
 * ls_hs_init / ls_hs_exit (types.h:61-62) start and stop the Haskell runtime; they belong to the
 * Haskell host library and are not exported here. */
void chpl__init_BatchedOperator(int64_t ln, int32_t fn);
void chpl__init_CommonParameters(int64_t ln, int32_t fn);
void chpl__init_ConcurrentAccessor(int64_t ln, int32_t fn);
void chpl__init_DistributedMatrixVector(int64_t ln, int32_t fn);
void chpl__init_FFI(int64_t ln, int32_t fn);
void chpl__init_ForeignTypes(int64_t ln, int32_t fn);
void chpl__init_LatticeSymmetries(int64_t ln, int32_t fn);
void chpl__init_StatesEnumeration(int64_t ln, int32_t fn);
void chpl__init_Vector(int64_t ln, int32_t fn);

/* Orbit-scan kernel data: replaces ls_internal_create_halide_kernel_data (kernels.c:112-189,
 * bound at Basis.hs:915-919). Uploads masks, characters and the per-site image table of the
 * group to the GPU. spin_inversion is 0, +1 or -1. */
void *ls_internal_create_halide_kernel_data(ls_hs_permutation_group const *group,
                                            int spin_inversion);
void ls_internal_destroy_halide_kernel_data(void *data);

/* Orbit-scan kernels, FunPtr-compatible: replace ls_hs_is_representative_halide_kernel
 * (kernels.c:195-244) and ls_hs_state_info_halide_kernel (kernels.c:246-319), bound at
 * Basis.hs:921-925.  Host pointers, any strides.
 *
 * Lane order: where several group elements map a state to its representative, the character
 * returned is the one the reference's Halide kernel picks, which depends on the lane width its
 * build vectorised with (generator.cpp:80, :155-164).  These kernels reproduce the x86-64 AVX2
 * build the reference ships (kernels/Makefile:21-28): 8 lanes for state_info and 4 for
 * is_representative (whose floating stabiliser sum is added in the same lane order).  A
 * reference built for another vector width can return a different (equally valid) character for
 * such states, and a different rounding residue of that sum. */
void ls_hs_is_representative_halide_kernel(ptrdiff_t batch_size, uint64_t const *alphas,
                                           ptrdiff_t alphas_stride, uint8_t *are_representatives,
                                           double *norms, void const *private_data);
void ls_hs_state_info_halide_kernel(ptrdiff_t batch_size, uint64_t const *alphas,
                                    ptrdiff_t alphas_stride, uint64_t *betas,
                                    ptrdiff_t betas_stride, ls_hs_scalar *characters,
                                    double *norms, void const *private_data);

/* State index: replaces indexing.c:94-125 and :273-325 (types.h:198-214; bound at
 * Basis.hs:904-908).  The table and the search run on the GPU. */
typedef struct ls_hs_state_index_binary_search_data ls_hs_state_index_binary_search_data;
ls_hs_state_index_binary_search_data *ls_hs_create_state_index_binary_search_kernel_data(
    chpl_external_array const *representatives, int number_bits, int prefix_bits);
void ls_hs_destroy_state_index_binary_search_kernel_data(
    ls_hs_state_index_binary_search_data *cache);
void ls_hs_state_index_binary_search_kernel(ptrdiff_t batch_size, uint64_t const *spins,
                                            ptrdiff_t spins_stride, ptrdiff_t *indices,
                                            ptrdiff_t indices_stride,
                                            void const *private_kernel_data);

/* Dispatchers through basis->kernels: reference.c:137-171 (types.h:216-230). */
void ls_hs_state_index(ls_hs_basis const *basis, ptrdiff_t batch_size, uint64_t const *spins,
                       ptrdiff_t spins_stride, ptrdiff_t *indices, ptrdiff_t indices_stride);
void ls_hs_is_representative(ls_hs_basis const *basis, ptrdiff_t batch_size,
                             uint64_t const *alphas, ptrdiff_t alphas_stride,
                             uint8_t *are_representatives, double *norms);
void ls_hs_state_info(ls_hs_basis const *basis, ptrdiff_t batch_size, uint64_t const *alphas,
                      ptrdiff_t alphas_stride, uint64_t *betas, ptrdiff_t betas_stride,
                      ls_hs_scalar *characters, double *norms);

/* Basis construction: reference.c:173-211 (types.h:231-235). */
void ls_hs_build_representatives(ls_hs_basis *basis, uint64_t lower, uint64_t upper);
void ls_hs_unchecked_set_representatives(ls_hs_basis *basis, chpl_external_array const *states,
                                         int cache_bits);

/* Combinadics: ForeignLibrary.hs:203-211 (Basis.hs:519-550). */
ptrdiff_t ls_hs_fixed_hamming_state_to_index(uint64_t basis_state);
uint64_t ls_hs_fixed_hamming_index_to_state(ptrdiff_t state_index, int hamming_weight);

/* Term generation on the host: reference.c:67-134 (types.h:238-249). */
void ls_internal_operator_apply_diag_x1(ls_hs_operator const *op, ptrdiff_t batch_size,
                                        uint64_t const *alphas, double *ys, double const *xs);
void ls_internal_operator_apply_off_diag_x1(ls_hs_operator const *op, ptrdiff_t batch_size,
                                            uint64_t const *alphas, uint64_t *betas,
                                            ls_hs_scalar *coeffs, ptrdiff_t *offsets,
                                            double const *xs);

/* Chapel drivers: StatesEnumeration.chpl:692-709, BatchedOperator.chpl:298-357,
 * DistributedMatrixVector.chpl:1090-1105 (chapel/lib/lattice_symmetries_chapel.h:7-41).
 * The matvec reads x and writes y in host memory; complex coefficients contribute their real part
 * (DistributedMatrixVector.chpl:126).  The reference accepts num_vectors == 1 only; here
 * num_vectors >= 1 vectors stored one after the other (x[v * D + i], y likewise) share one orbit
 * scan on the GPU, and num_vectors == 1 behaves exactly as in the reference. */
void ls_chpl_enumerate_representatives(ls_hs_basis *p, uint64_t lower, uint64_t upper,
                                       chpl_external_array *dest);
void ls_chpl_operator_apply_diag(ls_hs_operator *matrix, int64_t count, uint64_t *alphas,
                                 chpl_external_array *coeffs, int64_t num_tasks);
void ls_chpl_operator_apply_off_diag(ls_hs_operator *matrix, int64_t count, uint64_t *alphas,
                                     chpl_external_array *betas, chpl_external_array *coeffs,
                                     chpl_external_array *offsets, int64_t num_tasks);
void ls_chpl_matrix_vector_product(ls_hs_operator *matrix, int num_vectors, double const *x,
                                   double *y);

/* ---------------------------------------------------------------------------------------------
 * 2. Additive symbols (no counterpart in the reference).
 *
 * All return 0 on success and a negative code on failure; ls_gpu_last_error() gives the message.
 * `stream` is a cudaStream_t; NULL is the legacy default stream, as everywhere in CUDA.  Device
 * pointers are CUDA global memory on the current device.  Complex arrays are interleaved
 * (re, im) float64 pairs, 16-byte aligned.
 * ------------------------------------------------------------------------------------------- */

#define LS_GPU_OK 0
#define LS_GPU_ERR_INVALID (-1)   /* bad argument */
#define LS_GPU_ERR_CUDA (-2)      /* CUDA runtime error */
#define LS_GPU_ERR_BASIS (-3)     /* a generated state left the basis (operator breaks a conserved number) */
#define LS_GPU_ERR_NOT_BUILT (-4) /* basis has no representatives */
#define LS_GPU_ERR_TIMEOUT (-5)   /* a bounded device wait gave up */

char const *ls_gpu_last_error(void);
int ls_gpu_device_synchronize(void);

/* Number of representatives and device pointers of the GPU-resident basis (built by
 * ls_hs_build_representatives or set by ls_hs_unchecked_set_representatives).  norms are the
 * state_info norms sqrt(S/|G|) of the representatives (all 1 without projection). */
int ls_gpu_basis_info(ls_hs_basis const *basis, int64_t *number_states,
                      uint64_t const **d_representatives, double const **d_norms);

/* y[D][k] = A x[D][k] for k right-hand sides stored row-major with leading dimension ld
 * (ld >= k), A = H (adjoint = 0) or A = H^dagger (adjoint = 1).  Complex128 x and y.
 * Full complex arithmetic: complex characters and coefficients are kept.
 * Stream-ordered: returns after enqueueing (usable inside CUDA graph capture once the basis
 * and operator data are resident); a generated state that leaves the basis is recorded on the
 * device and reported by ls_gpu_check_errors. */
int ls_gpu_matvec_c128(ls_hs_operator const *op, int k, double const *d_x, int64_t ldx,
                       double *d_y, int64_t ldy, int adjoint, void *stream);
/* The same for real float64 vectors, with the reference's real-part semantics. */
int ls_gpu_matvec_f64(ls_hs_operator const *op, int k, double const *d_x, int64_t ldx,
                      double *d_y, int64_t ldy, int adjoint, void *stream);
/* Synchronises `stream`, returns LS_GPU_ERR_BASIS if a matvec since the last check generated a
 * state outside its basis (and clears the flag), else 0. */
int ls_gpu_check_errors(void *stream);
/* Number of off-diagonal matrix elements (generated targets found in the basis) of H. */
int ls_gpu_count_nonzeros(ls_hs_operator const *op, int64_t *nnz);
/* Per-stage timing, off by default (the counterpart of the reference's timing tree,
 * chapel/src/Utils.chpl:49-144): when on, the library's stages -- basis.enumerate,
 * basis.enumerate_compact, basis.index, basis.orbit_norms, matvec.prescale, matvec.kernel,
 * sectors.prescale, sectors.kernel, couplings.kernel, lanczos.gram, lanczos.update -- each open an
 * NVTX range and record a CUDA-event pair on their stream (no added synchronisation).  Do not
 * switch it on while a stream is being captured into a CUDA graph.  ls_gpu_trace_report waits for
 * the traced stages and writes one "stage count total_ms host_ms" line per stage (the time between
 * the stage's events on the GPU, and the wall time the calling thread spent in it) into buffer
 * (NUL-terminated, truncated to size); it returns the full length; reset != 0 clears the totals. */
int ls_gpu_set_tracing(int on);
int ls_gpu_trace_report(char *buffer, size_t size, int reset);
/* The kernel a matvec of `op` runs: *form = 2 for the packed projected kernel (its tables fit in
 * shared memory; *slots_per_lane = group elements per lane, 32 lanes per warp), 1 for the
 * fallback projected kernel (*slots_per_lane likewise), 0 for the thread-per-row kernel (no
 * permutation group; *slots_per_lane = 0).  Needs a built basis. */
int ls_gpu_matvec_kernel_info(ls_hs_operator const *op, int *form, int *slots_per_lane);

/* Releases the device copies of an operator's term tables (made on the first GPU use of `op`,
 * keyed by its address).  Call before freeing or reusing the ls_hs_operator; no-op otherwise. */
void ls_gpu_release_operator(ls_hs_operator const *op);

/* Term application on device batches of basis states, with the results, term order and layout of
 * ls_internal_operator_apply_diag_x1 / ls_internal_operator_apply_off_diag_x1 (reference.c:67-135,
 * called by BatchedOperator.chpl:298-357): ys[i] = sum of the real diagonal coefficients of
 * alphas[i]; off-diagonal targets betas / complex128 coeffs in compressed rows
 * (offsets[0 .. count], offsets[0] = 0).  betas and coeffs need count * number_off_diag_terms
 * entries.  Device pointers, stream-ordered; concurrent calls on different streams must not
 * overlap (they share a scratch buffer). */
int ls_gpu_operator_apply_diag(ls_hs_operator const *op, int64_t count, uint64_t const *d_alphas,
                               double *d_ys, void *stream);
int ls_gpu_operator_apply_off_diag(ls_hs_operator const *op, int64_t count, uint64_t const *d_alphas,
                                   uint64_t *d_betas, double *d_coeffs, int64_t *d_offsets,
                                   void *stream);

/* Per-coupling inner products out[c] = <g, H_c x> = sum_i conj(g_i) (H_c x)_i for an operator
 * H = sum_c H_c whose terms are tagged with coupling ids: term_coupling[t] in [0, n_couplings) for
 * the off-diagonal terms, then the diagonal terms, in table order (host array).  g, x: complex128
 * [D]; out: complex128 [n_couplings]; all device pointers, stream-ordered.  This is the gradient
 * of Re<g, H(theta) x> with respect to the couplings theta (Re out[c]).  One fused pass (the
 * packed orbit scan) for bases with lattice symmetries of at most 128 elements and at most 4
 * couplings; other operators return LS_GPU_ERR_INVALID (use one matvec per coupling).  No
 * counterpart in the reference. */
int ls_gpu_coupling_inner_products(ls_hs_operator const *op, int n_couplings,
                                   int32_t const *term_coupling, double const *d_g,
                                   double const *d_x, double *d_out, void *stream);

/* Orbit-scan data for spinful fermions with lattice symmetries: `group` permutes the 2n orbitals
 * (up site k -> orbital k, down site k -> orbital n + k; the same site permutation on both
 * species) and carries the characters.  Every element acts on Fock states with the sign of the
 * permutation it induces on the occupied orbitals, in state_info, is_representative, the norms,
 * the enumeration (which needs fixed N_up, N_down and keeps a state iff its stabiliser acts
 * trivially) and the matvec.  Install it in ls_hs_basis_kernels like the spin kernel data and set
 * requires_projection.  No counterpart in the reference, whose fermionic bases have no lattice
 * symmetries (Basis.hs:713-723).  Destroy with ls_internal_destroy_halide_kernel_data. */
void *ls_gpu_create_fermionic_kernel_data(ls_hs_permutation_group const *group, int number_sites);

/* Membership rule of the projected enumeration behind ls_hs_build_representatives and
 * ls_chpl_enumerate_representatives: 0 (default) keeps a state iff the reference's floating
 * stabiliser sum is positive (StatesEnumeration.chpl:242-268), 1 iff its stabiliser has only
 * trivial characters (exact).  They differ only in complex sectors, where the floating rule keeps
 * rounding residue: representatives whose exact norm is zero.  The matvec treats such states as
 * zero rows and columns.  Returns the previous rule.  No counterpart in the reference. */
int ls_gpu_set_enumeration_rule(int exact);

/* Batched multi-sector block matvec y_s = H_s x_s (or H_s^dagger x_s), complex128, for many
 * symmetry sectors at once.  No reference counterpart: the reference applies one operator to one
 * real vector per call (DistributedMatrixVector.chpl:1096-1097).
 *
 * A plan fixes the operators (one per sector, each on its own built basis), k right-hand sides and
 * the device vectors: d_x[s], d_y[s] point to [D_s][ld] complex128 blocks.  When all sectors share
 * the group's site images, the terms and the particle-number constraint (the usual case: the same
 * Hamiltonian in different momentum / inversion sectors of one group), each chunk of up to 16
 * right-hand sides is ONE persistent kernel launch over the rows of all sectors, so uneven sector
 * sizes balance across the GPU; otherwise the plan launches the sectors one after the other
 * (ls_gpu_sector_plan_is_batched tells which form runs).  Running a plan does not synchronise and
 * allocates only stream-ordered (cudaMallocAsync / cudaFreeAsync of the copy of x scaled by the
 * orbit norms), so it may be captured in a CUDA graph (make one uncaptured run first).  A plan keeps
 * device pointers of the operators' uploaded tables: changing an operator's terms invalidates it
 * (run then fails).  Errors of generated states (wrong particle number) go to the device error
 * word: check with ls_gpu_check_errors. */
int ls_gpu_sector_plan_create(int n_sectors, ls_hs_operator const *const *ops, int k,
                              double const *const *d_x, int64_t ldx, double *const *d_y,
                              int64_t ldy, int adjoint, void **plan);
int ls_gpu_sector_plan_run(void const *plan, void *stream);
int ls_gpu_sector_plan_is_batched(void const *plan);
/* Chooses the form: batched != 0 runs one launch per chunk over all sectors (LS_GPU_ERR_INVALID
 * if the sectors cannot share one), 0 one launch per sector. */
int ls_gpu_sector_plan_set_batched(void *plan, int batched);
/* Times both forms on `stream` (one warm-up and two timed runs each; they overwrite the output
 * blocks) and keeps the faster: one persistent launch wins for many small sectors, one launch per
 * sector can win for a few large ones.  Reports the choice and both times (ms per run; -1 for a
 * form the plan cannot run). */
int ls_gpu_sector_plan_autotune(void *plan, void *stream, int *batched, double *ms_batched,
                                double *ms_per_sector);
int ls_gpu_sector_plan_destroy(void *plan);

/* One-shot form of the above (leading dimension k); synchronises `stream` before returning. */
int ls_gpu_matvec_multi_sector_c128(int n_sectors, ls_hs_operator const *const *ops, int k,
                                    double const *const *d_x, double *const *d_y, int adjoint,
                                    void *stream);

/* Device-side orbit scan / index on device arrays (no host staging). */
int ls_gpu_state_info(ls_hs_basis const *basis, int64_t batch, uint64_t const *d_alphas,
                      uint64_t *d_betas, double *d_characters, double *d_norms, void *stream);
int ls_gpu_is_representative(ls_hs_basis const *basis, int64_t batch, uint64_t const *d_alphas,
                             uint8_t *d_flags, double *d_norms, void *stream);
int ls_gpu_state_index(ls_hs_basis const *basis, int64_t batch, uint64_t const *d_alphas,
                       int64_t *d_indices, void *stream);

/* Basis enumeration that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory: code running under a framework that owns every
 * device allocation (its pool reserves the GPU's memory and hands out buffers), or code between
 * stream captures, where cudaMalloc must not be called.  Writes the sorted representatives of
 * `basis` -- the same array ls_hs_build_representatives produces -- into the caller's device
 * buffer d_out of `capacity` entries and stores their number in *count (host memory).
 *
 * All scratch (the group tables, per-tile counts and offsets, scan sums) lives in one file-scope
 * device array of 16 MiB that every GPU loading the library holds until the process exits.  The
 * first call on a device looks up that array's device address (cudaGetSymbolAddress); make the
 * first call before any stream capture.  Limits: group tables up to 1 MiB and about 5.2e9
 * candidate states (LS_GPU_ERR_INVALID beyond, with a message); LS_GPU_ERR_INVALID also when
 * *count exceeds `capacity` (nothing is written past d_out[capacity - 1]) and when d_out is NULL
 * with a non-zero capacity.  This entry point does not set up the per-device runtime that the
 * other entry points share (their stream, error word and tables are allocated on first use), so
 * it may be the first call of the library on a device.  Calls share the array, so calls that
 * overlap on the GPU race; the call synchronises `stream` before returning. */
int ls_gpu_enumerate_noalloc(ls_hs_basis const *basis, uint64_t *d_out, int64_t capacity,
                             int64_t *count, void *stream);

/* Tuning knobs of the projected matvec kernels: threads per CTA (a multiple of 32, at most 1024;
 * 0 = each kernel's own maximum: 1024 for one right-hand side (768 for groups of more than 288
 * elements), 640 for FP64 blocks, 320 for the FP32-pair and batched kernels, lowered until the
 * shared-memory tables fit) and grid waves (the
 * grid is SMs x resident CTAs per SM x waves, one warp per row at a time; 0 = 4).  The fallback
 * kernel for groups whose packed tables do not fit (or 64-bit states) always runs 256-thread
 * CTAs. */
int ls_gpu_set_matvec_config(int threads_per_block, int waves);
/* Arithmetic of complex blocks of 8 or 16 right-hand sides in the plain and the batched
 * multi-sector kernels: 0 (default) = FP64; 1 = FP32 pairs for groups of at most 64 elements,
 * FP64 otherwise; 2 = FP32 pairs for every group.  In the pair form x_j * n_j is stored once per
 * call as two floats per component (16 bytes per complex element, like complex128), the
 * coefficient of each element is formed in FP64 and split, and the multiply-adds run on the
 * FP32 pipe with error-free products and two-sum accumulation: each product is below 2^-45
 * relative, so an output y_i = sum_j a_ij x_j is within about 2^-45 * sum_j |a_ij| |x_j| of the
 * exact sum (an absolute bound: an entry that cancels to near zero keeps that error, where FP64
 * gives ~1e-16 of the same sum); H X agrees with the FP64 form to ~1e-14 relative L2.  With a small group and 16 columns the FP64
 * form is bound by GB300's FP64 pipe (4 FP64 FMAs per element and column); with a large group
 * the integer orbit scan is the bound and FP64 is faster.  One right-hand side, real vectors and
 * blocks of 4 always run in FP64.  Returns LS_GPU_ERR_INVALID for other values. */
int ls_gpu_set_block_arithmetic(int mode);
int ls_gpu_get_block_arithmetic(void);
/* Most right-hand sides per kernel launch (16, 8, 4 or 1; larger k is split into launches). */
int ls_gpu_set_matvec_rhs_tile(int rhs_tile);
int ls_gpu_get_matvec_config(int *threads_per_block, int *waves, int *rhs_tile);
/* Autotuner: times the matvec of `op` on k complex right-hand sides over a table of
 * (threads, waves) pairs ({kernel maximum, 768, 512} x {1, 2, 4, 8}) and, for k >= 8,
 * right-hand-side tiles, and installs the fastest; reports the launch shape (threads 0 = the
 * kernel maximum) and its time (ms). */
int ls_gpu_autotune_matvec(ls_hs_operator const *op, int k, int *best_threads, int *best_waves,
                           double *best_ms);

/* Dense products of the block eigensolver on tall complex128 blocks: S sectors of D rows and
 * 1 <= k <= 16 columns, stored [S][D][k] row-major (interleaved re, im), device pointers.
 *   ls_gpu_block_gram:   G[s] = X[s]^H Y[s], G [S][k][k]; X == Y allowed.
 *   ls_gpu_block_update: out[s] = beta W[s] + X1[s] M1[s] + X2[s] M2[s], M [S][k][k]; X2 and M2
 *                        are NULL together; W may be NULL when beta == 0; out may alias W, X1
 *                        or X2 (each row is read before it is written).
 * The blocks stay FP64 in memory; the products are evaluated in FP32-pair arithmetic (each
 * FP64 input split into two floats, error-free hi*hi products, two-sum accumulation: about
 * below 2^-45 relative per product, every entry within ~1e-13 of the sum of its terms' magnitudes)
 * because GB300's FP64 pipe is a small fraction of its FP32 rate.  Range: products of two
 * entries must stay below ~1e38 in magnitude (else inf), and lose low-order bits below ~1e-30
 * (orthonormal and H-applied blocks are far inside).
 * Stream-ordered: the Gram allocates its partial sums with cudaMallocAsync on `stream`, so both
 * can be recorded in a CUDA graph.  No reference counterpart: the reference's eigensolvers are
 * scipy's eigsh over the matvec (python/lattice_symmetries/__init__.py:751-752) and PRIMME
 * (chapel/src/Diagonalize.chpl). */
int ls_gpu_block_gram(int64_t S, int64_t D, int k, double const *d_x, double const *d_y, double *d_g,
                      void *stream);
int ls_gpu_block_update(int64_t S, int64_t D, int k, double beta, double const *d_w,
                        double const *d_x1, double const *d_m1, double const *d_x2,
                        double const *d_m2, double *d_out, void *stream);
/* The Gram matrices on the tensor cores (same arguments as ls_gpu_block_gram).  Per tile of 128
 * rows every complex column of X and of Y gets a fixed-point frame above its largest magnitude in
 * the tile; values are cut into eight 7-bit digits (exact bf16), tcgen05 MMAs sum the digit
 * products of equal weight exactly in FP32, and each tile's sums are joined in 64-bit integers,
 * converted to FP64 once and accumulated in FP64 (per-CTA partials added in a fixed order:
 * deterministic).  Each tile adds an error below about 2^-46 2^(E_x + E_y) per entry (128 rows of
 * FP64-exact digit products truncated at weight 2^-56 of the frames 2^E, which are below twice
 * the tile's largest magnitudes), the size of an FP64 dot product's rounding error over the tile.
 * Inputs must be finite.  Stream-ordered (cudaMallocAsync / cudaMemsetAsync of the partials). */
int ls_gpu_block_gram_tc(int64_t S, int64_t D, int k, double const *d_x, double const *d_y,
                         double *d_g, void *stream);
/* The block update on the tensor cores (same arguments and aliasing rules as
 * ls_gpu_block_update).  Each row of [X1 | X2] and each column of [M1; M2] (as real matrices) is
 * put in a fixed-point frame above its largest magnitude and cut into eight 7-bit digits (exact
 * bf16 values); tcgen05 MMAs sum the digit products of equal weight exactly in FP32, and the
 * eight weight groups of an output are combined in 64-bit integers and rounded once to FP64
 * before beta W is added in FP64.  Each output is within about (4k + 2) 2^-54 2^(E_r + E_c) of
 * the exact value, where 2^E_r and 2^E_c (< 2x the largest magnitudes) are the row's and the
 * column's frames: the error bound of an FP64 dot product of the same length.  Inputs must be
 * finite.  Stream-ordered (one cudaMallocAsync for the digit image of M); a wait that times out
 * inside the kernel is reported as LS_GPU_ERR_CUDA by the next matvec call. */
int ls_gpu_block_update_tc(int64_t S, int64_t D, int k, double beta, double const *d_w,
                           double const *d_x1, double const *d_m1, double const *d_x2,
                           double const *d_m2, double *d_out, void *stream);

#if defined(__cplusplus)
} /* extern "C" */
#endif
