// matvec_dispatch.h -- per-translation-unit launchers of the gather kernels.
#pragma once
#include "lsg.h"

namespace lsg {
struct SmemLayout;
struct PackedLayout;
struct LaunchShape {
  int blocks;
  int threads;
};
// All return 0 on success, LS_GPU_ERR_INVALID when no instantiation matches.

// Fallback projected kernel (no packing), one right-hand side.
int launch_projected_real(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L,
                          LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy,
                          int* err, const uint64_t* binom, cudaStream_t s);
int launch_projected_cplx_k1(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L,
                             LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy,
                             int* err, const uint64_t* binom, cudaStream_t s);

// Packed projected kernel: real (k = 1) or complex (k in {1, 4, 8, 16}).  The packed launchers
// pick their own launch shape and shared-memory layout (packed_launch_shape).
int launch_packed(bool cplx, int k, int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx,
                  double* y, int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s);
#define LSG_DECLARE_PACKED(NAME)                                                                  \
  int NAME(int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx, double* y,    \
           int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s);
LSG_DECLARE_PACKED(launch_packed_real)
LSG_DECLARE_PACKED(launch_packed_real_k2)
LSG_DECLARE_PACKED(launch_packed_real_k4)
LSG_DECLARE_PACKED(launch_packed_real_k8)
LSG_DECLARE_PACKED(launch_packed_real_k16)
LSG_DECLARE_PACKED(launch_packed_cplx_k1)
LSG_DECLARE_PACKED(launch_packed_cplx_k4)
LSG_DECLARE_PACKED(launch_packed_cplx_k8)
LSG_DECLARE_PACKED(launch_packed_cplx_k16)

// Packed kernel for fermionic groups (gpl <= 4): real (k = 1) or complex (k in {1, 4, 8, 16}).
int launch_packed_fermi(bool cplx, int k, int gpl, const MatvecProblem& p, const double* x, int64_t ldx, double* y,
                        int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s);

// Batched multi-sector kernel (complex, k in {1, 4, 8, 16}, gpl in {1, 2, 3, 4}).
struct SectorDesc;
int launch_sectors(int k, int gpl, bool inv, const MatvecProblem& p, int n_sectors_layout, const SectorDesc* d_desc, int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy,
                   int* err, const uint64_t* binom, const double* xs_all, int64_t ldxs, int col, cudaStream_t s);
// FP32-pair variant (k in {8, 16}); xs_all holds x_j * n_j of all sectors as float pairs.
int launch_sectors_pair(int k, int gpl, bool inv, const MatvecProblem& p, int n_sectors_layout,
                        const SectorDesc* d_desc, int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy,
                        int* err, const uint64_t* binom, const double* xs_all, int64_t ldxs, int col,
                        cudaStream_t s);
// FP32-pair packed kernels (complex, k in {8, 16}; fermionic groups included); p.xs holds
// x_j * n_j as float pairs.
int launch_packed_pair(int k, int gpl, bool inv, const MatvecProblem& p, const double* x, int64_t ldx, double* y,
                       int64_t ldy, int* err, const uint64_t* binom, cudaStream_t s);
constexpr int kSectorMaxGpl = 4;
constexpr int kMaxSectors = 256;

// Launch shape of a packed kernel `kern` (compiled for at most max_threads threads per CTA) over
// `rows` rows: the configured thread count (default: max_threads) lowered until the layout fits
// in shared memory and a CTA is resident; a grid of SMs x resident CTAs per SM x waves.  Sets the
// kernel's dynamic shared-memory limit.  n_sectors > 0 for the batched kernel's layout.
int packed_launch_shape(const void* kern, int max_threads, const MatvecProblem& p, int n_sectors, int64_t rows,
                        LaunchShape* sh, PackedLayout* L);
// Largest dynamic shared memory of one CTA (sm_103: 227 KB opt-in).
constexpr size_t kMaxDynamicSmem = 227 * 1024;

// Unprojected / spin-inversion-only kernel.
int launch_plain(bool cplx, bool inv, int k, const MatvecProblem& p, const SmemLayout& L,
                 LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                 const uint64_t* binom, cudaStream_t s);
}  // namespace lsg
