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

// Packed projected kernel: real (k = 1) or complex (k in {1, 4, 8, 16}).
int launch_packed(bool cplx, int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L,
                  LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                  const uint64_t* binom, cudaStream_t s);
#define LSG_DECLARE_PACKED(NAME)                                                                  \
  int NAME(int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,      \
           const double* x, int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom, \
           cudaStream_t s);
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
int launch_packed_fermi(bool cplx, int k, int gpl, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,
                        const double* x, int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom,
                        cudaStream_t s);

// Batched multi-sector kernel (complex, k in {1, 4, 8, 16}, gpl in {1, 2, 3, 4}).
struct SectorDesc;
int launch_sectors(int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,
                   const SectorDesc* d_desc, int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy,
                   int* err, const uint64_t* binom, const double* xs_all, int64_t ldxs, int col, cudaStream_t s);
// FP32-pair variant (k in {8, 16}); xs_all holds x_j * n_j of all sectors as float pairs.
int launch_sectors_pair(int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,
                        const SectorDesc* d_desc, int n_sectors, int64_t total_rows, int64_t ldx, int64_t ldy,
                        int* err, const uint64_t* binom, const double* xs_all, int64_t ldxs, int col,
                        cudaStream_t s);
// FP32-pair packed kernels (complex, k in {8, 16}; fermionic groups included); p.xs holds
// x_j * n_j as float pairs.
int launch_packed_pair(int k, int gpl, bool inv, const MatvecProblem& p, const PackedLayout& L, LaunchShape sh,
                       const double* x, int64_t ldx, double* y, int64_t ldy, int* err, const uint64_t* binom,
                       cudaStream_t s);
constexpr int kSectorMaxGpl = 4;
constexpr int kMaxSectors = 256;

// Launch shape of the warp-per-row kernels: threads per block and grid waves (settable).
LaunchShape packed_shape(int64_t n_rows);

// Unprojected / spin-inversion-only kernel.
int launch_plain(bool cplx, bool inv, int k, const MatvecProblem& p, const SmemLayout& L,
                 LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                 const uint64_t* binom, cudaStream_t s);
}  // namespace lsg
