// matvec_dispatch.h -- per-translation-unit launchers of the gather kernels.
#pragma once
#include "lsg.h"

namespace lsg {
struct SmemLayout;
struct LaunchShape {
  int blocks;
  int threads;
};
// Returns 0 on success, LS_GPU_ERR_INVALID when no instantiation matches.
int launch_projected_real(int gpl, bool inv, const MatvecProblem& p, const SmemLayout& L,
                          LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy,
                          int* err, const uint64_t* binom, cudaStream_t s);
int launch_projected_cplx(int gpl, bool inv, int k, const MatvecProblem& p, const SmemLayout& L,
                          LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy,
                          int* err, const uint64_t* binom, cudaStream_t s);
int launch_plain(bool cplx, bool inv, int k, const MatvecProblem& p, const SmemLayout& L,
                 LaunchShape sh, const double* x, int64_t ldx, double* y, int64_t ldy, int* err,
                 const uint64_t* binom, cudaStream_t s);
// group elements per lane supported by the projected kernels (ascending)
constexpr int kGplChoices[] = {1, 2, 3, 4, 6, 9, 12, 16};
}  // namespace lsg
