// mg.h -- geometric multigrid V-cycle preconditioner for the hex8 operator.
//
// Levels halve the element grid in every direction while all three dimensions
// are even and the level has more than MG_COARSE_DOFS degrees of freedom.  A
// coarse element's scale is the mean of its eight children (rediscretisation:
// the coarse operator is K of the coarse grid, element edge 2h); a coarse node
// is constrained where the coincident fine node is fixed, and orphan coarse
// DOFs (no stiffness) are masked like fine ones.  Transfers are trilinear
// prolongation P and full weighting R = P^T.  Smoothing is damped Jacobi
// (omega 0.6, two sweeps before and after the coarse correction), the coarsest
// level is solved exactly with a dense inverse (Cholesky on the host, once per
// operator).  The V-cycle runs in FP32 with the engine's K*u kernels; it is a
// fixed symmetric positive definite operator, used inside the FP64 flexible CG.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "am_common.cuh"

namespace amk {

constexpr int MG_COARSE_DOFS = 200;   // coarsen while a level has more DOFs than this
constexpr int MG_DENSE_MAX = 1000;    // largest coarsest level solved densely

struct Mg;

// The hierarchy for a grid L0 of edge h (material E0, nu), or nullptr if the grid
// cannot be coarsened to at most MG_DENSE_MAX coarse DOFs (*err = cudaSuccess)
// or on an allocation failure (*err set).
Mg *mg_create(const Layout &L0, double E0, double nu, double h, cudaError_t *err);
void mg_destroy(Mg *m);
int mg_num_levels(const Mg *m);

// Builds the level operators for the fine operator: element scales s64 / s32,
// inverse diagonal dinv32 and constraint bits mask (fixed and orphan DOFs) of
// the fine grid, and the fine load case's fixed bits (per node, bit c =
// component c; nullptr: none).  Synchronises the stream (the coarsest level is
// factorised on the host).
cudaError_t mg_setup(Mg *m, const double *s64, const float *s32, const float *dinv32, const uint8_t *mask,
                     const uint8_t *fixed_bits, cudaStream_t st);

// z = M r for FP64 vectors in the device layout of the fine grid.
cudaError_t mg_apply(Mg *m, const double *r, double *z, cudaStream_t st);

}  // namespace amk
