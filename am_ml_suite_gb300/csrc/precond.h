// precond.h -- internal interface between the SIMP engine (am_gpu.cu) and the
// learned preconditioner (precond.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/am_gpu.h"
#include "am_common.cuh"

namespace amk {

// What the preconditioner reads of a problem: its layout, Jacobi diagonal, DOF
// mask and element densities (all device, internal layouts).
struct PrecondView {
    Layout L;
    const float *dinv32;    // per node; 0 on orphan nodes
    const uint8_t *mask;    // per node, bit c = component c constrained / orphan
    const double *rho;      // per element
    cudaStream_t st;
};

// z = M(r): the network's approximation of K^{-1} r (r, z device vectors [3][cs])
am_status precond_apply(am_precond *m, const PrecondView &v, const double *r, double *z);

// Training data: one density (its FP32 element scales and the operator
// constants) then residual snapshots at that density.  The first density fixes
// the training grid; later ones must have the same layout.
am_status precond_add_density(am_precond *m, const PrecondView &v, const Modal<float> &M32, const float *s32,
                              int *density_id);
// r32: the residual of the iterate xk (nullable) whose exact solution is xstar
// (nullable); with both, the sample also stores the error xstar - xk.
am_status precond_add_sample(am_precond *m, int density_id, const float *r32, const double *xk, const double *xstar,
                             cudaStream_t st);

}  // namespace amk
