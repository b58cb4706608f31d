// batch.cuh -- batched persistent kernels: many independent SIMP problems of
// uneven sizes advanced by one launch per step.
//
// Every problem of a batch has a BatchItem (its layout, the pointers of its
// arrays inside pooled allocations, its SIMP parameters, tile plans and solver
// scalars).  A kernel family is launched once for the whole batch over a work
// list of (problem, block) pairs; each CTA of the persistent grid loops over the
// work items and runs the same kernel body as the single-problem launch, with
// the per-problem block index and block count, so reductions and last-block
// hand-offs stay per problem.  A problem whose SIMP loop has ended (frozen) or
// whose PCG has converged (done) is skipped.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "am_common.cuh"

namespace amk {

struct BatchItem {
    Layout L;
    // element arrays (x-fastest)
    double *rho, *rho_new, *s64, *ce, *dc, *dcf, *oc_a, *oc_lo, *oc_hi;
    float *s32;
    uint8_t *design;
    // node arrays: [3][cs] vectors, per-node inverse diagonal / mask / constraint bits
    double *F, *x64, *r64, *dinv64;
    float *r32, *pa, *pb, *q32, *dinv32;
    float *xh, *xl;  // the FP32 PCG's iterate as a double-float pair (x64 = xh + xl)
    // padded copies of s32 and mask read by the tensor-copy staged K*u (rows of
    // round_up(nx, 4) scales, round_up(nx+1, 16) constraint bytes)
    float *s32pad;
    uint8_t *maskpad;
    uint8_t *mask, *fixed_bits;
    // nonzeros of F (node-plane index) for u.F and |F|^2
    const long long *f_idx;
    const double *f_val;
    int f_nnz;
    // sensitivity filter taps
    const int4 *tap_d;
    const double *tap_w;
    int ntaps;
    // SIMP parameters
    double penalty, emin, rho_min, move, vf, n_design, tol;
    int maxit;
    // tile plans: FP32 warp-row K*u (ku2) and FP64 tiled K*u
    int k2_tiles_x, k2_tiles_y, k2_tiles_z, k2_tz;
    int k64_tiles_x, k64_tiles_y, k64_tiles_z, k64_tz;
    // blocks per family: ku2 tiles, FP64 tiles, node-vector blocks, element blocks
    int n_k2, n_k64, n_vec, n_elem;
    double *partial;
    Scalars *S;
};

// (problem, block) pairs of one kernel family
struct WorkList {
    const int2 *w;
    int n;
};

// constants shared by every problem of a batch (one h, E0, nu)
struct BatchConst {
    Modal<double> M64;
    Modal<float> M32;
    double d0;  // KE[0][0]: the Jacobi diagonal is d0 * sum of the adjacent scales
};

constexpr int BATCH_VEC_THREADS = 256;

// element scales (C++ rule) and the FP32 copy; per-node inverse diagonal + mask
cudaError_t batch_operator(const BatchItem *it, WorkList elem, WorkList vec, const BatchConst &C, int grid,
                           cudaStream_t st);
// x64 = 0 on masked DOFs (warm start) and |F|^2 over the free DOFs -> S->b2
cudaError_t batch_prepare_solve(const BatchItem *it, WorkList vec, WorkList prob, int grid, cudaStream_t st);
// r64 = mask(F - K x64) (FP64), |r|^2 -> S->res_rr; element energies when energy != 0
cudaError_t batch_resid(const BatchItem *it, WorkList k64, const BatchConst &C, int energy, int grid,
                        cudaStream_t st);
// r32 = r64 and (xh, xl) = x64, then the FP32 PCG start (a problem whose FP64
// residual already meets tol is marked done)
cudaError_t batch_inner_start(const BatchItem *it, WorkList vec, int grid, cudaStream_t st);
// x64 = xh + xl after an FP32 PCG round
cudaError_t batch_inner_end(const BatchItem *it, WorkList vec, int grid, cudaStream_t st);
// one FP32 PCG iteration for every active problem: fused K*p + the bulk-copy
// update over `chunks` ((problem, chunk of 2048 DOFs) items).  warps = 4 or 8: one
// tile height for every problem, tiles in k2; warps = 0: each problem's own, the
// 8-warp problems' tiles in k2 and the 4-warp ones' in k2b
cudaError_t batch_pcg_iteration(const BatchItem *it, WorkList k2, WorkList k2b, WorkList chunks, const BatchConst &C,
                                int warps, int grid_k2, int grid_vec, cudaStream_t st);
// DOFs per chunk of the batched update's work items
constexpr int BATCH_UPD_CHUNK = 2048;
// plain FP32 K*u (y = q32, u = pa) over the batch, for the autotuner
cudaError_t batch_ku_plain(const BatchItem *it, WorkList k2, WorkList k2b, const BatchConst &C, int warps, int grid,
                           cudaStream_t st);
// The tensor-copy staged FP32 PCG K*u of the single-problem solver over a batch
// (ku3.cu): one CTA per (problem, tile) work item of k3, each problem's tensor maps
// and arguments in items; the padded scale and constraint copies it reads are
// refreshed by batch_ku3_pad after every change of the operator or mask.
struct Ku3BatchItem;
cudaError_t batch_ku3_init_attributes();
cudaError_t batch_ku3_pcg(const Ku3BatchItem *items, WorkList k3, const Modal<float> &M, cudaStream_t st);
cudaError_t batch_ku3_pad(const BatchItem *items, WorkList vec, int grid, cudaStream_t st);
// the K*u half of batch_pcg_iteration alone (warp-row kernel)
cudaError_t batch_pcg_ku(const BatchItem *it, WorkList k2, WorkList k2b, const BatchConst &C, int warps, int grid,
                         cudaStream_t st);
// the update half of batch_pcg_iteration alone (after batch_ku3_pcg)
cudaError_t batch_pcg_update(const BatchItem *it, WorkList chunks, int grid_vec, cudaStream_t st);
// sensitivities + u.F, filter, OC bisection (FP64), new density copied into rho
cudaError_t batch_update(const BatchItem *it, WorkList elem, WorkList prob, int grid, cudaStream_t st);

}  // namespace amk
