/*
 * am_gpu.h -- C ABI of the GB300 (sm_103a) SIMP topology-optimisation engine.
 *
 * Drop-in for the solver entry points of the reference engine
 * (ettoremiglioranza1012/AM_ML_suite):
 *   C++  TopologyOptimizer       cpp_engine/include/am/topology_optimizer.hpp:132-169
 *        GlobalAssembler         cpp_engine/include/am/global_assembler.hpp:113-131
 *        LinearSolver            cpp_engine/include/am/linear_solver.hpp:132-172
 *   Py   SIMPOptimizer.run       src/am/numerical/topopt.py:94-133, 266-411
 *        fem.solve_fem etc.      src/am/numerical/fem.py:175-383
 * Inputs are a voxel domain plus load cases; outputs are the density field and
 * the compliance / volume histories.  Every entry point takes caller-owned HOST
 * buffers unless its name ends in _device; device memory lives in the opaque
 * handle.  No entry point throws; each returns an am_status.
 *
 * Layout of host arrays:
 *   densities / grids: AM_LAYOUT_ZFASTEST  e = i*ny*nz + j*nz + k  (C-order (nx,ny,nz);
 *                      fem.py and global_assembler.hpp:162-164), or
 *                      AM_LAYOUT_XFASTEST  e = k*nx*ny + j*nx + i  (topology_optimizer.hpp:218-232,
 *                      am_topopt.cpp:167-171)
 *   DOF vectors (F, u): 3*(i*(ny+1)*(nz+1) + j*(nz+1) + k) + d  (fem.py:168-170,
 *                      global_assembler.cpp:45-50)
 *   grid values: -1 void, 0 design, 1 fixed solid (geometry.py:16-30)
 */
#ifndef AM_GPU_H
#define AM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference throws std::invalid_argument
 * (global_assembler.cpp:73-83, linear_solver.cpp:59-63), std::out_of_range
 * (linear_solver.cpp:69-73) and Python ValueError (fem.py:296-319); a solve that
 * does not converge is a warning plus converged=false (linear_solver.cpp:175-180),
 * which here is AM_OK with the converged flag cleared in the stats. */
typedef enum am_status {
    AM_OK = 0,
    AM_ERR_INVALID_ARG = 1,
    AM_ERR_SIZE_MISMATCH = 2,
    AM_ERR_DOF_OUT_OF_RANGE = 3,
    AM_ERR_NOT_CONVERGED = 4,
    AM_ERR_NAN_DETECTED = 5,
    AM_ERR_SINGULAR = 6,
    AM_ERR_CUDA = 7,
    AM_ERR_TIMEOUT = 8,
    AM_ERR_OOM = 9,
    AM_ERR_NO_DEVICE = 10
} am_status;

enum { AM_LAYOUT_ZFASTEST = 0, AM_LAYOUT_XFASTEST = 1 };

/* Which reference loop the SIMP entry points follow.
 * AM_VARIANT_CPP: TopologyOptimizer (topology_optimizer.cpp:294-520): relative E_min,
 *   elements with rho < rho_min skipped in the stiffness (global_assembler.cpp:147-149),
 *   design mask from the initial density, filter sum w rho dc / sum w rho
 *   (:168-198), OC bisection 1e-20/1e20 to 1e-4 (:205-287), compliance u.F.
 * AM_VARIANT_PY: SIMPOptimizer (topopt.py:266-411): absolute E_min, void/fixed grid
 *   cells, density pre-filter + normalised reflect-mode cone filter, OC bisection
 *   1e-9/1e9 to 1e-3, compliance sum of element energies, several load cases. */
enum { AM_VARIANT_CPP = 0, AM_VARIANT_PY = 1 };

/* AM_PREC_FP64: every kernel in FP64 (the parity mode).
 * AM_PREC_MIXED: FP32 Jacobi PCG (FP32 K*u, r and p, double-float iterate and dot
 *   accumulation) with FP64 residual replacement (AM_MIXED_RELIABLE, the default), or
 *   an FP64 flexible CG preconditioned by FP32 Jacobi-PCG inner solves
 *   (AM_MIXED_FLEXIBLE; always with the learned preconditioner); a solve is
 *   accepted on its recomputed FP64 residual r = f - K u.  Compliance, element
 *   energies, filter and the new densities are FP64; the OC bisection passes run in
 *   double-float. */
enum { AM_PREC_FP64 = 0, AM_PREC_MIXED = 1 };
enum { AM_MIXED_RELIABLE = 0, AM_MIXED_FLEXIBLE = 1 };

/* AM_PRECOND_JACOBI: the diagonal; AM_PRECOND_LEARNED: the network of
 * am_problem_set_preconditioner; AM_PRECOND_MG: a geometric multigrid V-cycle (FP32;
 * rediscretised coarse grids of averaged element scales, trilinear transfers,
 * damped-Jacobi smoothing, dense coarsest solve) inside the FP64 flexible CG, for
 * grids whose dimensions halve down to at most 1000 coarse DOFs -- other grids
 * solve with the Jacobi path.  In place of the reference's IncompleteCholesky
 * (linear_solver.cpp:133-140). */
enum { AM_PRECOND_JACOBI = 0, AM_PRECOND_LEARNED = 1, AM_PRECOND_MG = 2 };

/* SIMP configuration: SIMPConfig (topology_optimizer.hpp:49-59) + SIMPParams
 * (topopt.py:30-52) + the solver knobs of SolverConfig (linear_solver.hpp:66-75). */
typedef struct am_simp_config {
    double volume_fraction;   /* target volume fraction */
    double penalty;           /* SIMP exponent p */
    double filter_radius;     /* rmin in elements */
    double move_limit;
    double rho_min;
    double E_min;             /* relative (CPP) or absolute in units of E0 (PY) */
    double convergence_tol;   /* max |delta rho| */
    int max_iterations;
    int variant;              /* AM_VARIANT_* */
    int precision;            /* AM_PREC_* */
    int preconditioner;       /* AM_PRECOND_* */
    double cg_tol;            /* relative residual ||f - K u|| / ||f|| of every solve */
    int cg_max_iterations;    /* cap on (inner) PCG iterations per solve (100000 by default) */
    int warm_start;           /* 1: each solve starts from the previous displacement */
    double inner_tol;         /* MIXED: residual reduction of the FP32 sequence between two FP64
                                 residual replacements (RELIABLE), or of each FP32 inner solve
                                 that preconditions the flexible CG (FLEXIBLE; it stops at
                                 max(inner_tol |r|, 0.3 cg_tol |f|)); <= 0 (the default) picks
                                 0.1 (RELIABLE) or 0.01 (FLEXIBLE) */
    int max_outer;            /* MIXED: cap on FP64 replacements / outer flexible-CG iterations
                                 per solve */
    int layout;               /* AM_LAYOUT_* of density arrays */
    int verbose;
    int mixed_solver;         /* MIXED with the Jacobi preconditioner: AM_MIXED_* */
    int mg_deflation;         /* AM_PRECOND_MG: 1 (the default) balances the V-cycle with the
                                 rigid-body modes of the passive solid inclusions (elements
                                 held at density 1), whose near-free motion once their
                                 surroundings turn void no coarse grid represents; 0: the
                                 V-cycle alone */
    int cpp_assembly_index;   /* AM_VARIANT_CPP: 1 builds the element stiffness scales the way the
                                 reference C++ engine does, reading the density vector with the
                                 assembler's z-fastest element index (global_assembler.hpp:162-164)
                                 although the optimizer stores it x-fastest
                                 (topology_optimizer.hpp:218-232) -- for replaying runs of
                                 am_topopt; 0 (the default) reads every density at its own element */
} am_simp_config;

/* Per-solve statistics (SolveStats, linear_solver.hpp:48-56). */
typedef struct am_solve_stats {
    int iterations;           /* PCG iterations (sum of inner iterations in MIXED) */
    int outer_iterations;     /* MIXED: FP64 residual replacements or outer flexible-CG
                                 iterations; 1 in FP64 */
    double residual;          /* final ||f - K u|| / ||f||, computed in FP64 */
    int converged;
    double solve_time_s;
    double max_displacement;
    double min_displacement;
    int learned_applications; /* outer iterations preconditioned by the learned network */
} am_solve_stats;

/* IterationResult (topology_optimizer.hpp:65-74) plus the extra fields of this engine. */
typedef struct am_iteration_result {
    double compliance;         /* CPP: u.F ; PY: sum over load cases of element energies */
    double compliance_energy;  /* sum_e scale_e u_e^T KE u_e (both variants) */
    double volume_fraction;    /* mean density over the design mask after the update */
    double max_density_change;
    int solver_iterations;
    int solver_outer_iterations;
    double solver_residual;
    int solver_converged;
    int oc_passes;             /* bisection passes of the OC update */
    double assembly_time_s;    /* scale / diagonal set-up (no global K is assembled) */
    double solve_time_s;
    double sensitivity_time_s;
    double update_time_s;      /* filter + OC */
    int solver_learned_applications; /* outer iterations preconditioned by the learned network */
} am_iteration_result;

typedef struct am_problem am_problem;

/* Human-readable status name; detail of the last error of this thread. */
const char *am_status_string(am_status s);
const char *am_last_error(void);

/* Library / device information.  get_max_threads of the missing Python binding
 * (notebook cells 23-24) maps to the SM count; is_available to a usable device. */
int am_is_available(void);
am_status am_device_info(int *sm_count, size_t *free_bytes, size_t *total_bytes);

/* 24x24 row-major element stiffness of a cube of edge h, material (E, nu), as
 * applied by the kernels (the 2x2x2-Gauss KE of ElementKernel::computeStiffness
 * element_kernel.cpp:155-179 / get_element_stiffness_matrix fem.py:43-135;
 * node order element_kernel.cpp:41-50). */
am_status am_element_stiffness(double E, double nu, double h, double *ke);

/* Fills cfg with the defaults of the chosen variant (SIMPConfig defaults for CPP,
 * SIMPParams defaults for PY), MIXED precision, Jacobi, cg_tol 1e-6. */
void am_simp_config_default(am_simp_config *cfg, int variant);

/* Creates a problem on the current CUDA device: nx*ny*nz cubic elements of edge h,
 * isotropic material (E0, nu).  grid (nullable = all design) uses `layout`.
 * Replaces TopologyOptimizer::TopologyOptimizer (topology_optimizer.cpp:16-53). */
am_status am_problem_create(int nx, int ny, int nz, double h, double E0, double nu,
                            const int8_t *grid, int layout, am_problem **out);
am_status am_problem_destroy(am_problem *p);

/* Load cases: F is n_cases x N (N = 3 (nx+1)(ny+1)(nz+1)), fixed is the
 * concatenation of the constrained DOFs of each case, n_fixed[c] entries for
 * case c.  Replaces LoadCase.get_force_vector / get_constrained_dofs
 * (loads.py:125-156) and the F / fixed_dofs arguments of TopologyOptimizer::run.
 * A DOF index outside [0, N) -> AM_ERR_DOF_OUT_OF_RANGE. */
am_status am_problem_set_loads(am_problem *p, int n_cases, const double *F,
                               const int64_t *fixed, const int64_t *n_fixed);

/* y = K(rho) u for the unconstrained operator (the assembled K of
 * GlobalAssembler::assemble global_assembler.cpp:61-222 / fem.py:175-248, applied
 * matrix-free).  precision AM_PREC_FP64 or AM_PREC_MIXED (FP32 K*u). */
am_status am_ku_apply(am_problem *p, const am_simp_config *cfg, const double *rho,
                      const double *u, double *y, int precision);

/* One K*u step of the FP32 inner PCG on host data (the kernel every inner
 * iteration of am_solve / am_simp_* runs; the product part of the Eigen
 * ConjugateGradient iteration of LinearSolver::solve linear_solver.cpp:136-155):
 * with the operator of rho, its Jacobi diagonal D and the constraint bits of load
 * case `load_case` (fixed and orphan DOFs), p = D^-1 r + beta p_prev and
 * q = mask(K p) in FP32, and *pq = p.q.  Vectors in the reference DOF order, FP64
 * in and out.  impl 3: the kernel the solver uses (tensor-copy staged, a CTA
 * barrier per plane, tensor-store output tiles); impl 4: the staged kernel
 * without a CTA-wide barrier per plane (per-warp-pair mailboxes, per-lane
 * stores); impl 2: the register-direct kernel (all three the same arithmetic,
 * bitwise equal results). */
am_status am_ku_pcg_step(am_problem *p, const am_simp_config *cfg, const double *rho, int load_case,
                         const double *r, const double *p_prev, double beta, int impl, double *p_out,
                         double *q_out, double *pq);

/* Solves K(rho) u = F_case with the constrained and orphan DOFs eliminated
 * (LinearSolver::solveWithBCs linear_solver.cpp:186-203; solve_fem fem.py:251-325).
 * u_out (nullable) receives u in the reference DOF order. */
am_status am_solve(am_problem *p, const am_simp_config *cfg, const double *rho, int load_case,
                   double *u_out, am_solve_stats *stats);

/* Element energies ce = u_e^T KE u_e, sensitivities dc = -p rho^(p-1) ce (CPP:
 * every element, topology_optimizer.cpp:126-161; PY: design elements only,
 * topopt.py:158-198) and the compliance sum_e scale_e ce (fem.py:328-383). */
am_status am_sensitivities(am_problem *p, const am_simp_config *cfg, const double *rho,
                           const double *u, double *dc, double *ce, double *compliance);

/* Filters.  which = 0: C++ sensitivity filter sum w rho dc / sum w rho
 * (topology_optimizer.cpp:60-119,168-198), x = dc, rho used;
 * which = 1: Python normalised cone convolution, reflect boundary
 * (topopt.py:135-156), rho ignored. */
am_status am_filter(am_problem *p, const am_simp_config *cfg, int which, const double *x,
                    const double *rho, double *out);

/* OC update of the chosen variant (topology_optimizer.cpp:205-287 /
 * topopt.py:200-264).  design[e] != 0 marks design elements.  Outputs the new
 * density, max |change| and the bisection pass count. */
am_status am_oc_update(am_problem *p, const am_simp_config *cfg, const double *rho,
                       const double *dc, const uint8_t *design, double *rho_new,
                       double *max_change, int *passes);

/* Full SIMP run (TopologyOptimizer::run topology_optimizer.cpp:391-520 /
 * SIMPOptimizer.run topopt.py:266-411).  rho0 (nullable: volume_fraction
 * everywhere, CPP keeps fixed / void cells at 1 / rho_min) in cfg->layout.
 * Histories need room for cfg->max_iterations entries; change_hist nullable. */
am_status am_simp_run(am_problem *p, const am_simp_config *cfg, const double *rho0,
                      double *rho_out, double *compliance_hist, double *volume_hist,
                      double *change_hist, int *iterations, int *converged);

/* Stepwise form of the same loop on device-resident state:
 * am_simp_begin uploads rho0 and builds the design mask / filter;
 * am_simp_step runs one iteration (TopologyOptimizer::runIteration
 * topology_optimizer.cpp:294-384); am_simp_get_density downloads rho. */
am_status am_simp_begin(am_problem *p, const am_simp_config *cfg, const double *rho0);
am_status am_simp_step(am_problem *p, am_iteration_result *res);
am_status am_simp_get_density(am_problem *p, double *rho_out);

/* ---- measurement (no counterpart in the reference, whose timers are the
 * std::chrono phase times of IterationResult, topology_optimizer.hpp:65-74) ---- */

/* Self-test of the bounded copy waits (no reference counterpart).  Every stage
 * of the solver's copy pipelines waits on its barrier for at most one second and
 * then ends the solve with an error instead of spinning; this launches one
 * thread that waits, with the same code shortened to limit_ms (0 < limit_ms <=
 * 100), on a barrier that nothing completes.  *timed_out = 1 and *waited_ms about
 * limit_ms when the wait gave up as it should. */
am_status am_selftest_copy_wait(double limit_ms, int *timed_out, double *waited_ms);

/* Self-test of the status a solve returns when one of its kernels reports that a
 * bounded copy wait ran out (no reference counterpart).  No wait is made to run
 * out: the flag such a kernel sets is set on the host before the first PCG
 * chunk of am_solve(p, cfg, rho, load_case); every kernel then completes
 * normally and the PCG ends at its first update with the timeout status.
 * *solve_status receives what am_solve returned (AM_ERR_TIMEOUT), and the flag
 * is cleared again so the problem stays usable. */
am_status am_selftest_solve_timeout(am_problem *p, const am_simp_config *cfg, const double *rho, int load_case,
                                    int *solve_status);

/* Kernel launches this library has issued so far (CUDA-graph replays add the
 * kernel nodes they contain). */
long long am_launch_count(void);

/* Times `reps` single launches of one kernel on the problem's stream with CUDA
 * events, after am_simp_begin (on the state the last am_simp_step left, or, before
 * the first step, on the initial density with zero vectors): which = 0 the
 * fused FP32 PCG K*u the solver runs (tensor-copy staged, 4 stages, a CTA
 * barrier per plane), 12 the same kernel, 13 the staged kernel without a
 * CTA-wide barrier per plane (4 stages), 1 the FP64
 * residual K*u, 2 the FP32 PCG vector update, 3 the plain FP32 K*u, 4 the
 * register-direct FP32 PCG K*u it replaced, 5 the staged kernel with 3 stages (8-warp tiles),
 * 14 the double-float residual of the mixed solvers (1 is its FP64 form),
 * 6 / 7 the FP32 PCG vector update of an even (residual only) / odd (residual
 * and folded iterate) iteration, 8 the C++ cone sensitivity filter
 * (shared-memory stencil), 9 one OC bisection pass (double-float) -- these two
 * on the state of the last am_simp_step --, 10 one multigrid V-cycle and 11 the
 * V-cycle balanced by the rigid-body modes of the passive solid inclusions (both
 * a sequence of launches, timed as a whole).  flush_l2 != 0 overwrites a 512 MB buffer before each
 * launch so the kernel reads from HBM, then reads that buffer back so the write's
 * dirty L2 lines are written back before the timed launch.  Solver state is restored afterwards. */
am_status am_bench_kernel(am_problem *p, int which, int reps, int flush_l2, double *avg_ms, double *min_ms);

/* The CUDA stream (cudaStream_t) on which every kernel of the problem runs, for
 * callers that order their own work after it or time it with CUDA events.  The
 * reference has no counterpart (its solves are synchronous CPU calls). */
am_status am_problem_stream(am_problem *p, void **stream);

/* Sizes of the device layout: reference node count, element count, the padded
 * component stride of a device vector, and the K*u tile count. */
am_status am_problem_layout(am_problem *p, long long *nodes, long long *elements, long long *vector_stride,
                            int *ku_tiles);

/* ---- learned preconditioner -------------------------------------------------------
 * No counterpart in the reference (its am.ai package is an unrelated placeholder,
 * src/am/ai/model.py:18-67).  A 3-D convolutional encoder-decoder on the node grid
 * (4 levels, 16/32/64/128 channels, 3x3x3 kernels, skip connections, 1,461,456
 * BF16 weights, FP32 accumulate) maps a residual r (and the node densities) to
 * z ~ K^-1 r.  It works on the Jacobi-scaled system D^-1/2 K D^-1/2 and adds its
 * output to the Jacobi step, so the untrained network is Jacobi.  Training
 * minimises |K z - r|^2 / |r|^2 in that scaling, on residuals harvested from the
 * engine's own Jacobi PCG solves, with Adam on FP32 master weights; forward and
 * backward run on the GPU's tensor cores (conv3d.cu). */
typedef struct am_precond am_precond;

typedef struct am_train_config {
    int epochs;
    int batch;        /* samples per Adam step */
    float lr;         /* 1e-3 */
    float beta1, beta2, eps;
    uint64_t seed;    /* sample order */
    int verbose;
    int loss;         /* 0: |K z - r|^2 / |r|^2 (residual norm); 1: 1 - (z.r)^2 / ((z.Kz)(e.r)),
                         e = K^-1 r the harvested error: the share of the error energy
                         that the best multiple of z misses */
} am_train_config;

/* seed: weight initialisation; capacity: training samples the set can hold. */
am_status am_precond_create(uint64_t seed, long long capacity, am_precond **out);
am_status am_precond_destroy(am_precond *m);
long long am_precond_num_params(am_precond *m);
long long am_precond_num_samples(am_precond *m);
/* FP32 master weights, layer by layer, each [27 taps][cout][cin]. */
am_status am_precond_get_params(am_precond *m, float *w);
am_status am_precond_set_params(am_precond *m, const float *w);
/* Network on host tensors [n][gz][gy][gx][4] -> [n][gz][gy][gx][3] (grid dims
 * multiples of 8), and the weight gradient of sum(out * dout); for inspection and
 * gradient checks. */
am_status am_precond_forward(am_precond *m, int n, int gz, int gy, int gx, const float *in, float *out);
am_status am_precond_param_grad(am_precond *m, int n, int gz, int gy, int gx, const float *in, const float *dout,
                                float *grad);
/* Times `reps` forward passes of the network on an n x gz x gy x gx device tensor
 * (multiples of 8) with CUDA events; *flops = the convolutions' 2*27*cin*cout per
 * voxel summed over the layers (measurement; no reference counterpart). */
am_status am_precond_bench_forward(am_precond *m, int n, int gz, int gy, int gx, int reps, double *avg_ms,
                                   double *flops);
/* Selects the kernels of every convolution of the network, process-wide:
 * impl 1 (the default) tcgen05.mma with tensor-memory accumulators and tiled
 * tensor-copy staging; impl 0 the legacy mma.sync/ldmatrix/cp.async kernels,
 * kept as the baseline the tensor-core kernels are checked and timed against.
 * A tensor-core convolution whose bounded wait runs out makes the call that ran
 * it return AM_ERR_TIMEOUT. */
am_status am_precond_set_kernels(int impl);
/* Adds training samples: at density rho (host, cfg->layout) the problem's FP32
 * Jacobi PCG runs from u = 0 on load case `load_case`; the residual r_k and the
 * error e_k = u* - u_k after each iteration count k in iters[0..n_iters)
 * (ascending; 0 = the load itself) form a sample, u* from an FP64-accepted solve
 * to 1e-10.  All samples of one preconditioner come from one grid size. */
am_status am_precond_harvest(am_precond *m, am_problem *p, const am_simp_config *cfg, const double *rho,
                             int load_case, const int *iters, int n_iters);
/* Adam over the samples for cfg->epochs; epoch_loss[e] (nullable) the mean loss. */
am_status am_precond_train(am_precond *m, const am_train_config *cfg, float *epoch_loss);
/* Mean loss (loss: as in am_train_config) over samples [first, first + count). */
am_status am_precond_eval(am_precond *m, long long first, long long count, int loss, double *mean_loss);
/* Solves of `p` with preconditioner AM_PRECOND_LEARNED use `m` (NULL detaches):
 * FP64 flexible CG whose preconditioner is the network's z = M(r) refined by FP32
 * Jacobi PCG on r - K z to inner_tol; if the residual stops falling (less than
 * 10 % over 5 outer iterations) the solve continues with Jacobi PCG alone.  The
 * FP64 residual accepts every solve, as with Jacobi. */
am_status am_problem_set_preconditioner(am_problem *p, am_precond *m);

/* How an inner FP32 (or FP64) PCG solve is driven.  on != 0 (the default): one
 * CUDA-graph launch per solve, a device-side while loop over chunks of 32
 * iterations that ends when the solve ends or after maxit / 32 + 4 chunks; the
 * host waits once.  on == 0: one graph launch per chunk, the host reading the
 * solver state between chunks.  Both run the same kernels in the same order (same
 * results); no reference counterpart (Eigen's CG loop runs on the host,
 * linear_solver.cpp:136-155). */
am_status am_problem_set_device_loop(am_problem *p, int on);

/* The tile height of the FP32 inner PCG's staged K*u (tiles of 28 node columns and
 * 2 warps - 1 node rows).  warps 0 (the default): 7 warps where the 7-warp tiles'
 * one-wave plan keeps more CTA slots busy than the 8-warp tiles' (the 256x128x128
 * cantilever: 300 tiles against 270), else 8; 7 or 8 pins it.  Every choice gives
 * the same p and q; p.q is summed over different tiles.  The barrier-free
 * measurement kernel (am_ku_pcg_step impl 4, am_bench_kernel 13) needs 8-warp tiles.
 * No reference counterpart. */
am_status am_problem_set_ku_plan(am_problem *p, int warps);
/* The staged K*u's plan in use: warps per tile, tiles per launch, node planes per
 * z chunk (each nullable). */
am_status am_problem_get_ku_plan(am_problem *p, int *warps, int *tiles, int *z_chunk);

/* The arithmetic of the residuals r = mask(f - K u) (with the element energies)
 * that the mixed-precision solvers (AM_PREC_MIXED) recompute at every residual
 * replacement and accept a solve on.  AM_RESID_DOUBLE_FLOAT (the default): the
 * element operator and node sums as double-float pairs on the FP32 pipes (~48
 * significant bits; FP64 inputs, outputs and dot products), several times faster
 * than FP64 on GB300; AM_RESID_FP64: the FP64 kernel.  AM_PREC_FP64 solves always
 * use the FP64 kernel.  No reference counterpart (the reference solves in FP64). */
enum { AM_RESID_DOUBLE_FLOAT = 0, AM_RESID_FP64 = 1 };
am_status am_problem_set_residual_arithmetic(am_problem *p, int mode);

/* ---- density-predicting U-Net (the reference's am.ai TopOptUNet) -----------------------
 * A 3-D U-Net predicting the optimised density field from a problem encoding: the
 * network the reference declares in src/am/ai/model.py:18-67 (in_channels 4,
 * out_channels 1, features (32, 64, 128, 256)) and leaves unimplemented.  Four levels
 * of width f0, 2 f0, 4 f0, 8 f0 (two 3x3x3 convolutions + ReLU each), mean pooling
 * down, nearest upsampling up, concatenated skips, a 3x3x3 output convolution and a
 * sigmoid; BF16 weights and activations, FP32 accumulate, on the tensor cores.
 * Tensors are channels-last [n][gz][gy][gx][c] on grids whose dimensions are
 * multiples of 8. */
typedef struct am_unet am_unet;

/* 1 <= in_channels, out_channels <= 16; f0 = 16 or 32. */
am_status am_unet_create(int in_channels, int out_channels, int f0, uint64_t seed, am_unet **out);
am_status am_unet_destroy(am_unet *u);
long long am_unet_num_params(am_unet *u);
/* FP32 master weights, layer by layer, each [27 taps][cout][cin] (channels padded to 16). */
am_status am_unet_get_params(am_unet *u, float *w);
am_status am_unet_set_params(am_unet *u, const float *w);
/* in [n][gz][gy][gx][in_channels] -> out [n][gz][gy][gx][out_channels] (sigmoid != 0:
 * the sigmoid of the output, else the raw output). */
am_status am_unet_forward(am_unet *u, int n, int gz, int gy, int gx, const float *in, float *out, int sigmoid);
/* Weight gradient of sum(raw output * dout) (for gradient checks). */
am_status am_unet_param_grad(am_unet *u, int n, int gz, int gy, int gx, const float *in, const float *dout,
                             float *grad);
/* Training set on the device: inputs [S][gz][gy][gx][in_channels], target densities
 * [S][gz][gy][gx], mask [S][gz][gy][gx] (nonzero: the cell counts in the loss). */
am_status am_unet_set_data(am_unet *u, int n_samples, int gz, int gy, int gx, const float *inputs,
                           const float *targets, const uint8_t *mask);
/* Adam on the binary cross-entropy of the sigmoid output against the target
 * densities over the masked cells; epoch_loss (nullable) receives each epoch's mean
 * squared error of the sigmoid output.  cfg->loss unused. */
am_status am_unet_train(am_unet *u, const am_train_config *cfg, float *epoch_loss);
/* Mean squared error over the whole training set. */
am_status am_unet_eval(am_unet *u, double *mse);

/* ---- batched SIMP ---------------------------------------------------------------
 * Many independent C++-variant problems of uneven sizes run together: one launch
 * of each kernel family per step for the whole batch (persistent CTAs over a
 * (problem, block) work list), FP32 Jacobi-PCG iterations in CUDA-graph chunks,
 * FP64 defect correction to each problem's cg_tol, FP64 OC.  The reference runs
 * one TopologyOptimizer per problem (topology_optimizer.hpp:132-169); per problem
 * the results follow TopologyOptimizer::run (topology_optimizer.cpp:391-520). */
typedef struct am_batch am_batch;

/* n problems on the current device; problem i has shapes[3i] x shapes[3i+1] x
 * shapes[3i+2] cubic elements of edge h; material (E0, nu) is shared.  Each
 * problem is stored in the axis order in which the batched K*u's tiles (30 node
 * columns x 15 node rows) overhang its grid least.  That is exact for cubic
 * elements, the cone filter and the OC step when the displacement components
 * are permuted with the axes.  Loads, constraints and densities cross this
 * boundary in the caller's order (am_batch_axes reports the order chosen). */
am_status am_batch_create(int n, const int *shapes, double h, double E0, double nu, am_batch **out);
am_status am_batch_destroy(am_batch *b);
/* The internal axis order of problem i: axes[a] is the caller's axis (0 = x,
 * 1 = y, 2 = z) that the batch stores as its axis a (a = 0 is the tiles' 30-column
 * axis).  No reference counterpart. */
am_status am_batch_axes(am_batch *b, int i, int *axes);

/* One load case per problem: F concatenates the problems' force vectors
 * (3 (nx+1)(ny+1)(nz+1) entries each, reference DOF order), fixed their
 * constrained-DOF lists, n_fixed[i] entries for problem i. */
am_status am_batch_set_loads(am_batch *b, const double *F, const int64_t *fixed, const int64_t *n_fixed);

/* Autotuner of the batched FP32 K*u: times `reps` launches of each candidate plan
 * (4 or 8 warps per CTA for every problem, or -- warps 0 -- per problem the tile
 * height that computes fewer element slots on its grid; z chunks of 8, 16 or all
 * node planes; 1-4 CTAs per SM in the persistent grid) and keeps the fastest for
 * the following runs.  Outputs (nullable) the chosen plan and its time per launch. */
am_status am_batch_autotune(am_batch *b, int reps, int *warps, int *z_chunk, int *ctas_per_sm, double *best_ms);
/* Pins a plan of the batched FP32 K*u without timing: warps 0 (per problem), 4 or 8;
 * z_chunk 0 (all planes) or >= 1; ctas_per_sm 1-4. */
am_status am_batch_set_plan(am_batch *b, int warps, int z_chunk, int ctas_per_sm);

/* Which kernel runs the batch's FP32 PCG K*u.  on != 0 (the default): the
 * single-problem solver's tensor-copy staged kernel, one CTA per tile of 28 x 15
 * nodes over all of a problem's planes, each problem's tensor maps in device
 * memory; 0: the warp-row kernel with the plan of am_batch_autotune /
 * am_batch_set_plan.  Both compute the same p and q.  No reference counterpart. */
am_status am_batch_set_staged(am_batch *b, int on);
/* Times the batch's FP32 PCG K*u (the kernel am_batch_set_staged selects) with CUDA
 * events over `reps` launches after one warm-up, every problem iterating, on the
 * residual and densities the last am_batch_simp_step left; the solver state is
 * restored afterwards.  Measurement only; no reference counterpart. */
am_status am_batch_bench_ku(am_batch *b, int reps, double *avg_ms);

/* The CUDA stream the batch's kernels run on (cudaStream_t). */
am_status am_batch_stream(am_batch *b, void **stream);

/* As am_problem_set_device_loop, for the batch's FP32 PCG rounds: on != 0 (the
 * default) each round's chunks run in one graph launch whose device-side while
 * loop ends when no problem is iterating (or at the chunk cap); on == 0 the host
 * checks every problem between chunks. */
am_status am_batch_set_device_loop(am_batch *b, int on);

/* Starts every problem's SIMP loop with its own config cfgs[i] (variant must be
 * AM_VARIANT_CPP); rho0 as for am_batch_simp_run.  Resets the solver state. */
am_status am_batch_simp_begin(am_batch *b, const am_simp_config *cfgs, const double *rho0);

/* One SIMP iteration of every problem whose loop has not ended (runIteration,
 * topology_optimizer.cpp:294-384).  compliance / volume / change (nullable, [n])
 * receive the stepped problems' results, pcg_iterations (nullable, [n]) each
 * problem's FP32 PCG iterations since am_batch_simp_begin, *n_active the problems
 * still running. */
am_status am_batch_simp_step(am_batch *b, double *compliance, double *volume, double *change,
                             long long *pcg_iterations, int *n_active);

/* Current densities of all problems, concatenated, each in its config's layout. */
am_status am_batch_get_density(am_batch *b, double *rho_out);

/* Runs every problem's SIMP loop with its own config cfgs[i] (variant must be
 * AM_VARIANT_CPP; the solve is FP32 Jacobi PCG inside FP64 defect correction to
 * cfgs[i].cg_tol).  rho0 concatenates the initial densities in each config's
 * layout (NULL: volume_fraction everywhere); rho_out receives the final ones.
 * Histories (nullable) are [n][H], H = max_i cfgs[i].max_iterations, entries past
 * a problem's last iteration untouched; iterations[i], converged[i] and
 * pcg_iterations[i] (total FP32 PCG iterations) are per problem (nullable). */
am_status am_batch_simp_run(am_batch *b, const am_simp_config *cfgs, const double *rho0, double *rho_out,
                            double *compliance_hist, double *volume_hist, int *iterations, int *converged,
                            long long *pcg_iterations);

/* ---- problem set-up: the reference's BRK-A-01 bracket ------------------------------
 * The voxel grid of create_bracket_domain (src/am/core/geometry.py:79-196; the C++
 * driver's BracketDomain, cpp_engine/src/am_topopt.cpp:98-239) and the loads of
 * create_brk_a_01_static_case_1/2 (src/am/core/loads.py:163-306; createForceVector /
 * createFixedDofs, am_topopt.cpp:248-334), computed by device kernels and returned
 * in caller-owned host buffers, identical cell for cell and DOF for DOF to the
 * reference's. */
typedef struct am_bracket_params {
    double size_mm[3];          /* bounding box (x, y, z) */
    double resolution_mm;       /* voxel edge */
    double base_thickness_mm;   /* flange: fixed element layers int(t / res), at least 1 */
    double hole_diameter_mm;    /* four void holes through the flange ... */
    double hole_offset_mm;      /* ... int(offset / res) elements from the x and y edges */
    double eyelet_diameter_mm;  /* void hole of the eyelet (axis along z at (nx/2, ny/2)) */
    double eyelet_offset_mm;    /* fixed ring of material around it; also the pillar radius */
    double eyelet_z_offset_mm;  /* eyelet centre below the top */
    double eyelet_height_mm;    /* eyelet extent in z */
    int nx, ny, nz;             /* grid (the reference: int(size_mm / resolution_mm) per axis;
                                   the load builders take the caller's domain shape) */
} am_bracket_params;

/* The reference defaults (geometry.py:79-86, am_topopt.cpp:47-63) at the given
 * resolution, with nx, ny, nz = int(size_mm / resolution_mm). */
void am_bracket_params_default(am_bracket_params *p, double resolution_mm);

/* Every output is nullable.  grid: nx*ny*nz cells -1 void / 0 design / 1 fixed in
 * `layout`.  F: 3 (nx+1)(ny+1)(nz+1) forces in the reference DOF order,
 * total_force[3] spread evenly over the load ring of the eyelet (static case 1:
 * (0, 0, -15000); case 2: (10000 sin 30, 0, -10000 cos 30) computed by the caller).
 * fixed / n_fixed: the 3 (nx+1)(ny+1) DOFs of the nodes at z = 0, ascending.
 * load_nodes / n_load_nodes: the ring's node indices in the reference's loop order
 * (load_nodes_capacity entries available; too few -> AM_ERR_SIZE_MISMATCH). */
am_status am_bracket_build(const am_bracket_params *p, const double total_force[3], int layout, int8_t *grid,
                           double *F, int64_t *fixed, int64_t *n_fixed, int64_t *load_nodes,
                           int64_t *n_load_nodes, int64_t load_nodes_capacity);

/* ---- result writers (host only) ----------------------------------------------------
 * The output files of the reference's C++ driver (cpp_engine/src/am_topopt.cpp), with
 * its formats: numbers as a default C++ stream prints them (6 significant digits). */

/* density_field.npy: NumPy v1.0, '<f8', C order (nx, ny, nz) (saveNpy, :344-396);
 * rho in `layout`. */
am_status am_write_density_npy(const char *path, const double *rho, int nx, int ny, int nz, int layout);

/* history.csv: "iteration,compliance,volume" then one line per iteration (:622-629). */
am_status am_write_history_csv(const char *path, const double *compliance, const double *volume, int n);

/* metadata.json fields (saveMetadata, :401-447). */
typedef struct am_run_metadata {
    const char *case_name, *mode, *provenance;   /* e.g. "BRK-A-01", "cpp_standalone", "cpp_hpc_engine" */
    double resolution_mm;
    int nx, ny, nz;
    long long n_elements, n_design, n_fixed, n_void;
    double volume_fraction_target;
    int has_history;                             /* 1: write the two *_final fields */
    double volume_fraction_final, compliance_final;
    int iterations, converged;
    double elapsed_time_s;
    int threads;                                 /* written as "openmp_threads" */
    double filter_radius, E_min, penalty, move_limit;
} am_run_metadata;
am_status am_write_metadata_json(const char *path, const am_run_metadata *m);

/* ---- allocation-free residual (no counterpart in the reference) ----------------
 * For callers that cannot allocate device memory once they are running -- code
 * inside another framework's fixed memory pool, allocation-free real-time or
 * certified loops, plugins whose host owns every buffer -- and so cannot use the
 * handle API above (am_problem_create allocates a workspace).
 *
 * Computes, in FP64 on the current device, r = f - K(scale) u with the
 * constrained components of r set to 0, and rr = |r|^2, for an nx*ny*nz grid of
 * cubic hex8 elements of edge h and material (E0, nu).  Every argument is a
 * caller-owned DEVICE buffer in the compact layout:
 *   u, f, r : three component planes of (nx+1)(ny+1)(nz+1) nodes each, node
 *             (ix,iy,iz) at (iz*(ny+1) + iy)*(nx+1) + ix of its plane;
 *   scale   : nx*ny*nz element stiffness factors, element (ex,ey,ez) at
 *             (ez*ny + ey)*nx + ex (0 removes an element);
 *   mask    : one byte per node, bit c set = component c constrained;
 *   rr      : one double.
 * The call is asynchronous on `stream` (a cudaStream_t, NULL = default stream);
 * results are ready when the stream reaches that point.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: its scratch (per-tile partial sums and
 * a block of solver scalars, 512 KB in total) is a file-scope __device__ array
 * present on every device that loads the library until the process exits.  The
 * first call on a device looks up that array's device address with the device
 * current (this may load the library's device code); make the first call on each
 * device before any stream capture.  Every call shares the scratch and the
 * previous call's contents remain in it, so calls whose executions overlap on the
 * GPU (different streams, or host threads) race; the call clears what must start
 * at zero.  Limit: ceil((nx+1)/32) * ceil((ny+1)/4) <= 32768 (for example
 * 1023 x 4095 x any nz); larger grids return AM_ERR_SIZE_MISMATCH before any
 * device work.  Errors are read with am_last_error(). */
am_status am_residual_noalloc(int nx, int ny, int nz, double h, double E0, double nu, const double *scale,
                              const double *u, const double *f, const uint8_t *mask, double *r, double *rr,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif /* AM_GPU_H */
