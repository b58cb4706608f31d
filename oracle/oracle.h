/*
 * oracle.h -- FP64 CPU restatement of the reference SIMP inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle of the CUDA path's tests:
 * only tests/, __graft_entry__.smoke() and the cpu_baseline / reference arm of
 * bench.py may load it.  The product library (libamgpu.so) never links or
 * calls it, and has no CPU fallback.
 *
 * Pinning: KE, the DOF map, K*u, the Python solve/compliance/filter/OC and a
 * 5-iteration Python SIMP history are checked against vectors generated by
 * importing the reference Python package (tests/golden/make_golden.py).  The
 * C++-variant filter/OC/sensitivity rules (which need Eigen to build) are
 * checked against the reference's own recorded C++ run outputs (notebook
 * debug run history and data/cpp_test_run history/density), replayed with the
 * reference's element-index convention.
 *
 * Layout used by every function here (the reference's Python / assembler
 * convention):
 *   element e = i*ny*nz + j*nz + k          (C-order (nx,ny,nz), z fastest)
 *   node    n = i*(ny+1)*(nz+1) + j*(nz+1) + k
 *   DOF       = 3*n + d,  d in {x,y,z}
 */
#ifndef AM_ORACLE_H
#define AM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Element stiffness of a cube of edge h, 2x2x2 Gauss (element_kernel.cpp:155-179,
 * fem.py:43-135).  ke is 24x24 row-major. */
void orc_ke(double E, double nu, double h, double *ke);

/* 24 global DOFs of element (i,j,k) (element_kernel.cpp:186-216, fem.py:138-172). */
void orc_element_dofs(int i, int j, int k, int nx, int ny, int nz, int64_t *dofs);

/* Per-element stiffness scale.
 * variant 0 = C++ GlobalAssembler (global_assembler.cpp:132-159 +
 *             simpInterpolation global_assembler.hpp:171-173): grid -1 -> 0 (skipped),
 *             rho < rho_min -> 0 (skipped), grid 1 -> 1, else emin + rho^p (1-emin)
 *             (emin relative).
 * variant 1 = Python assemble_global_stiffness (fem.py:214-230): grid -1 -> 0,
 *             grid 1 -> 1, else (emin + rho^p (E - emin)) / E (emin absolute).
 * grid may be NULL (all design). */
void orc_scales(int variant, int64_t nel, const int8_t *grid, const double *rho,
                double p, double emin, double rho_min, double E, double *s);

/* y = K(s) u, matrix free, reference DOF order (node-centric gather, OpenMP). */
void orc_ku(int nx, int ny, int nz, const double *ke, const double *s,
            const double *u, double *y);

/* CSR of K(s) on the full 27-node block pattern (3x3 blocks).
 * orc_csr_nnz returns nnz; orc_csr_build fills rowptr[N+1], col[nnz], val[nnz]. */
int64_t orc_csr_nnz(int nx, int ny, int nz);
void orc_csr_build(int nx, int ny, int nz, const double *ke, const double *s,
                   int64_t *rowptr, int32_t *col, double *val);
void orc_csr_spmv(int64_t n, const int64_t *rowptr, const int32_t *col,
                  const double *val, const double *x, double *y);

/* Diagonal of K(s): diag = KE[0][0] * sum of the scales of the <=8 elements at the node
 * (every diagonal entry of the cube KE is equal). */
void orc_diag(int nx, int ny, int nz, const double *ke, const double *s, double *diag);

/* Jacobi-PCG on the free DOFs (Dirichlet by elimination, fem.py:274-293 semantics:
 * DOFs with |K_ii| < 1e-15 are added to the constrained set).
 * constrained[N]: 1 = fixed.  u: in = initial guess, out = solution (0 on constrained).
 * Stops when ||r||^2 < tol^2 ||b||^2 (b = F on the free DOFs) or after maxit.
 * use_csr: 1 = assemble CSR once and use SpMV (the reference's assembled-operator
 * structure), 0 = matrix-free.  Returns iterations; *relres = ||r||/||b||. */
int orc_pcg(int nx, int ny, int nz, const double *ke, const double *s,
            const uint8_t *constrained, const double *F, double *u, double tol,
            int maxit, int use_csr, double *relres);

/* ce[e] = u_e^T KE u_e for every element (topology_optimizer.cpp:147-152,
 * topopt.py:189-192, fem.py:365-370). */
void orc_element_energy(int nx, int ny, int nz, const double *ke, const double *u,
                        double *ce);

/* C++ sensitivity filter (buildFilter topology_optimizer.cpp:60-119 +
 * filterSensitivities :168-198): neighbours with |d| <= r, w = r - |d|, out of
 * the grid skipped; out = sum w rho dc / sum w rho, or dc if the denominator
 * <= 1e-15. */
void orc_filter_cpp(int nx, int ny, int nz, double r, const double *dc,
                    const double *rho, double *out);

/* Python filter (topopt.py:135-156): cone kernel k = r - |d| (|d| <= r) on a
 * (2 ceil(r)+1)^3 box, normalised by its sum, scipy.ndimage.convolve with
 * mode='reflect' (half-sample symmetric boundary). */
void orc_filter_py(int nx, int ny, int nz, double r, const double *x, double *out);

/* C++ OC update (updateDensitiesOC topology_optimizer.cpp:205-287).  rho is
 * updated in place; returns max |rho_new - rho|.  design[e] != 0 marks design
 * elements; n_design == 0 falls back to nel. *passes = bisection passes run. */
double orc_oc_cpp(int64_t nel, double *rho, const double *dc, const uint8_t *design,
                  int64_t n_design, double vf, double move, double rho_min,
                  int *passes);

/* Python OC update (_oc_update topopt.py:200-264).  Writes rho_new; returns
 * the number of bisection passes. */
int orc_oc_py(int64_t nel, const double *rho, const double *dc, const uint8_t *design,
              double vf, double move, double rho_min, double *rho_new);

/* Parameters of a SIMP run (union of SIMPConfig topology_optimizer.hpp:49-59 and
 * SIMPParams topopt.py:30-52). */
typedef struct orc_simp_params {
    double volume_fraction;
    double penalty;
    double filter_radius;
    double move_limit;
    double rho_min;
    double E_min;
    double convergence_tol;
    int max_iterations;
    double cg_tol;
    int cg_maxit;
    int bug_d1;   /* C++ variant only: assembly reads the density with the
                     assembler's z-fastest index while the optimizer stores it
                     x-fastest (global_assembler.hpp:162-164 vs
                     topology_optimizer.hpp:218-232) */
    int warm_start; /* 1: start each solve from the previous displacement */
    int use_csr;    /* 1: re-assemble a CSR K every iteration (the reference's
                       assemble-then-solve structure), 0: matrix-free */
} orc_simp_params;

/* C++ TopologyOptimizer::run (topology_optimizer.cpp:391-520) with the solve done
 * by Jacobi PCG to cg_tol.  rho0 / rho_out are C-order physical fields.
 * Histories have room for max_iterations entries.  Returns iterations run. */
int orc_simp_cpp(int nx, int ny, int nz, double h, double E, double nu,
                 const orc_simp_params *prm, const double *rho0, const double *F,
                 const int64_t *fixed, int64_t n_fixed, double *rho_out,
                 double *compliance_hist, double *volume_hist, double *change_hist,
                 int *cg_iters_hist, int *converged);

/* Python SIMPOptimizer.run (topopt.py:266-411), n_cases load cases; F is
 * n_cases x N, fixed is the concatenation of each case's constrained DOFs with
 * counts n_fixed[c]. */
int orc_simp_py(int nx, int ny, int nz, double h, double E, double nu,
                const orc_simp_params *prm, const int8_t *grid, int n_cases,
                const double *F, const int64_t *fixed, const int64_t *n_fixed,
                double *rho_out, double *compliance_hist, double *volume_hist,
                double *change_hist, int *converged);

/* Timed sample of one C++-variant SIMP iteration of the CPU restatement, for the
 * CPU baseline: CSR assembly of K (the reference re-assembles every iteration,
 * topology_optimizer.cpp:309-315), `pcg_iters` Jacobi-PCG iterations on the CSR
 * matrix, sensitivities, the C++ filter and the OC update.  times[0..5] =
 * scales+assembly, PCG set-up, mean time of one PCG iteration, sensitivities,
 * filter, OC (seconds).  Returns the OpenMP thread count used. */
int orc_baseline_sample(int nx, int ny, int nz, const orc_simp_params *prm, const double *rho,
                        const double *F, const int64_t *fixed, int64_t n_fixed, int pcg_iters,
                        double *times);

#ifdef __cplusplus
}
#endif
#endif
