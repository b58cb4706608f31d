/*
 * oracle.c -- FP64 CPU restatement of the reference SIMP inner loop.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle the tests compare against, never the
 * product): loaded by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm.
 * Every function cites the reference file:line whose behaviour it restates;
 * the declarations and the layout convention are in oracle.h.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* std::min / std::max of the C++ reference: min(a,b) = (b < a) ? b : a,
 * max(a,b) = (a < b) ? b : a (NaN handling follows those expressions). */
static inline double cmin(double a, double b) { return (b < a) ? b : a; }
static inline double cmax(double a, double b) { return (a < b) ? b : a; }
/* numpy.minimum / numpy.maximum: NaN propagates. */
static inline double npmin(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    return a < b ? a : b;
}
static inline double npmax(double a, double b) {
    if (isnan(a) || isnan(b)) return NAN;
    return a > b ? a : b;
}

/* Local node order of the hex8 element (element_kernel.cpp:41-50, fem.py:75-84,
 * fem.py:160-163): offsets (di,dj,dk) in {0,1}. */
static const int NODE_OFF[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
/* inverse map: LOCAL[di][dj][dk] -> local node */
static const int LOCAL[2][2][2] = {{{0, 4}, {3, 7}}, {{1, 5}, {2, 6}}};

/* ------------------------------------------------------------------------- */
/* A1: element stiffness by 2x2x2 Gauss quadrature of B^T C B detJ            */
/* element_kernel.cpp:71-179, fem.py:43-135                                  */
/* ------------------------------------------------------------------------- */
void orc_ke(double E, double nu, double h, double *ke) {
    double C[6][6];
    memset(C, 0, sizeof(C));
    const double f = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = f * (i == j ? 1.0 - nu : nu);
    for (int i = 3; i < 6; ++i) C[i][i] = f * (1.0 - 2.0 * nu) / 2.0;

    const double a = h / 2.0, inv_a = 1.0 / a, detJ = a * a * a;
    const double g = 1.0 / sqrt(3.0);
    memset(ke, 0, sizeof(double) * 576);
    for (int q = 0; q < 8; ++q) {
        /* Gauss points in the same corner order as the nodes */
        const double xi = (NODE_OFF[q][0] ? g : -g);
        const double eta = (NODE_OFF[q][1] ? g : -g);
        const double zeta = (NODE_OFF[q][2] ? g : -g);
        double B[6][24];
        memset(B, 0, sizeof(B));
        for (int n = 0; n < 8; ++n) {
            const double xn = NODE_OFF[n][0] ? 1.0 : -1.0;
            const double yn = NODE_OFF[n][1] ? 1.0 : -1.0;
            const double zn = NODE_OFF[n][2] ? 1.0 : -1.0;
            const double dx = inv_a * 0.125 * xn * (1.0 + yn * eta) * (1.0 + zn * zeta);
            const double dy = inv_a * 0.125 * yn * (1.0 + xn * xi) * (1.0 + zn * zeta);
            const double dz = inv_a * 0.125 * zn * (1.0 + xn * xi) * (1.0 + yn * eta);
            const int c = 3 * n;
            B[0][c] = dx;
            B[1][c + 1] = dy;
            B[2][c + 2] = dz;
            B[3][c] = dy;
            B[3][c + 1] = dx;
            B[4][c + 1] = dz;
            B[4][c + 2] = dy;
            B[5][c] = dz;
            B[5][c + 2] = dx;
        }
        double CB[6][24];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 24; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += C[i][k] * B[k][j];
                CB[i][j] = acc;
            }
        for (int i = 0; i < 24; ++i)
            for (int j = 0; j < 24; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += B[k][i] * CB[k][j];
                ke[i * 24 + j] += acc * detJ;
            }
    }
}

/* A2: element_kernel.cpp:186-216, fem.py:138-172 */
void orc_element_dofs(int i, int j, int k, int nx, int ny, int nz, int64_t *dofs) {
    (void)nx;
    const int64_t ny1 = ny + 1, nz1 = nz + 1;
    for (int n = 0; n < 8; ++n) {
        const int64_t node = (int64_t)(i + NODE_OFF[n][0]) * ny1 * nz1 +
                             (int64_t)(j + NODE_OFF[n][1]) * nz1 + (k + NODE_OFF[n][2]);
        dofs[3 * n] = 3 * node;
        dofs[3 * n + 1] = 3 * node + 1;
        dofs[3 * n + 2] = 3 * node + 2;
    }
}

/* A3 / A3py element scale rules */
void orc_scales(int variant, int64_t nel, const int8_t *grid, const double *rho,
                double p, double emin, double rho_min, double E, double *s) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int g = grid ? grid[e] : 0;
        double v;
        if (variant == 0) {
            /* global_assembler.cpp:135-159 */
            if (g == -1 || rho[e] < rho_min) v = 0.0;
            else if (g == 1) v = 1.0;
            else v = emin + pow(rho[e], p) * (1.0 - emin);
        } else {
            /* fem.py:214-230 */
            if (g == -1) v = 0.0;
            else if (g == 1) v = 1.0;
            else v = (emin + pow(rho[e], p) * (E - emin)) / E;
        }
        s[e] = v;
    }
}

/* Matrix-free y = K(s) u: each node gathers the rows of its <= 8 elements
 * (same sum as the assembled K of global_assembler.cpp:128-216 / fem.py:211-247). */
void orc_ku(int nx, int ny, int nz, const double *ke, const double *s,
            const double *u, double *y) {
    const int64_t ny1 = ny + 1, nz1 = nz + 1;
    const int64_t nn = (int64_t)(nx + 1) * ny1 * nz1;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n / (ny1 * nz1));
        const int j = (int)((n / nz1) % ny1);
        const int k = (int)(n % nz1);
        double acc[3] = {0.0, 0.0, 0.0};
        for (int ei = i - 1; ei <= i; ++ei) {
            if (ei < 0 || ei >= nx) continue;
            for (int ej = j - 1; ej <= j; ++ej) {
                if (ej < 0 || ej >= ny) continue;
                for (int ek = k - 1; ek <= k; ++ek) {
                    if (ek < 0 || ek >= nz) continue;
                    const double se = s[(int64_t)ei * ny * nz + (int64_t)ej * nz + ek];
                    if (se == 0.0) continue;
                    const int ln = LOCAL[i - ei][j - ej][k - ek];
                    int64_t dofs[24];
                    orc_element_dofs(ei, ej, ek, nx, ny, nz, dofs);
                    for (int c = 0; c < 3; ++c) {
                        const double *row = ke + (3 * ln + c) * 24;
                        double t = 0.0;
                        for (int b = 0; b < 24; ++b) t += row[b] * u[dofs[b]];
                        acc[c] += se * t;
                    }
                }
            }
        }
        y[3 * n] = acc[0];
        y[3 * n + 1] = acc[1];
        y[3 * n + 2] = acc[2];
    }
}

static inline int nb_count(int i, int n) { /* neighbours of node i within +-1 in [0,n] */
    int c = 0;
    for (int d = -1; d <= 1; ++d)
        if (i + d >= 0 && i + d <= n) ++c;
    return c;
}

int64_t orc_csr_nnz(int nx, int ny, int nz) {
    int64_t t = 0;
    for (int i = 0; i <= nx; ++i)
        for (int j = 0; j <= ny; ++j)
            for (int k = 0; k <= nz; ++k)
                t += (int64_t)nb_count(i, nx) * nb_count(j, ny) * nb_count(k, nz);
    return 9 * t;
}

/* CSR assembly of K(s) (global_assembler.cpp:61-222 builds the same matrix from
 * triplets; here the 27-node block pattern is filled row by row). */
void orc_csr_build(int nx, int ny, int nz, const double *ke, const double *s,
                   int64_t *rowptr, int32_t *col, double *val) {
    const int64_t ny1 = ny + 1, nz1 = nz + 1;
    const int64_t nn = (int64_t)(nx + 1) * ny1 * nz1;
    /* row pointers (serial prefix) */
    rowptr[0] = 0;
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n / (ny1 * nz1)), j = (int)((n / nz1) % ny1), k = (int)(n % nz1);
        const int64_t cnt = 3 * (int64_t)nb_count(i, nx) * nb_count(j, ny) * nb_count(k, nz);
        for (int c = 0; c < 3; ++c) rowptr[3 * n + c + 1] = rowptr[3 * n + c] + cnt;
    }
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n / (ny1 * nz1)), j = (int)((n / nz1) % ny1), k = (int)(n % nz1);
        for (int c = 0; c < 3; ++c) {
            int64_t pos = rowptr[3 * n + c];
            for (int mi = i - 1; mi <= i + 1; ++mi) {
                if (mi < 0 || mi > nx) continue;
                for (int mj = j - 1; mj <= j + 1; ++mj) {
                    if (mj < 0 || mj > ny) continue;
                    for (int mk = k - 1; mk <= k + 1; ++mk) {
                        if (mk < 0 || mk > nz) continue;
                        const int64_t m = (int64_t)mi * ny1 * nz1 + (int64_t)mj * nz1 + mk;
                        double blk[3] = {0.0, 0.0, 0.0};
                        /* elements containing both nodes */
                        const int ei0 = (i > mi ? i : mi) - 1, ei1 = (i < mi ? i : mi);
                        const int ej0 = (j > mj ? j : mj) - 1, ej1 = (j < mj ? j : mj);
                        const int ek0 = (k > mk ? k : mk) - 1, ek1 = (k < mk ? k : mk);
                        for (int ei = ei0; ei <= ei1; ++ei) {
                            if (ei < 0 || ei >= nx) continue;
                            for (int ej = ej0; ej <= ej1; ++ej) {
                                if (ej < 0 || ej >= ny) continue;
                                for (int ek = ek0; ek <= ek1; ++ek) {
                                    if (ek < 0 || ek >= nz) continue;
                                    const double se = s[(int64_t)ei * ny * nz + (int64_t)ej * nz + ek];
                                    const int ln = LOCAL[i - ei][j - ej][k - ek];
                                    const int lm = LOCAL[mi - ei][mj - ej][mk - ek];
                                    for (int d = 0; d < 3; ++d)
                                        blk[d] += se * ke[(3 * ln + c) * 24 + 3 * lm + d];
                                }
                            }
                        }
                        for (int d = 0; d < 3; ++d) {
                            col[pos] = (int32_t)(3 * m + d);
                            val[pos] = blk[d];
                            ++pos;
                        }
                    }
                }
            }
        }
    }
}

void orc_csr_spmv(int64_t n, const int64_t *rowptr, const int32_t *col,
                  const double *val, const double *x, double *y) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
        double acc = 0.0;
        for (int64_t p = rowptr[r]; p < rowptr[r + 1]; ++p) acc += val[p] * x[col[p]];
        y[r] = acc;
    }
}

void orc_diag(int nx, int ny, int nz, const double *ke, const double *s, double *diag) {
    const int64_t ny1 = ny + 1, nz1 = nz + 1;
    const int64_t nn = (int64_t)(nx + 1) * ny1 * nz1;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n / (ny1 * nz1)), j = (int)((n / nz1) % ny1), k = (int)(n % nz1);
        double acc[3] = {0, 0, 0};
        for (int ei = i - 1; ei <= i; ++ei) {
            if (ei < 0 || ei >= nx) continue;
            for (int ej = j - 1; ej <= j; ++ej) {
                if (ej < 0 || ej >= ny) continue;
                for (int ek = k - 1; ek <= k; ++ek) {
                    if (ek < 0 || ek >= nz) continue;
                    const double se = s[(int64_t)ei * ny * nz + (int64_t)ej * nz + ek];
                    const int ln = LOCAL[i - ei][j - ej][k - ek];
                    for (int c = 0; c < 3; ++c) acc[c] += se * ke[(3 * ln + c) * 25];
                }
            }
        }
        for (int c = 0; c < 3; ++c) diag[3 * n + c] = acc[c];
    }
}

static double dot(int64_t n, const double *a, const double *b) {
    double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (int64_t i = 0; i < n; ++i) acc += a[i] * b[i];
    return acc;
}

/* A4py + A5 (solution semantics): Jacobi PCG on K_ff.  The reference C++ solves
 * the penalty system with Eigen CG + IncompleteCholesky (linear_solver.cpp:35-183);
 * the reference Python eliminates constrained and orphan DOFs and solves
 * directly (fem.py:251-325).  Both approximate the same u; this solves K_ff u = F_f
 * to a relative residual tol (Eigen's stopping rule: |r|^2 < tol^2 |b|^2). */
int orc_pcg(int nx, int ny, int nz, const double *ke, const double *s,
            const uint8_t *constrained, const double *F, double *u, double tol,
            int maxit, int use_csr, double *relres) {
    const int64_t N = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double *dinv = malloc(sizeof(double) * N);
    double *r = malloc(sizeof(double) * N);
    double *z = malloc(sizeof(double) * N);
    double *p = malloc(sizeof(double) * N);
    double *q = malloc(sizeof(double) * N);
    double *b = malloc(sizeof(double) * N);
    uint8_t *fixed = malloc(N);
    int64_t *rowptr = NULL;
    int32_t *col = NULL;
    double *val = NULL;
    if (use_csr) {
        const int64_t nnz = orc_csr_nnz(nx, ny, nz);
        rowptr = malloc(sizeof(int64_t) * (N + 1));
        col = malloc(sizeof(int32_t) * nnz);
        val = malloc(sizeof(double) * nnz);
        orc_csr_build(nx, ny, nz, ke, s, rowptr, col, val);
    }
    orc_diag(nx, ny, nz, ke, s, dinv);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        /* orphan DOFs (fem.py:275-281) join the constrained set */
        fixed[i] = (uint8_t)((constrained && constrained[i]) || fabs(dinv[i]) < 1e-15);
        dinv[i] = fixed[i] ? 0.0 : 1.0 / dinv[i];
        b[i] = fixed[i] ? 0.0 : F[i];
        if (fixed[i]) u[i] = 0.0;
    }
#define APPLY_K(src, dst)                                                   \
    do {                                                                    \
        if (use_csr) orc_csr_spmv(N, rowptr, col, val, src, dst);           \
        else orc_ku(nx, ny, nz, ke, s, src, dst);                           \
    } while (0)

    const double bnorm2 = dot(N, b, b);
    int it = 0;
    double rr = 0.0;
    if (bnorm2 == 0.0) {
        memset(u, 0, sizeof(double) * N);
    } else {
        APPLY_K(u, q);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            r[i] = fixed[i] ? 0.0 : b[i] - q[i];
            z[i] = dinv[i] * r[i];
            p[i] = z[i];
        }
        double rz = dot(N, r, z);
        const double thr = tol * tol * bnorm2;
        rr = dot(N, r, r);
        while (it < maxit && rr >= thr) {
            APPLY_K(p, q);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i)
                if (fixed[i]) q[i] = 0.0;
            const double alpha = rz / dot(N, p, q);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i) {
                u[i] += alpha * p[i];
                r[i] -= alpha * q[i];
                z[i] = dinv[i] * r[i];
            }
            const double rz_new = dot(N, r, z);
            const double beta = rz_new / rz;
            rz = rz_new;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
            rr = dot(N, r, r);
            ++it;
        }
    }
    if (relres) *relres = bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0;
#undef APPLY_K
    free(dinv); free(r); free(z); free(p); free(q); free(b); free(fixed);
    free(rowptr); free(col); free(val);
    return it;
}

/* A6: element strain energy with the unit-stiffness KE */
void orc_element_energy(int nx, int ny, int nz, const double *ke, const double *u,
                        double *ce) {
    const int64_t nel = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        int64_t dofs[24];
        double ue[24];
        orc_element_dofs(i, j, k, nx, ny, nz, dofs);
        for (int a = 0; a < 24; ++a) ue[a] = u[dofs[a]];
        double acc = 0.0;
        for (int a = 0; a < 24; ++a) {
            double t = 0.0;
            for (int b = 0; b < 24; ++b) t += ke[a * 24 + b] * ue[b];
            acc += ue[a] * t;
        }
        ce[e] = acc;
    }
}

/* A7: C++ sensitivity filter */
void orc_filter_cpp(int nx, int ny, int nz, double r, const double *dc,
                    const double *rho, double *out) {
    const int R = (int)ceil(r);
    const int64_t nel = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double num = 0.0, den = 0.0;
        /* neighbour order of the C++ search: dz outer, dy, dx inner */
        for (int dk = -R; dk <= R; ++dk) {
            const int kk = k + dk;
            if (kk < 0 || kk >= nz) continue;
            for (int dj = -R; dj <= R; ++dj) {
                const int jj = j + dj;
                if (jj < 0 || jj >= ny) continue;
                for (int di = -R; di <= R; ++di) {
                    const int ii = i + di;
                    if (ii < 0 || ii >= nx) continue;
                    const double dist = sqrt((double)(di * di + dj * dj + dk * dk));
                    if (dist <= r) {
                        const double w = cmax(0.0, r - dist);
                        const int64_t n = (int64_t)ii * ny * nz + (int64_t)jj * nz + kk;
                        num += w * rho[n] * dc[n];
                        den += w * rho[n];
                    }
                }
            }
        }
        out[e] = (den > 1e-15) ? num / den : dc[e];
    }
}

static inline int reflect_index(int i, int n) {
    const int period = 2 * n;
    int m = i % period;
    if (m < 0) m += period;
    if (m >= n) m = period - 1 - m;
    return m;
}

/* A7py: ndimage.convolve(x, k / sum(k), mode='reflect') with the cone kernel */
void orc_filter_py(int nx, int ny, int nz, double r, const double *x, double *out) {
    const int R = (int)ceil(r);
    const int S = 2 * R + 1;
    double *w = malloc(sizeof(double) * S * S * S);
    double tot = 0.0;
    for (int a = 0; a < S; ++a)
        for (int b = 0; b < S; ++b)
            for (int c = 0; c < S; ++c) {
                const double dist = sqrt((double)((a - R) * (a - R) + (b - R) * (b - R) + (c - R) * (c - R)));
                const double v = (dist <= r) ? r - dist : 0.0;
                w[(a * S + b) * S + c] = v;
                tot += v;
            }
    for (int t = 0; t < S * S * S; ++t) w[t] /= tot;
    const int64_t nel = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double acc = 0.0;
        for (int a = 0; a < S; ++a) {
            const int ii = reflect_index(i + a - R, nx);
            for (int b = 0; b < S; ++b) {
                const int jj = reflect_index(j + b - R, ny);
                for (int c = 0; c < S; ++c) {
                    const double wt = w[(a * S + b) * S + c];
                    if (wt == 0.0) continue;
                    const int kk = reflect_index(k + c - R, nz);
                    acc += wt * x[(int64_t)ii * ny * nz + (int64_t)jj * nz + kk];
                }
            }
        }
        out[e] = acc;
    }
    free(w);
}

/* A8: C++ OC bisection */
double orc_oc_cpp(int64_t nel, double *rho, const double *dc, const uint8_t *design,
                  int64_t n_design, double vf, double move, double rho_min,
                  int *passes) {
    double l1 = 1e-20, l2 = 1e20;
    double *rho_new = malloc(sizeof(double) * nel);
    if (n_design == 0) n_design = nel;
    int it = 0;
    for (; it < 100; ++it) {
        if ((l2 - l1) / (l1 + l2) < 1e-4) break;
        const double lmid = 0.5 * (l1 + l2);
        double vol = 0.0;
#pragma omp parallel for reduction(+ : vol) schedule(static)
        for (int64_t e = 0; e < nel; ++e) {
            const double r0 = rho[e];
            if (!design[e]) {
                rho_new[e] = r0;
                continue;
            }
            const double Be = sqrt(-dc[e] / (lmid * 1.0 + 1e-20));
            double cand = r0 * Be;
            cand = cmax(rho_min, cmax(r0 - move, cmin(1.0, cmin(r0 + move, cand))));
            rho_new[e] = cand;
            vol += cand;
        }
        if (vol / (double)n_design > vf) l1 = lmid;
        else l2 = lmid;
    }
    double mc = 0.0;
    for (int64_t e = 0; e < nel; ++e) {
        const double c = fabs(rho_new[e] - rho[e]);
        if (c > mc) mc = c;
    }
    memcpy(rho, rho_new, sizeof(double) * nel);
    free(rho_new);
    if (passes) *passes = it;
    return mc;
}

/* A8py: Python OC bisection */
int orc_oc_py(int64_t nel, const double *rho, const double *dc, const uint8_t *design,
              double vf, double move, double rho_min, double *rho_new) {
    double l1 = 1e-9, l2 = 1e9;
    int64_t n_design = 0;
    for (int64_t e = 0; e < nel; ++e) n_design += design[e] ? 1 : 0;
    int it = 0;
    for (; it < 100; ++it) {
        if (l1 + l2 < 1e-12) break;
        const double den = (l1 + l2) > 1e-10 ? (l1 + l2) : 1e-10;
        if ((l2 - l1) / den <= 1e-3) break;
        const double lmid = 0.5 * (l1 + l2);
        double vol = 0.0;
#pragma omp parallel for reduction(+ : vol) schedule(static)
        for (int64_t e = 0; e < nel; ++e) {
            const double r0 = rho[e];
            if (!design[e]) {
                rho_new[e] = r0;
                continue;
            }
            const double Be = sqrt(-dc[e] / (1.0 * lmid + 1e-10));
            const double v = npmax(rho_min, npmax(r0 - move, npmin(1.0, npmin(r0 + move, r0 * Be))));
            rho_new[e] = v;
            vol += v;
        }
        if (vol / (double)n_design > vf) l1 = lmid;
        else l2 = lmid;
    }
    return it;
}

/* fixed-DOF list -> per-DOF flag */
static void mark_fixed(int64_t N, const int64_t *fixed, int64_t n_fixed, uint8_t *flag) {
    memset(flag, 0, N);
    for (int64_t t = 0; t < n_fixed; ++t)
        if (fixed[t] >= 0 && fixed[t] < N) flag[fixed[t]] = 1;
}

/* A9: C++ TopologyOptimizer::run / runIteration (topology_optimizer.cpp:294-520) */
int orc_simp_cpp(int nx, int ny, int nz, double h, double E, double nu,
                 const orc_simp_params *prm, const double *rho0, const double *F,
                 const int64_t *fixed, int64_t n_fixed, double *rho_out,
                 double *compliance_hist, double *volume_hist, double *change_hist,
                 int *cg_iters_hist, int *converged) {
    const int64_t nel = (int64_t)nx * ny * nz;
    const int64_t N = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double ke[576];
    orc_ke(E, nu, h, ke);
    double *rho = malloc(sizeof(double) * nel);
    double *arho = malloc(sizeof(double) * nel);
    double *s = malloc(sizeof(double) * nel);
    double *ce = malloc(sizeof(double) * nel);
    double *dc = malloc(sizeof(double) * nel);
    double *dcf = malloc(sizeof(double) * nel);
    double *u = calloc(N, sizeof(double));
    uint8_t *design = malloc(nel);
    uint8_t *cons = malloc(N);
    int64_t *perm = NULL;
    memcpy(rho, rho0, sizeof(double) * nel);
    mark_fixed(N, fixed, n_fixed, cons);
    if (prm->bug_d1) {
        /* assembly position (i,j,k) reads flat index q = i*ny*nz + j*nz + k of the
         * optimizer's x-fastest vector, i.e. the physical element
         * (q % nx, (q / nx) % ny, q / (nx*ny)). */
        perm = malloc(sizeof(int64_t) * nel);
        for (int64_t q = 0; q < nel; ++q) {
            const int64_t pi = q % nx, pj = (q / nx) % ny, pk = q / ((int64_t)nx * ny);
            perm[q] = pi * ny * nz + pj * nz + pk;
        }
    }
    /* design mask from the initial density (topology_optimizer.cpp:419-428) */
    int64_t n_design = 0;
    for (int64_t e = 0; e < nel; ++e) {
        design[e] = (uint8_t)(rho[e] > prm->rho_min + 1e-6 && rho[e] < 0.99);
        n_design += design[e];
    }
    const double p = prm->penalty;
    int it = 0;
    *converged = 0;
    for (; it < prm->max_iterations; ++it) {
        for (int64_t e = 0; e < nel; ++e) arho[e] = perm ? rho[perm[e]] : rho[e];
        /* optimizer assembles without a domain mask (topology_optimizer.cpp:309-315) */
        orc_scales(0, nel, NULL, arho, p, prm->E_min, prm->rho_min, 1.0, s);
        if (!prm->warm_start) memset(u, 0, sizeof(double) * N);
        double relres = 0.0;
        const int cgit = orc_pcg(nx, ny, nz, ke, s, cons, F, u, prm->cg_tol, prm->cg_maxit,
                                 prm->use_csr, &relres);
        const double comp = dot(N, u, F); /* computeCompliance: u . F */
        orc_element_energy(nx, ny, nz, ke, u, ce);
        for (int64_t e = 0; e < nel; ++e) dc[e] = -p * pow(rho[e], p - 1.0) * ce[e];
        orc_filter_cpp(nx, ny, nz, prm->filter_radius, dc, rho, dcf);
        const double change = orc_oc_cpp(nel, rho, dcf, design, n_design, prm->volume_fraction,
                                         prm->move_limit, prm->rho_min, NULL);
        double vs = 0.0;
        int64_t dcnt = 0;
        for (int64_t e = 0; e < nel; ++e)
            if (design[e]) {
                vs += rho[e];
                ++dcnt;
            }
        compliance_hist[it] = comp;
        volume_hist[it] = dcnt > 0 ? vs / dcnt : vs / nel;
        if (change_hist) change_hist[it] = change;
        if (cg_iters_hist) cg_iters_hist[it] = cgit;
        if (change < prm->convergence_tol) {
            *converged = 1;
            ++it;
            break;
        }
    }
    memcpy(rho_out, rho, sizeof(double) * nel);
    free(rho); free(arho); free(s); free(ce); free(dc); free(dcf); free(u);
    free(design); free(cons); free(perm);
    return it;
}

/* A9py: Python SIMPOptimizer.run (topopt.py:266-411) */
int orc_simp_py(int nx, int ny, int nz, double h, double E, double nu,
                const orc_simp_params *prm, const int8_t *grid, int n_cases,
                const double *F, const int64_t *fixed, const int64_t *n_fixed,
                double *rho_out, double *compliance_hist, double *volume_hist,
                double *change_hist, int *converged) {
    const int64_t nel = (int64_t)nx * ny * nz;
    const int64_t N = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    const double p = prm->penalty;
    double ke[576];
    orc_ke(E, nu, h, ke);
    double *rho = malloc(sizeof(double) * nel);
    double *old = malloc(sizeof(double) * nel);
    double *rf = malloc(sizeof(double) * nel);
    double *s = malloc(sizeof(double) * nel);
    double *ce = malloc(sizeof(double) * nel);
    double *dct = malloc(sizeof(double) * nel);
    double *tmp = malloc(sizeof(double) * nel);
    double *dcf = malloc(sizeof(double) * nel);
    double *u = calloc((size_t)N * (n_cases > 0 ? n_cases : 1), sizeof(double));
    uint8_t *design = malloc(nel);
    uint8_t *cons = malloc(N);
    for (int64_t e = 0; e < nel; ++e) {
        rho[e] = prm->volume_fraction;
        design[e] = (uint8_t)(grid[e] == 0);
    }
    int it = 0;
    *converged = 0;
    for (; it < prm->max_iterations; ++it) {
        orc_filter_py(nx, ny, nz, prm->filter_radius, rho, rf);
        for (int64_t e = 0; e < nel; ++e) rf[e] = npmin(npmax(rf[e], prm->rho_min), 1.0);
        double total_c = 0.0;
        memset(dct, 0, sizeof(double) * nel);
        orc_scales(1, nel, grid, rf, p, prm->E_min, prm->rho_min, E, s);
        int64_t off = 0;
        for (int lc = 0; lc < n_cases; ++lc) {
            double *ul = u + (size_t)lc * N;
            mark_fixed(N, fixed + off, n_fixed[lc], cons);
            off += n_fixed[lc];
            if (!prm->warm_start) memset(ul, 0, sizeof(double) * N);
            double relres;
            orc_pcg(nx, ny, nz, ke, s, cons, F + (size_t)lc * N, ul, prm->cg_tol, prm->cg_maxit,
                    prm->use_csr, &relres);
            orc_element_energy(nx, ny, nz, ke, ul, ce);
            double c = 0.0;
            for (int64_t e = 0; e < nel; ++e) {
                if (grid[e] == -1) continue;
                double er;
                if (grid[e] == 0)
                    er = prm->E_min / E + pow(rf[e], p) * (1.0 - prm->E_min / E);
                else
                    er = 1.0;
                c += er * ce[e];
            }
            total_c += c;
            for (int64_t e = 0; e < nel; ++e) {
                double d = design[e] ? -p * pow(rf[e], p - 1.0) * ce[e] : 0.0;
                if (isnan(d)) d = 0.0;
                dct[e] += d;
            }
        }
        for (int64_t e = 0; e < nel; ++e) tmp[e] = dct[e] * rho[e];
        orc_filter_py(nx, ny, nz, prm->filter_radius, tmp, dcf);
        for (int64_t e = 0; e < nel; ++e) dcf[e] = dcf[e] / npmax(rho[e], 1e-3);
        memcpy(old, rho, sizeof(double) * nel);
        orc_oc_py(nel, old, dcf, design, prm->volume_fraction, prm->move_limit, prm->rho_min, rho);
        double vs = 0.0;
        int64_t nd = 0;
        double change = 0.0;
        for (int64_t e = 0; e < nel; ++e) {
            if (design[e]) {
                vs += rho[e];
                ++nd;
            }
            const double c = fabs(rho[e] - old[e]);
            if (c > change) change = c;
        }
        compliance_hist[it] = total_c;
        volume_hist[it] = vs / (double)nd;
        if (change_hist) change_hist[it] = change;
        if (change < prm->convergence_tol) {
            *converged = 1;
            ++it;
            break;
        }
    }
    memcpy(rho_out, rho, sizeof(double) * nel);
    free(rho); free(old); free(rf); free(s); free(ce); free(dct); free(tmp); free(dcf);
    free(u); free(design); free(cons);
    return it;
}

static double wtime(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

int orc_baseline_sample(int nx, int ny, int nz, const orc_simp_params *prm, const double *rho,
                        const double *F, const int64_t *fixed, int64_t n_fixed, int pcg_iters,
                        double *times) {
    const int64_t nel = (int64_t)nx * ny * nz;
    const int64_t N = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    double ke[576];
    orc_ke(1.0, 0.3, 1.0, ke);
    double *s = malloc(sizeof(double) * nel);
    double *u = calloc(N, sizeof(double));
    double *ce = malloc(sizeof(double) * nel);
    double *dc = malloc(sizeof(double) * nel);
    double *dcf = malloc(sizeof(double) * nel);
    double *r2 = malloc(sizeof(double) * nel);
    uint8_t *design = malloc(nel);
    uint8_t *cons = malloc(N);
    mark_fixed(N, fixed, n_fixed, cons);
    int64_t nd = 0;
    for (int64_t e = 0; e < nel; ++e) {
        design[e] = (uint8_t)(rho[e] > prm->rho_min + 1e-6 && rho[e] < 0.99);
        nd += design[e];
    }
    /* assembly */
    double t0 = wtime();
    orc_scales(0, nel, NULL, rho, prm->penalty, prm->E_min, prm->rho_min, 1.0, s);
    const int64_t nnz = orc_csr_nnz(nx, ny, nz);
    int64_t *rowptr = malloc(sizeof(int64_t) * (N + 1));
    int32_t *col = malloc(sizeof(int32_t) * nnz);
    double *val = malloc(sizeof(double) * nnz);
    orc_csr_build(nx, ny, nz, ke, s, rowptr, col, val);
    double t1 = wtime();
    /* PCG: set-up (diagonal, initial residual) and `pcg_iters` iterations */
    double *dinv = malloc(sizeof(double) * N), *r = malloc(sizeof(double) * N);
    double *z = malloc(sizeof(double) * N), *p = malloc(sizeof(double) * N), *q = malloc(sizeof(double) * N);
    orc_diag(nx, ny, nz, ke, s, dinv);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        const int fx = cons[i] || fabs(dinv[i]) < 1e-15;
        dinv[i] = fx ? 0.0 : 1.0 / dinv[i];
        r[i] = fx ? 0.0 : F[i];
        z[i] = dinv[i] * r[i];
        p[i] = z[i];
    }
    double rz = dot(N, r, z);
    double t2 = wtime();
    for (int it = 0; it < pcg_iters; ++it) {
        orc_csr_spmv(N, rowptr, col, val, p, q);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i)
            if (cons[i]) q[i] = 0.0;
        const double alpha = rz / dot(N, p, q);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            u[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
        }
        const double rzn = dot(N, r, z);
        const double beta = rzn / rz;
        rz = rzn;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
        (void)dot(N, r, r);
    }
    double t3 = wtime();
    orc_element_energy(nx, ny, nz, ke, u, ce);
    for (int64_t e = 0; e < nel; ++e) dc[e] = -prm->penalty * pow(rho[e], prm->penalty - 1.0) * ce[e];
    double t4 = wtime();
    orc_filter_cpp(nx, ny, nz, prm->filter_radius, dc, rho, dcf);
    double t5 = wtime();
    memcpy(r2, rho, sizeof(double) * nel);
    (void)orc_oc_cpp(nel, r2, dcf, design, nd, prm->volume_fraction, prm->move_limit, prm->rho_min, NULL);
    double t6 = wtime();
    times[0] = t1 - t0;
    times[1] = t2 - t1;
    times[2] = pcg_iters > 0 ? (t3 - t2) / pcg_iters : 0.0;
    times[3] = t4 - t3;
    times[4] = t5 - t4;
    times[5] = t6 - t5;
    free(s); free(u); free(ce); free(dc); free(dcf); free(r2); free(design); free(cons);
    free(rowptr); free(col); free(val); free(dinv); free(r); free(z); free(p); free(q);
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
