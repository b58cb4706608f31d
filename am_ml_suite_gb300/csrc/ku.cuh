// ku.cuh -- matrix-free hex8 K*u for sm_103a.
//
// Replaces global K assembly + SpMV (global_assembler.cpp:61-222,
// linear_solver.cpp:136-155; fem.py:175-248).  y = sum_e s_e KE u_e with the
// 24x24 unit-stiffness KE of a cube (element_kernel.cpp:155-179) never formed:
// the element product is evaluated in the Walsh basis of trilinear monomials
// {1, xi, eta, zeta, xi eta, eta zeta, xi zeta, xi eta zeta}, where KE is
// block-sparse.  Per element: an 8-point butterfly per component (forward), the
// stress of 7 strain slices (constant, three linear, three bilinear modes), the
// transposed butterfly.  ~230 flops instead of the 1152 of the dense product,
// exact for the 2x2x2-Gauss KE (the quadrature integrates these products exactly).
//
// Tiling: a CTA owns TX x TY node columns and a chunk of tz node planes, and
// marches up z one element layer at a time.  Each layer stages the next node
// plane (with a one-node halo) in shared memory, computes the (TX+1)(TY+1)
// elements that touch its nodes, writes their 8 corner contributions to shared
// memory, and every owned node then gathers its 4 elements of the layer in a
// fixed order (no atomics, bitwise reproducible).  The top-face contributions are
// carried in registers to the next plane.
#pragma once
#include "am_common.cuh"

namespace amk {

// PLAIN: y = K u.  PCG: p = dinv r + beta p_prev, q = mask(K p), p.q.  RESID:
// r = mask(f - K u) in FP64.  DOT: q = mask(K u) and u.q (the FP64 matvec of the
// outer flexible CG).
enum { KU_PLAIN = 0, KU_PCG = 1, KU_RESID = 2, KU_DOT = 3 };

template <typename T>
struct KuArgs {
    Layout L;
    const T *s;            // element scales
    const T *u;            // PLAIN / RESID: the vector multiplied; PCG: previous p
    const T *r;            // PCG: residual
    const T *dinv;         // PCG / RESID: per-node inverse diagonal
    const double *f;       // RESID: right-hand side (FP64)
    T *y;                  // PLAIN: K u ; PCG: q = K p ; RESID: r = f - K u
    T *p_out;              // PCG: p = dinv r + beta p_prev
    T *pa, *pb;            // PCG ping-pong pair: iteration it reads p[it & 1], writes the other
                           // (it = S->it, so a solve can stop and resume at any parity)
    const uint8_t *mask;   // per-node constrained bits (bit c = DOF component c)
    double *partial;       // per-tile partial sums (2 per tile)
    double *ce;            // RESID with energy: u_e^T KE u_e per owned element
    Scalars *S;
    Modal<T> M;
    int tiles_x, tiles_y, tiles_z, tz;
    int energy;
};

// The element operator.  u[c][a]: component c of local node a (reference node
// order (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1),
// element_kernel.cpp:41-50).  y[c][a] = scale * (KE u)[3a+c].  If en != nullptr,
// *en = u^T KE u (unscaled).
template <typename T>
__host__ __device__ __forceinline__ void hex8_apply(const T (&u)[3][8], T (&y)[3][8], const Modal<T> &M,
                                           T scale, T *en) {
    T A[8][3];  // A[m][c]: unnormalised Walsh coefficient of mode m, component c
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T s00 = u[c][1] + u[c][0], d00 = u[c][1] - u[c][0];
        const T s10 = u[c][2] + u[c][3], d10 = u[c][2] - u[c][3];
        const T s01 = u[c][5] + u[c][4], d01 = u[c][5] - u[c][4];
        const T s11 = u[c][6] + u[c][7], d11 = u[c][6] - u[c][7];
        const T ss0 = s10 + s00, sd0 = s10 - s00, ss1 = s11 + s01, sd1 = s11 - s01;
        const T ds0 = d10 + d00, dd0 = d10 - d00, ds1 = d11 + d01, dd1 = d11 - d01;
        A[0][c] = ss1 + ss0;
        A[3][c] = ss1 - ss0;
        A[2][c] = sd1 + sd0;
        A[5][c] = sd1 - sd0;
        A[1][c] = ds1 + ds0;
        A[6][c] = ds1 - ds0;
        A[4][c] = dd1 + dd0;
        A[7][c] = dd1 - dd0;
    }
    const T lam = M.lam, mu = M.mu, twomu = mu + mu;
    T Y[8][3];
    // constant-strain mode: rows xi, eta, zeta = A1, A2, A3
    {
        const T tr = A[1][0] + A[2][1] + A[3][2];
        const T s00 = lam * tr + twomu * A[1][0];
        const T s11 = lam * tr + twomu * A[2][1];
        const T s22 = lam * tr + twomu * A[3][2];
        const T s01 = mu * (A[1][1] + A[2][0]);
        const T s02 = mu * (A[1][2] + A[3][0]);
        const T s12 = mu * (A[2][2] + A[3][1]);
        Y[1][0] = M.c1 * s00; Y[1][1] = M.c1 * s01; Y[1][2] = M.c1 * s02;
        Y[2][0] = M.c1 * s01; Y[2][1] = M.c1 * s11; Y[2][2] = M.c1 * s12;
        Y[3][0] = M.c1 * s02; Y[3][1] = M.c1 * s12; Y[3][2] = M.c1 * s22;
    }
    // linear modes: monomial xi (rows eta = A4, zeta = A6), eta (xi = A4, zeta = A5),
    // zeta (xi = A6, eta = A5)
    {
        const T trx = A[4][1] + A[6][2];
        const T sh_x = mu * (A[4][2] + A[6][1]);
        const T tre = A[4][0] + A[5][2];
        const T sh_e = mu * (A[4][2] + A[5][0]);
        const T trz = A[6][0] + A[5][1];
        const T sh_z = mu * (A[6][1] + A[5][0]);
        Y[4][0] = M.c2 * (mu * A[4][0] + lam * tre + twomu * A[4][0]);
        Y[4][1] = M.c2 * (lam * trx + twomu * A[4][1] + mu * A[4][1]);
        Y[4][2] = M.c2 * (sh_x + sh_e);
        Y[6][0] = M.c2 * (mu * A[6][0] + lam * trz + twomu * A[6][0]);
        Y[6][1] = M.c2 * (sh_x + sh_z);
        Y[6][2] = M.c2 * (lam * trx + twomu * A[6][2] + mu * A[6][2]);
        Y[5][0] = M.c2 * (sh_e + sh_z);
        Y[5][1] = M.c2 * (mu * A[5][1] + lam * trz + twomu * A[5][1]);
        Y[5][2] = M.c2 * (lam * tre + twomu * A[5][2] + mu * A[5][2]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) Y[7][c] = M.c7 * A[7][c];
    if (en) {
        T e = 0;
#pragma unroll
        for (int m = 1; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) e += A[m][c] * Y[m][c];
        *en = e;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T y1 = scale * Y[1][c], y2 = scale * Y[2][c], y3 = scale * Y[3][c];
        const T y4 = scale * Y[4][c], y5 = scale * Y[5][c], y6 = scale * Y[6][c];
        const T y7 = scale * Y[7][c];
        const T ss1 = y3, ss0 = -y3;  // mode 0 (rigid translation) has no stiffness
        const T sd1 = y2 + y5, sd0 = y2 - y5;
        const T ds1 = y1 + y6, ds0 = y1 - y6;
        const T dd1 = y4 + y7, dd0 = y4 - y7;
        const T s10 = ss0 + sd0, s00 = ss0 - sd0, s11 = ss1 + sd1, s01 = ss1 - sd1;
        const T d10 = ds0 + dd0, d00 = ds0 - dd0, d11 = ds1 + dd1, d01 = ds1 - dd1;
        y[c][1] = s00 + d00;
        y[c][0] = s00 - d00;
        y[c][2] = s10 + d10;
        y[c][3] = s10 - d10;
        y[c][5] = s01 + d01;
        y[c][4] = s01 - d01;
        y[c][6] = s11 + d11;
        y[c][7] = s11 - d11;
    }
}

template <int TX, int TY>
struct KuShape {
    static constexpr int EX = TX + 1, EY = TY + 1, NE = EX * EY;  // elements per layer
    static constexpr int SX = TX + 2, SY = TY + 2, NS = SX * SY;  // staged nodes per plane
    static constexpr int NT = (NE + 31) / 32 * 32;                // threads
    template <typename T>
    static constexpr size_t smem_bytes() {
        return sizeof(T) * (size_t)(2 * 3 * NS + 8 * 3 * NE);
    }
};

// One tile (block B.b of B.n) of the tiled K*u; the kernel below runs one tile
// per CTA, the batched persistent kernel one tile per work item.
template <typename T, int TX, int TY, int MODE>
__device__ __forceinline__ void ku_tile_body(KuArgs<T> A, const Blk B) {
    using Sh = KuShape<TX, TY>;
    constexpr int EX = Sh::EX, NE = Sh::NE, SX = Sh::SX, NS = Sh::NS, NT = Sh::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *us = reinterpret_cast<T *>(smem_raw);  // [2 slots][3][NS]
    T *yb = us + 2 * 3 * NS;                  // [8 corners][3][NE]
    __shared__ double red[2 * (NT / 32)];
    __shared__ int last_flag;

    if (MODE == KU_PCG && A.S->done) return;
    const Layout L = A.L;
    const int tid = threadIdx.x;
    int b = B.b;
    const int tx_ = b % A.tiles_x;
    b /= A.tiles_x;
    const int ty_ = b % A.tiles_y;
    const int tz_ = b / A.tiles_y;
    const int x0 = tx_ * TX, y0 = ty_ * TY, z0 = tz_ * A.tz;
    const int z1 = min(z0 + A.tz, L.nz + 1);
    const long long cs = L.cs;
    T beta = T(0);
    if (MODE == KU_PCG) {
        beta = (T)A.S->beta;
        if (A.pa) {
            const bool odd = (A.S->it & 1) != 0;
            A.u = odd ? A.pb : A.pa;
            A.p_out = odd ? A.pa : A.pb;
        }
    }

    auto stage = [&](int iz, int slot) {
        T *dst = us + slot * 3 * NS;
        for (int t = tid; t < NS; t += NT) {
            const int lx = t % SX, ly = t / SX;
            const int ix = x0 - 1 + lx, iy = y0 - 1 + ly;
            T v0 = T(0), v1 = T(0), v2 = T(0);
            if (ix >= 0 && ix <= L.nx && iy >= 0 && iy <= L.ny && iz >= 0 && iz <= L.nz) {
                const long long n = node_index(L, ix, iy, iz);
                if (MODE == KU_PCG) {
                    const T d = A.dinv[n];
                    v0 = d * A.r[n];
                    v1 = d * A.r[n + cs];
                    v2 = d * A.r[n + 2 * cs];
                    if (beta != T(0)) {
                        v0 += beta * A.u[n];
                        v1 += beta * A.u[n + cs];
                        v2 += beta * A.u[n + 2 * cs];
                    }
                    if (lx >= 1 && lx <= TX && ly >= 1 && ly <= TY && iz >= z0 && iz < z1) {
                        A.p_out[n] = v0;
                        A.p_out[n + cs] = v1;
                        A.p_out[n + 2 * cs] = v2;
                    }
                } else {
                    v0 = A.u[n];
                    v1 = A.u[n + cs];
                    v2 = A.u[n + 2 * cs];
                }
            }
            dst[t] = v0;
            dst[NS + t] = v1;
            dst[2 * NS + t] = v2;
        }
    };

    T acc[3] = {T(0), T(0), T(0)};
    // PCG: p of the owned node on the plane completed by the current layer.  It
    // is read from shared memory one layer ahead (slot of plane ez+1, which is
    // not restaged before layer ez+2) because the slot of plane ez is restaged
    // by faster threads while the owner phase of layer ez is still running.
    T pcur[3] = {T(0), T(0), T(0)};
    Acc<T> d0, d1;  // partial sums: PCG (p.q); RESID (r.r, r.dinv.r)
    stage(z0 - 1, (z0 - 1) & 1);
    for (int ez = z0 - 1; ez < z1; ++ez) {
        stage(ez + 1, (ez + 1) & 1);
        __syncthreads();
        if (tid < NE) {
            const int exl = tid % EX, eyl = tid / EX;
            const int ex = x0 - 1 + exl, ey = y0 - 1 + eyl;
            T se = T(0);
            long long e = -1;
            if (ex >= 0 && ex < L.nx && ey >= 0 && ey < L.ny && ez >= 0 && ez < L.nz) {
                e = elem_index(L, ex, ey, ez);
                se = A.s[e];
            }
            T yo[3][8];
            const bool want_en = MODE == KU_RESID && A.energy && e >= 0 && exl >= 1 && eyl >= 1 &&
                                 ez >= z0;
            if (se != T(0) || want_en) {
                const T *ub = us + (ez & 1) * 3 * NS;
                const T *ut = us + ((ez + 1) & 1) * 3 * NS;
                const int i00 = eyl * SX + exl;
                T uu[3][8];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    uu[c][0] = ub[c * NS + i00];
                    uu[c][1] = ub[c * NS + i00 + 1];
                    uu[c][2] = ub[c * NS + i00 + SX + 1];
                    uu[c][3] = ub[c * NS + i00 + SX];
                    uu[c][4] = ut[c * NS + i00];
                    uu[c][5] = ut[c * NS + i00 + 1];
                    uu[c][6] = ut[c * NS + i00 + SX + 1];
                    uu[c][7] = ut[c * NS + i00 + SX];
                }
                T en = T(0);
                hex8_apply<T>(uu, yo, A.M, se, want_en ? &en : nullptr);
                if (want_en) A.ce[e] = (double)en;
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int k = 0; k < 8; ++k) yo[c][k] = T(0);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
#pragma unroll
                for (int c = 0; c < 3; ++c) yb[(k * 3 + c) * NE + tid] = yo[c][k];
        }
        __syncthreads();
        if (tid < TX * TY) {
            const int lx = tid % TX, ly = tid / TX;
            const int e00 = ly * EX + lx;  // element (ix-1, iy-1): node is its corner 2 / 6
            const int e10 = e00 + 1;       // element (ix,   iy-1): corner 3 / 7
            const int e01 = e00 + EX;      // element (ix-1, iy  ): corner 1 / 5
            const int e11 = e00 + EX + 1;  // element (ix,   iy  ): corner 0 / 4
            T val[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T bot = yb[(2 * 3 + c) * NE + e00] + yb[(3 * 3 + c) * NE + e10] +
                              yb[(1 * 3 + c) * NE + e01] + yb[(0 * 3 + c) * NE + e11];
                const T top = yb[(6 * 3 + c) * NE + e00] + yb[(7 * 3 + c) * NE + e10] +
                              yb[(5 * 3 + c) * NE + e01] + yb[(4 * 3 + c) * NE + e11];
                val[c] = acc[c] + bot;
                acc[c] = top;
            }
            const int ix = x0 + lx, iy = y0 + ly;
            if (ez >= z0 && ix <= L.nx && iy <= L.ny) {
                const long long n = node_index(L, ix, iy, ez);
                if (MODE == KU_PLAIN) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) A.y[n + c * cs] = val[c];
                } else {
                    const unsigned m = A.mask[n];
                    if (MODE == KU_PCG || MODE == KU_DOT) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const T q = ((m >> c) & 1u) ? T(0) : val[c];
                            A.y[n + c * cs] = q;
                            d0.add_prod(pcur[c], q);
                        }
                    } else {  // RESID (dinv nullable: r.(D^-1 r) is then 0)
                        const T dv = A.dinv ? A.dinv[n] : T(0);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const T rr = ((m >> c) & 1u) ? T(0) : (T)(A.f[n + c * cs] - (double)val[c]);
                            A.y[n + c * cs] = rr;
                            d0.add_prod(rr, rr);
                            d1.add_prod(rr, dv * rr);
                        }
                    }
                }
            }
            if (MODE == KU_PCG || MODE == KU_DOT) {
                const T *pn = us + ((ez + 1) & 1) * 3 * NS + (ly + 1) * SX + (lx + 1);
#pragma unroll
                for (int c = 0; c < 3; ++c) pcur[c] = pn[c * NS];
            }
        }
    }
    if (MODE == KU_PLAIN) return;

    // per-tile partials, then the last tile reduces them (fixed order)
    double v[2] = {d0.value(), d1.value()};
    block_sum<2>(v, red);
    if (tid == 0) {
        A.partial[2 * B.b] = v[0];
        A.partial[2 * B.b + 1] = v[1];
    }
    if (!arrive_last_n(&A.S->cnt_ku, &last_flag, B.n)) return;
    double tot[2];
    reduce_partials<2>(A.partial, B.n, 2, tot, red);
    if (tid == 0) {
        Scalars *S = A.S;
        if (MODE == KU_PCG) {
            const double pq = tot[0];
            S->pq = pq;
            if (!(pq > 0.0) || !isfinite(pq)) {
                S->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
                S->done = 1;
                S->alpha = 0.0;
            } else {
                S->alpha = S->rz / pq;
            }
        } else if (MODE == KU_DOT) {
            const double pq = tot[0];
            S->o_pq = pq;
            if (!(pq > 0.0) || !isfinite(pq)) {
                S->o_status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
                S->o_alpha = 0.0;
            } else {
                S->o_alpha = S->o_zr / pq;
            }
        } else {
            S->res_rr = tot[0];
            S->res_rz = tot[1];
        }
        S->cnt_ku = 0;
    }
}

template <typename T, int TX, int TY, int MODE>
__global__ void __launch_bounds__(KuShape<TX, TY>::NT) ku_tile_kernel(KuArgs<T> A) {
    ku_tile_body<T, TX, TY, MODE>(A, grid_blk());
}

}  // namespace amk
