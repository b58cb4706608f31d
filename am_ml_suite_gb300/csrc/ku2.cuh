// ku2.cuh -- FP32 matrix-free hex8 K*u, warp-row form with packed FP32x2 math.
//
// Same operator as ku.cuh (y = sum_e s_e KE u_e in the Walsh basis of trilinear
// monomials), organised for instruction economy on sm_103a:
//   * a warp owns two element rows (ey, ey+1) of a tile and marches up z; its
//     lanes are element columns; the two elements of a lane run in the two halves
//     of packed FP32x2 instructions (__fadd2_rn / __ffma2_rn / __fmul2_rn);
//   * the x-stage and y-stage of the element transform of a node plane
//     ("face modes") are computed once per plane and carried to the next layer,
//     and the transposed transform of a plane is done once on the sum of the two
//     layers that share it (sum factorisation in z);
//   * x neighbours come from warp shuffles, the one shared node row between
//     warps goes through shared memory: one barrier per layer;
//   * the element scale multiplies three modal constants, not 24 outputs.
// Tile: 30 owned node columns (lane 0 and lane 31 are halo), 2W-1 owned node
// rows, a chunk of tz node planes.  Nodes are gathered in a fixed order, so the
// result is bitwise reproducible.
#pragma once
#include "am_common.cuh"

namespace amk {

template <int W>
struct Ku2Shape {
    static constexpr int NT = 32 * W;
    static constexpr int TX = 30;         // owned node columns per tile
    static constexpr int TY = 2 * W - 1;  // owned node rows per tile
};

struct Ku2Args {
    Layout L;
    const float *s;        // element scales
    const float *u;        // PLAIN: the vector multiplied
    float *pa, *pb;        // PCG: ping-pong pair, iteration it reads p[it & 1], writes the other
    const float *r;        // PCG: residual
    const float *dinv;     // PCG: per-node inverse diagonal
    const uint8_t *mask;   // PCG: per-node constrained bits
    float *y;              // PLAIN: K u ; PCG: q = mask(K p)
    double *partial;       // PCG: per-tile p.q
    Scalars *S;
    Modal<float> M;
    int tiles_x, tiles_y, tiles_z, tz;
};

namespace k2 {
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 splat(float a) { return make_float2(a, a); }

// face modes of one node plane for the lane's two elements: rows (0,1) for the
// first element, (1,2) for the second; v = own column, vn = column + 1.
struct Face {
    float2 ss, sd, ds, dd;
};
__device__ __forceinline__ Face face_modes(float v0, float v1, float v2, float n0, float n1, float n2) {
    const float2 vlo = make_float2(v0, v1), vhi = make_float2(v1, v2);
    const float2 nlo = make_float2(n0, n1), nhi = make_float2(n1, n2);
    const float2 slo = add(nlo, vlo), dlo = sub(nlo, vlo);
    const float2 shi = add(nhi, vhi), dhi = sub(nhi, vhi);
    Face f;
    f.ss = add(shi, slo);
    f.sd = sub(shi, slo);
    f.ds = add(dhi, dlo);
    f.dd = sub(dhi, dlo);
    return f;
}
// The element transform of one layer for the lane's two elements: face modes of
// the bottom (FB) and top (FT) node planes -> Walsh coefficients -> scaled modal
// stiffness -> transposed transform.  The bottom half of the result joins the
// carry CT of the plane below and gives V: rows 0..2 of the bottom plane at this
// lane's column, with the left neighbour lane's elements added (row 0 still lacks
// the warp below's elements, row 2 is passed to the warp above).  The top half
// becomes the new carry.
__device__ __forceinline__ void layer_math(const Face (&FB)[3], const Face (&FT)[3], Face (&CT)[3], const float2 sc,
                                           const Modal<float> &M, const float2 lam, const float2 mu,
                                           const float2 twomu, const float2 thrmu, float (&V)[3][3]) {
    const float2 c1 = mul(sc, splat(M.c1)), c2 = mul(sc, splat(M.c2)), c7 = mul(sc, splat(M.c7));
    // ---- z stage: Walsh coefficients A[m][c] of both elements --------------
    float2 A1[3], A2[3], A3[3], A4[3], A5[3], A6[3], A7[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        A1[c] = add(FT[c].ds, FB[c].ds);
        A6[c] = sub(FT[c].ds, FB[c].ds);
        A2[c] = add(FT[c].sd, FB[c].sd);
        A5[c] = sub(FT[c].sd, FB[c].sd);
        A3[c] = sub(FT[c].ss, FB[c].ss);
        A4[c] = add(FT[c].dd, FB[c].dd);
        A7[c] = sub(FT[c].dd, FB[c].dd);
    }
    // ---- modal stiffness (scaled) ---------------------------------------------
    float2 Y1[3], Y2[3], Y3[3], Y4[3], Y5[3], Y6[3], Y7[3];
    {
        const float2 lt = mul(lam, add(add(A1[0], A2[1]), A3[2]));
        const float2 s00 = fma(twomu, A1[0], lt), s11 = fma(twomu, A2[1], lt), s22 = fma(twomu, A3[2], lt);
        const float2 s01 = mul(mu, add(A1[1], A2[0]));
        const float2 s02 = mul(mu, add(A1[2], A3[0]));
        const float2 s12 = mul(mu, add(A2[2], A3[1]));
        Y1[0] = mul(c1, s00); Y1[1] = mul(c1, s01); Y1[2] = mul(c1, s02);
        Y2[0] = Y1[1];        Y2[1] = mul(c1, s11); Y2[2] = mul(c1, s12);
        Y3[0] = Y1[2];        Y3[1] = Y2[2];        Y3[2] = mul(c1, s22);
        const float2 ltx = mul(lam, add(A4[1], A6[2]));
        const float2 lte = mul(lam, add(A4[0], A5[2]));
        const float2 ltz = mul(lam, add(A6[0], A5[1]));
        const float2 shx = mul(mu, add(A4[2], A6[1]));
        const float2 she = mul(mu, add(A4[2], A5[0]));
        const float2 shz = mul(mu, add(A6[1], A5[0]));
        Y4[0] = mul(c2, fma(thrmu, A4[0], lte));
        Y4[1] = mul(c2, fma(thrmu, A4[1], ltx));
        Y4[2] = mul(c2, add(shx, she));
        Y6[0] = mul(c2, fma(thrmu, A6[0], ltz));
        Y6[1] = mul(c2, add(shx, shz));
        Y6[2] = mul(c2, fma(thrmu, A6[2], ltx));
        Y5[0] = mul(c2, add(she, shz));
        Y5[1] = mul(c2, fma(thrmu, A5[1], ltz));
        Y5[2] = mul(c2, fma(thrmu, A5[2], lte));
#pragma unroll
        for (int c = 0; c < 3; ++c) Y7[c] = mul(c7, A7[c]);
    }
    // ---- transposed z stage; the bottom half joins the carry of the plane ----
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        Face P;  // face modes of plane ez: carried top half of layer ez-1 + bottom half of layer ez
        P.ss = sub(CT[c].ss, Y3[c]);
        P.sd = add(CT[c].sd, sub(Y2[c], Y5[c]));
        P.ds = add(CT[c].ds, sub(Y1[c], Y6[c]));
        P.dd = add(CT[c].dd, sub(Y4[c], Y7[c]));
        CT[c].ss = Y3[c];
        CT[c].sd = add(Y2[c], Y5[c]);
        CT[c].ds = add(Y1[c], Y6[c]);
        CT[c].dd = add(Y4[c], Y7[c]);
        // transposed y and x stages
        const float2 sHi = add(P.ss, P.sd), sLo = sub(P.ss, P.sd);
        const float2 dHi = add(P.ds, P.dd), dLo = sub(P.ds, P.dd);
        const float2 loR = add(sLo, dLo), loL = sub(sLo, dLo);
        const float2 hiR = add(sHi, dHi), hiL = sub(sHi, dHi);
        // rows: 0 <- first element lo; 1 <- first hi + second lo; 2 <- second hi
        const float R0 = loR.x, R1 = hiR.x + loR.y, R2 = hiR.y;
        V[0][c] = loL.x + __shfl_up_sync(0xffffffffu, R0, 1);
        V[1][c] = (hiL.x + loL.y) + __shfl_up_sync(0xffffffffu, R1, 1);
        V[2][c] = hiL.y + __shfl_up_sync(0xffffffffu, R2, 1);
    }
}
}  // namespace k2

// One tile (block B.b of B.n); ku2_kernel runs one tile per CTA, the batched
// persistent kernel one tile per work item.  UNPRED: node loads are not
// predicated on the grid bounds.  A lane then reads, for nodes outside the grid,
// whatever finite values lie there (padding, a neighbouring row or plane, or the
// ku2_slack() zero slack around the vectors); those values only enter elements
// outside the grid, whose scale is 0, so the result is bitwise the same as with
// zeros.  The vectors must be finite and allocated with ku2_slack() entries
// (kernels.cuh) on both sides.
template <int W, int MODE, bool UNPRED = false>
__device__ __forceinline__ void ku2_body(const Ku2Args &A, const Blk B) {
    using namespace k2;
    constexpr int TY = 2 * W - 1;
    __shared__ float xch[2][W][3][32];  // row-2 partials of each warp, double-buffered by layer
    __shared__ double red[2 * W];
    __shared__ int last_flag;

    if (MODE == KU_PCG && A.S->done) return;
    const Layout L = A.L;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int b = B.b;
    const int tx_ = b % A.tiles_x;
    b /= A.tiles_x;
    const int ty_ = b % A.tiles_y;
    const int tz_ = b / A.tiles_y;
    const int x0 = tx_ * 30, y0 = ty_ * TY, z0 = tz_ * A.tz;
    const int z1 = min(z0 + A.tz, L.nz + 1);
    // 32-bit node and element indices (the host guarantees 3 cs < 2^31): the
    // address arithmetic of the 30-odd loads and stores per lane and layer is the
    // largest integer cost of the kernel
    const int cs = (int)L.cs, sx = L.sx, sxy = (int)L.sxy, enx = L.nx, enxy = L.nx * L.ny;

    const int gx = x0 - 1 + lane;            // this lane's node column (element column for lanes < 31)
    const int gy0 = y0 - 1 + 2 * w;          // node rows gy0, gy0+1, gy0+2
    const bool col_in = gx >= 0 && gx <= L.nx;
    const bool row_in[3] = {gy0 >= 0 && gy0 <= L.ny, gy0 + 1 >= 0 && gy0 + 1 <= L.ny,
                            gy0 + 2 >= 0 && gy0 + 2 <= L.ny};
    const bool lane_owned = lane >= 1 && lane <= 30 && gx <= L.nx;
    // this lane's offsets of rows gy0 .. gy0+2 within a node plane (plane iz adds iz sxy)
    const int rowoff[3] = {gy0 * sx + gx, (gy0 + 1) * sx + gx, (gy0 + 2) * sx + gx};
    const bool rowok[3] = {col_in && row_in[0], col_in && row_in[1], col_in && row_in[2]};
    const int erowA = gy0 * enx + gx, erowB = (gy0 + 1) * enx + gx;  // element rows (layer ez adds ez nx ny)
    const bool elem_col = lane <= 30 && gx >= 0 && gx < L.nx;
    const bool elemA_row = gy0 >= 0 && gy0 < L.ny, elemB_row = gy0 + 1 >= 0 && gy0 + 1 < L.ny;

    const float *pin = nullptr;
    float *pout = nullptr;
    float beta = 0.f;
    if (MODE == KU_PCG) {
        const bool odd = (A.S->it & 1) != 0;
        pin = odd ? A.pb : A.pa;
        pout = odd ? A.pa : A.pb;
        beta = (float)A.S->beta;
    }
    const float2 lam = splat(A.M.lam), mu = splat(A.M.mu), twomu = splat(2.f * A.M.mu), thrmu = splat(3.f * A.M.mu);

    const float *__restrict__ gr = A.r;
    const float *__restrict__ gd = A.dinv;
    const float *__restrict__ gu = MODE == KU_PCG ? pin : A.u;
    const bool use_p = MODE != KU_PCG || beta != 0.f;
    // loads node values of plane iz (3 rows of this lane's column); PCG writes p.
    // Every load of the plane is issued before the first store so the three rows'
    // memory round trips overlap.
    auto load_plane = [&](int iz, float (&v)[3][3]) {
        float d[3], rv[3][3], pv[3][3];
        int n[3];
        bool ok[3];
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) {
            if constexpr (UNPRED) {
                ok[rr] = rowok[rr];  // stores happen only for iz in [z0, z1), inside the grid
                n[rr] = iz * sxy + rowoff[rr];
            } else {
                ok[rr] = rowok[rr] && iz >= 0 && iz <= L.nz;
                n[rr] = ok[rr] ? iz * sxy + rowoff[rr] : 0;
            }
            d[rr] = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) rv[rr][c] = pv[rr][c] = 0.f;
            if (UNPRED || ok[rr]) {
                if (MODE == KU_PCG) {
                    d[rr] = __ldg(gd + n[rr]);
#pragma unroll
                    for (int c = 0; c < 3; ++c) rv[rr][c] = __ldg(gr + n[rr] + c * cs);
                }
                if (use_p) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pv[rr][c] = __ldg(gu + n[rr] + c * cs);
                }
            }
        }
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                v[rr][c] = MODE == KU_PCG ? fmaf(beta, pv[rr][c], d[rr] * rv[rr][c]) : pv[rr][c];
        }
        if (MODE == KU_PCG && lane_owned && iz >= z0 && iz < z1) {
            // rows 1 and 2 (2 only below the last warp) are owned by this warp
#pragma unroll
            for (int rr = 1; rr < 3; ++rr) {
                if (!ok[rr] || (rr == 2 && w == W - 1)) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) pout[n[rr] + c * cs] = v[rr][c];
            }
        }
    };

    Face FB[3];         // face modes of the bottom plane of the current layer
    Face CT[3];         // transposed-transform face modes carried from the layer below
    float pcur[2][3];   // PCG: p of rows 0,1 on the plane completed by the current layer
    Acc<float> dot;
    {
        float v[3][3];
        load_plane(z0 - 1, v);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float n0 = __shfl_down_sync(0xffffffffu, v[0][c], 1);
            const float n1 = __shfl_down_sync(0xffffffffu, v[1][c], 1);
            const float n2 = __shfl_down_sync(0xffffffffu, v[2][c], 1);
            FB[c] = face_modes(v[0][c], v[1][c], v[2][c], n0, n1, n2);
            CT[c].ss = CT[c].sd = CT[c].ds = CT[c].dd = make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            pcur[0][c] = v[0][c];
            pcur[1][c] = v[1][c];
        }
    }

    const float *__restrict__ gs = A.s;
    const uint8_t *__restrict__ gm = A.mask;
    for (int ez = z0 - 1; ez < z1; ++ez) {
        // ---- element scales (0 outside the grid and for lane 31) and the
        // constraint bits of this layer's output nodes, issued first ----------------
        float sA = 0.f, sB = 0.f;
        if (elem_col && ez >= 0 && ez < L.nz) {
            if (elemA_row) sA = __ldg(gs + ez * enxy + erowA);
            if (elemB_row) sB = __ldg(gs + ez * enxy + erowB);
        }
        unsigned mrow[2] = {0u, 0u};
        if (MODE == KU_PCG && ez >= z0 && lane_owned) {
            if (row_in[0]) mrow[0] = __ldg(gm + ez * sxy + rowoff[0]);
            if (row_in[1]) mrow[1] = __ldg(gm + ez * sxy + rowoff[1]);
        }
        // ---- top plane of this layer -----------------------------------------
        float v[3][3];
        load_plane(ez + 1, v);
        Face FT[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float n0 = __shfl_down_sync(0xffffffffu, v[0][c], 1);
            const float n1 = __shfl_down_sync(0xffffffffu, v[1][c], 1);
            const float n2 = __shfl_down_sync(0xffffffffu, v[2][c], 1);
            FT[c] = face_modes(v[0][c], v[1][c], v[2][c], n0, n1, n2);
        }
        float V[3][3];  // node values of rows 0..2 of plane ez (this warp's part)
        layer_math(FB, FT, CT, make_float2(sA, sB), A.M, lam, mu, twomu, thrmu, V);
        // ---- shared row with the warp above -------------------------------------
        const int slot = ez & 1;
#pragma unroll
        for (int c = 0; c < 3; ++c) xch[slot][w][c][lane] = V[2][c];
        __syncthreads();
        if (w >= 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) V[0][c] += xch[slot][w - 1][c][lane];
        }
        // ---- outputs: rows 0 (w >= 1) and 1 of plane ez -------------------------
        if (ez >= z0 && lane_owned) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                if ((rr == 0 && w == 0) || !row_in[rr]) continue;
                const int n = ez * sxy + rowoff[rr];
                if (MODE == KU_PLAIN) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) A.y[n + c * cs] = V[rr][c];
                } else {
                    const unsigned m = mrow[rr];
                    float ds = 0.f;  // FP32 over a node's three DOFs, double-float across layers
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float q = ((m >> c) & 1u) ? 0.f : V[rr][c];
                        A.y[n + c * cs] = q;
                        ds = fmaf(pcur[rr][c], q, ds);
                    }
                    dot.add(ds);
                }
            }
        }
        // ---- carry to the next layer ------------------------------------------------
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            FB[c] = FT[c];
            pcur[0][c] = v[0][c];
            pcur[1][c] = v[1][c];
        }
    }
    if (MODE == KU_PLAIN) return;

    double dv[1] = {dot.value()};
    block_sum<1>(dv, red);
    if (threadIdx.x == 0) A.partial[2 * B.b] = dv[0];
    if (!arrive_last_n(&A.S->cnt_ku, &last_flag, B.n)) return;
    double tot[1];
    reduce_partials<1>(A.partial, B.n, 2, tot, red);
    if (threadIdx.x == 0) {
        Scalars *S = A.S;
        const double pq = tot[0];
        S->pq = pq;
        if (!(pq > 0.0) || !isfinite(pq)) {
            S->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
            S->done = 1;
            S->alpha = 0.0;
        } else {
            S->alpha = S->rz / pq;
        }
        S->cnt_ku = 0;
    }
}

template <int W, int MODE, bool UNPRED>
__global__ void __launch_bounds__(32 * W, 2) ku2_kernel(Ku2Args A) {
    ku2_body<W, MODE, UNPRED>(A, grid_blk());
}

}  // namespace amk
