// kudf.cuh -- the FP64-accurate residual r = mask(f - K u) and outer product
// q = mask(K p) of the mixed-precision solvers in double-float arithmetic on the
// FP32 pipes.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and the residual
// replacements of the mixed solver (one FP64 K*u every time the FP32 recursion
// has gained a decade, about eight per solve) were its largest FP64 cost.  Here
// the same tile kernel as ku.cuh (same staging, element order and node gather)
// evaluates hex8_apply on `dflt` values: an unevaluated sum hi + lo of two floats,
// ~48 significant bits, whose sums and products are formed with the exact
// two-sum and FMA-based two-product error terms (Dekker / Knuth; the
// "double-float" / "double-single" arithmetic of the GPU literature).  Inputs and
// outputs stay FP64: u is split on staging, r = f - K u is subtracted in FP64 from
// the recombined product, and r.r, r.dinv.r and the element energies are summed in
// FP64.  The rounding error of a double-float sum is a few units of 2^-48 of its
// operands, against 2^-53 for FP64: the residual agrees with the FP64 kernel's to
// ~1e-12 of |f| (tested), far below the 1e-6 the solver accepts on.
#pragma once
#include "ku.cuh"

namespace amk {

struct dflt {
    float hi, lo;
    dflt() = default;
    __host__ __device__ constexpr dflt(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr dflt(int z) : hi((float)z), lo(0.f) {}
};

// round-to-nearest float operations that the compiler never contracts or reorders
// (the error terms below depend on each rounding)
__host__ __device__ __forceinline__ float rn_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float s = a + b;
    return s;
#endif
}
__host__ __device__ __forceinline__ float rn_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float s = a - b;
    return s;
#endif
}
__host__ __device__ __forceinline__ float rn_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float s = a * b;
    return s;
#endif
}
__host__ __device__ __forceinline__ float rn_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// hi + lo of x rounded to the nearest pair
__host__ __device__ __forceinline__ dflt to_dflt(double x) {
    const float h = (float)x;
    return dflt(h, (float)(x - (double)h));
}
__host__ __device__ __forceinline__ double from_dflt(dflt a) { return (double)a.hi + (double)a.lo; }

// s = a + b with its exact error (Knuth's two-sum: no magnitude ordering needed)
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = rn_add(a, b);
    const float bb = rn_sub(s, a);
    e = rn_add(rn_sub(a, rn_sub(s, bb)), rn_sub(b, bb));
}
// renormalise (|s| >= |e| up to the rounding of s)
__host__ __device__ __forceinline__ dflt fast_renorm(float s, float e) {
    const float h = rn_add(s, e);
    return dflt(h, rn_sub(e, rn_sub(h, s)));
}
__host__ __device__ __forceinline__ dflt operator+(dflt a, dflt b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = rn_add(e, rn_add(a.lo, b.lo));
    return fast_renorm(s, e);
}
__host__ __device__ __forceinline__ dflt operator-(dflt a) { return dflt(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dflt operator-(dflt a, dflt b) { return a + (-b); }
__host__ __device__ __forceinline__ dflt operator*(dflt a, dflt b) {
    const float p = rn_mul(a.hi, b.hi);
    float e = rn_fma(a.hi, b.hi, -p);  // exact error of the product
    e = rn_fma(a.hi, b.lo, rn_fma(a.lo, b.hi, e));
    return fast_renorm(p, e);
}
__host__ __device__ __forceinline__ dflt &operator+=(dflt &a, dflt b) {
    a = a + b;
    return a;
}
__host__ __device__ __forceinline__ bool operator!=(dflt a, dflt b) { return a.hi != b.hi || a.lo != b.lo; }

inline Modal<dflt> modal_dflt(const Modal<double> &M) {
    return Modal<dflt>{to_dflt(M.lam), to_dflt(M.mu), to_dflt(M.c1), to_dflt(M.c2), to_dflt(M.c3), to_dflt(M.c7)};
}

// The ku_tile_body RESID and DOT passes with the element operator and the node
// gather in double-float: staged planes and element corner sums hold dflt (8
// bytes, the shared-memory layout of the FP64 kernel); u, f, s, dinv, the output
// (r = mask(f - K u), or q = mask(K u) for DOT) and ce are FP64.
template <int TX, int TY, int MODE = KU_RESID>
__device__ __forceinline__ void ku_df_body(const KuArgs<double> &A, const Modal<dflt> &M, const Blk B) {
    static_assert(MODE == KU_RESID || MODE == KU_DOT, "double-float K*u: residual or outer product");
    using Sh = KuShape<TX, TY>;
    constexpr int EX = Sh::EX, NE = Sh::NE, SX = Sh::SX, NS = Sh::NS, NT = Sh::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    dflt *us = reinterpret_cast<dflt *>(smem_raw);  // [2 slots][3][NS]
    dflt *yb = us + 2 * 3 * NS;                     // [8 corners][3][NE]
    __shared__ double red[2 * (NT / 32)];
    __shared__ int last_flag;

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

    auto stage = [&](int iz, int slot) {
        dflt *dst = us + slot * 3 * NS;
        for (int t = tid; t < NS; t += NT) {
            const int lx = t % SX, ly = t / SX;
            const int ix = x0 - 1 + lx, iy = y0 - 1 + ly;
            dflt v0(0), v1(0), v2(0);
            if (ix >= 0 && ix <= L.nx && iy >= 0 && iy <= L.ny && iz >= 0 && iz <= L.nz) {
                const long long n = node_index(L, ix, iy, iz);
                v0 = to_dflt(A.u[n]);
                v1 = to_dflt(A.u[n + cs]);
                v2 = to_dflt(A.u[n + 2 * cs]);
            }
            dst[t] = v0;
            dst[NS + t] = v1;
            dst[2 * NS + t] = v2;
        }
    };

    dflt acc[3] = {dflt(0), dflt(0), dflt(0)};
    Acc<double> d0, d1;  // r.r, r.dinv.r
    stage(z0 - 1, (z0 - 1) & 1);
    for (int ez = z0 - 1; ez < z1; ++ez) {
        stage(ez + 1, (ez + 1) & 1);
        __syncthreads();
        if (tid < NE) {
            const int exl = tid % EX, eyl = tid / EX;
            const int ex = x0 - 1 + exl, ey = y0 - 1 + eyl;
            double se = 0.0;
            long long e = -1;
            if (ex >= 0 && ex < L.nx && ey >= 0 && ey < L.ny && ez >= 0 && ez < L.nz) {
                e = elem_index(L, ex, ey, ez);
                se = A.s[e];
            }
            dflt yo[3][8];
            const bool want_en = MODE == KU_RESID && A.energy && e >= 0 && exl >= 1 && eyl >= 1 && ez >= z0;
            if (se != 0.0 || want_en) {
                const dflt *ub = us + (ez & 1) * 3 * NS;
                const dflt *ut = us + ((ez + 1) & 1) * 3 * NS;
                const int i00 = eyl * SX + exl;
                dflt uu[3][8];
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
                dflt en(0);
                hex8_apply<dflt>(uu, yo, M, to_dflt(se), want_en ? &en : nullptr);
                if (want_en) A.ce[e] = from_dflt(en);
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int k = 0; k < 8; ++k) yo[c][k] = dflt(0);
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
            dflt val[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const dflt bot = yb[(2 * 3 + c) * NE + e00] + yb[(3 * 3 + c) * NE + e10] +
                                 yb[(1 * 3 + c) * NE + e01] + yb[(0 * 3 + c) * NE + e11];
                const dflt top = yb[(6 * 3 + c) * NE + e00] + yb[(7 * 3 + c) * NE + e10] +
                                 yb[(5 * 3 + c) * NE + e01] + yb[(4 * 3 + c) * NE + e11];
                val[c] = acc[c] + bot;
                acc[c] = top;
            }
            const int ix = x0 + lx, iy = y0 + ly;
            if (ez >= z0 && ix <= L.nx && iy <= L.ny) {
                const long long n = node_index(L, ix, iy, ez);
                const unsigned m = A.mask[n];
                if (MODE == KU_RESID) {
                    const double dv = A.dinv ? A.dinv[n] : 0.0;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        // f - (hi + lo): the two FP64 subtractions keep the product's ~48 bits
                        const double rr =
                            ((m >> c) & 1u) ? 0.0 : (A.f[n + c * cs] - (double)val[c].hi) - (double)val[c].lo;
                        A.y[n + c * cs] = rr;
                        d0.add_prod(rr, rr);
                        d1.add_prod(rr, dv * rr);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double q = ((m >> c) & 1u) ? 0.0 : from_dflt(val[c]);
                        A.y[n + c * cs] = q;
                        d0.add_prod(A.u[n + c * cs], q);
                    }
                }
            }
        }
    }

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
        if (MODE == KU_DOT) {
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

template <int TX, int TY, int MODE>
__global__ void __launch_bounds__(KuShape<TX, TY>::NT) ku_df_kernel(KuArgs<double> A, Modal<dflt> M) {
    ku_df_body<TX, TY, MODE>(A, M, grid_blk());
}

}  // namespace amk
