// am_common.cuh -- device data layout, solver scalars and small helpers shared by
// the kernels of the GB300 SIMP engine.
//
// Device layout (chosen for coalescing, converted at the ABI boundary):
//   nodes   (ix, iy, iz), ix fastest: n = iz*sxy + iy*sx + ix, sx = (nx+1) rounded
//           up to a multiple of 4 (16-byte rows), sxy = sx*(ny+1);
//   vectors three component planes [3][cs], cs = sxy*(nz+1) rounded up to 64;
//   elements (ex, ey, ez), ex fastest: e = (ez*ny + ey)*nx + ex.
// Padding nodes (ix > nx, or n >= sxy*(nz+1)) hold zeros in every vector and are
// never written by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace amk {

struct Layout {
    int nx, ny, nz;     // elements per axis
    int sx;             // node row stride
    long long sxy;      // node plane stride
    long long cs;       // component stride of a vector
    long long nel;      // nx*ny*nz
};

__host__ __device__ inline long long node_index(const Layout &L, int ix, int iy, int iz) {
    return (long long)iz * L.sxy + (long long)iy * L.sx + ix;
}
__host__ __device__ inline long long elem_index(const Layout &L, int ex, int ey, int ez) {
    return ((long long)ez * L.ny + ey) * L.nx + ex;
}

// Constants of the hex8 element operator in the Walsh (trilinear monomial)
// basis: lam, mu are the Lame parameters; c1 = a/8, c2 = a/24, c3 = a/72 fold the
// quadrature weights (8, 8/3, 8/9 over [-1,1]^3), the Jacobian a = h/2 and the two
// 1/8 normalisations of the unnormalised transforms; c7 = c3 (lam + 4 mu).
template <typename T>
struct Modal {
    T lam, mu, c1, c2, c3, c7;
};

// Solver / OC scalars shared between kernels on the device.  Written only by the
// last block of a kernel (or by the host between launches).
struct Scalars {
    // PCG
    double rz, rr, pq, alpha, beta, thr;
    double rz_prev;     // r.z of the previous iteration (beta after a residual replacement)
    double thr_update;  // mixed precision: recursive |r|^2 that triggers a reliable update
    double alpha_prev;  // FP32 PCG: alpha of an even iteration whose alpha p is still owed to x
    int it, maxit, done, status;      // status: 0 ok, 1 converged, 2 max it, 3 breakdown, 4 nan,
                                      // 5 reliable update due
    // residual kernel results
    double res_rr, res_rz, energy;
    // OC bisection
    double l1, l2, oc_t, oc_cur, oc_t_last;
    int oc_pass, oc_done, oc_variant, pad0;
    double oc_change, oc_volume;
    // sensitivities
    double comp_fu, comp_energy;
    // outer flexible CG (FP64): z.r, z.q, alpha, beta, p.q, r.r
    double o_zr, o_zq, o_alpha, o_beta, o_pq, o_rr;
    int o_status, pad1;
    // last-block counters (one per kernel family so overlapping uses never clash)
    unsigned int cnt_ku, cnt_upd, cnt_oc, cnt_misc, cnt_fcg, pad2;
    // batched runs: |F|^2 on the free DOFs, and 1 once the problem's SIMP loop ended
    double b2;
    int frozen, pad3;
    // set by a kernel whose bounded wait on its bulk copies ran out (ST_TIMEOUT)
    int kerr;
    int loops;  // chunks run by the device-side loop of the current solve
};

enum { ST_RUNNING = 0, ST_CONVERGED = 1, ST_MAXIT = 2, ST_BREAKDOWN = 3, ST_NAN = 4, ST_UPDATE = 5, ST_TIMEOUT = 6 };

// Double-float accumulator: an unevaluated sum hi + lo of two floats.  Products of
// FP32 operands are added exactly (FMA error term) and the running sum keeps ~48
// significant bits, so FP32 dot products are accumulated to FP64-like accuracy on
// the FP32 pipes (FP64 throughput on GB300 is a small fraction of FP32).
struct DF {
    float hi, lo;
};
__device__ __forceinline__ void df_add_prod(DF &a, float x, float y) {
    const float p = x * y;
    const float pe = fmaf(x, y, -p);
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += e + pe;
}
__device__ __forceinline__ void df_add(DF &a, float p) {
    const float s = a.hi + p;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += e;
}
__device__ __forceinline__ double df_value(const DF &a) { return (double)a.hi + (double)a.lo; }

// Per-thread accumulator of a dot product: FP64 for double operands, double-float
// for float operands.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
    double v = 0.0;
    __device__ __forceinline__ void add_prod(double x, double y) { v = fma(x, y, v); }
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double value() const { return v; }
};
template <>
struct Acc<float> {
    DF v{0.f, 0.f};
    __device__ __forceinline__ void add_prod(float x, float y) { df_add_prod(v, x, y); }
    __device__ __forceinline__ void add(float x) { df_add(v, x); }
    __device__ __forceinline__ double value() const { return df_value(v); }
};

// Block-wide sum of NV doubles in a fixed order (deterministic).  `red` needs
// NV * (blockDim.x / 32) doubles of shared memory.  Result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[k * nw + wid] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += red[k * nw + w];
            v[k] = s;
        }
    }
    __syncthreads();
}

// Block-wide max of one double (result valid in thread 0).
__device__ __forceinline__ double block_max(double x, double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) red[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = red[0];
        for (int w = 1; w < nw; ++w) m = fmax(m, red[w]);
        x = m;
    }
    __syncthreads();
    return x;
}

// Block coordinates of a kernel body: the body runs either as a stand-alone grid
// (b = blockIdx.x, n = gridDim.x) or as one work item of a batched persistent
// grid (b = the item's block within its problem, n = that problem's block count).
struct Blk {
    int b, n;
};
__device__ __forceinline__ Blk grid_blk() { return Blk{(int)blockIdx.x, (int)gridDim.x}; }

// Last-block-done protocol: every block of a body publishes its partials, then
// the block that arrives last (ticket == nblocks - 1) reduces them in index order
// and resets the counter.  Returns true in every thread of the last block.
__device__ __forceinline__ bool arrive_last_n(unsigned int *counter, int *flag_smem, int nblocks) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(counter, 1u);
        *flag_smem = (t == (unsigned int)nblocks - 1u) ? 1 : 0;
    }
    __syncthreads();
    if (*flag_smem) __threadfence();
    return *flag_smem != 0;
}
__device__ __forceinline__ bool arrive_last(unsigned int *counter, int *flag_smem) {
    return arrive_last_n(counter, flag_smem, (int)gridDim.x);
}
// The same hand-off for a block that arrives for `weight` of the `total` work
// items at once (it published their partials together).
__device__ __forceinline__ bool arrive_last_weighted(unsigned int *counter, int *flag_smem, int weight, int total) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(counter, (unsigned int)weight);
        *flag_smem = (t + (unsigned int)weight == (unsigned int)total) ? 1 : 0;
    }
    __syncthreads();
    if (*flag_smem) __threadfence();
    return *flag_smem != 0;
}

// Sum partial[b*stride + k] over b in [0, nb) in a fixed order, for k < NV.
// Called by all threads of one block; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void reduce_partials(const double *partial, int nb, int stride,
                                                double (&out)[NV], double *red) {
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] += __ldcg(partial + (long long)b * stride + k);
    }
    block_sum<NV>(out, red);
}

// std::min / std::max of the C++ reference (min(a,b) = b < a ? b : a).
template <typename T>
__device__ __forceinline__ T cmin(T a, T b) { return (b < a) ? b : a; }
template <typename T>
__device__ __forceinline__ T cmax(T a, T b) { return (a < b) ? b : a; }
// numpy.minimum / numpy.maximum (NaN propagates).
template <typename T>
__device__ __forceinline__ T npmin(T a, T b) { return (a != a || b != b) ? (a + b) : (a < b ? a : b); }
template <typename T>
__device__ __forceinline__ T npmax(T a, T b) { return (a != a || b != b) ? (a + b) : (a > b ? a : b); }

}  // namespace amk
