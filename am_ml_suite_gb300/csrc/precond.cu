// precond.cu -- the learned preconditioner: a 4-level 3-D convolutional
// encoder-decoder (16/32/64/128 channels, 3x3x3 kernels, skip connections,
// BF16 weights and activations, FP32 accumulate) applied to residuals on the
// node grid, trained on the GPU with Adam by the engine's own kernels
// (conv3d.cu for the network, the FP32 K*u for the loss).
//
// The network works on the Jacobi-scaled system K~ = D^-1/2 K D^-1/2 (unit
// diagonal).  For a residual r it takes r~ = D^-1/2 r / rms(D^-1/2 r) (three node
// channels) and the node densities (a fourth channel) and returns the correction
// N(r~); the preconditioned vector is z = D^-1/2 (r~ + N(r~)) rms.  With the last
// layer initialised to zero the untrained network is exactly Jacobi.  Training
// minimises |K~ (r~ + N(r~)) - r~|^2 / |r~|^2 over residuals harvested from the
// engine's own PCG solves.
//
// Layers (conv 3x3x3 + ReLU unless noted; e = encoder, d = decoder, cat = the
// concatenation buffers that the skip tensors are written into in place):
//   L0  in(4, padded to 16) -> 16     L1  16 -> 16  = e1 -> cat1[32:48]
//   L2  pool(e1) 16 -> 32             L3  32 -> 32  = e2 -> cat2[64:96]
//   L4  pool(e2) 32 -> 64             L5  64 -> 64  = e3 -> cat3[128:192]
//   L6  pool(e3) 64 -> 128            L7  128 -> 128 = e4
//   L8  cat3 = [up(e4), e3] 192 -> 64 L9  64 -> 64  = d3
//   L10 cat2 = [up(d3), e2] 96 -> 32  L11 32 -> 32  = d2
//   L12 cat1 = [up(d2), e1] 48 -> 16  L13 16 -> 16  = d1
//   L14 16 -> 16 (3 used), no ReLU, FP32 output
// pool = 2x2x2 mean, up = nearest 2x; 1,472,256 stored weights, 1,461,456 of them
// trainable (the rest pad channel counts to multiples of 16); no biases.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "conv3d.cuh"
#include "kernels.cuh"
#include "precond.h"

using namespace amk;

namespace {

am_status pfail(am_status s, const std::string &msg) {
    set_last_error(msg.c_str());
    return s;
}
#define PCK(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return pfail(e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,      \
                         std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)
#define PCKS(expr)                  \
    do {                            \
        am_status s_ = (expr);      \
        if (s_ != AM_OK) return s_; \
    } while (0)

typedef __nv_bfloat16 bf16;

// AM_ERR_TIMEOUT if a tensor-core convolution on `st` gave up a bounded wait
am_status conv_status(cudaStream_t st) {
    int f = 0;
    PCK(conv3d_tc_error(&f, true, st));
    if (f) return pfail(AM_ERR_TIMEOUT, "a bounded copy / MMA wait of a tensor-core convolution ran out");
    return AM_OK;
}


struct LayerSpec {
    int cin, cout, cin_used, cout_used;
};
constexpr int kLayers = 15;
constexpr LayerSpec kSpec[kLayers] = {{16, 16, 4, 16},   {16, 16, 16, 16},   {16, 32, 16, 32},  {32, 32, 32, 32},
                                      {32, 64, 32, 64},  {64, 64, 64, 64},   {64, 128, 64, 128}, {128, 128, 128, 128},
                                      {192, 64, 192, 64}, {64, 64, 64, 64},  {96, 32, 96, 32},  {32, 32, 32, 32},
                                      {48, 16, 48, 16},  {16, 16, 16, 16},   {16, 16, 16, 3}};

template <typename T>
struct Buf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        if (p && n >= count) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) {
            n = count;
            e = cudaMemset(p, 0, std::max<size_t>(count, 1) * sizeof(T));
        }
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// activation and gradient tensors of one (batch, grid) shape
struct Acts {
    int n = 0, gz = 0, gy = 0, gx = 0;
    bool grads = false;
    Buf<bf16> pool;
    Buf<float> out;
    bf16 *x0, *a0, *cat1, *p1, *a2, *cat2, *p2, *a4, *cat3, *p3, *a6, *e4, *a8, *d3, *a10, *d2, *a12, *d1;
    bf16 *gout, *g_d1, *g_a12, *g_cat1, *g_d2, *g_a10, *g_cat2, *g_d3, *g_a8, *g_cat3, *g_e4, *g_a6, *g_p3, *g_a4,
        *g_p2, *g_a2, *g_p1, *g_a0;
    Grid5 G(int level) const { return Grid5{n, gz >> level, gy >> level, gx >> level}; }
};

cudaError_t ensure_acts(Acts &A, int n, int gz, int gy, int gx, bool grads) {
    if (A.pool.p && A.n == n && A.gz == gz && A.gy == gy && A.gx == gx && (A.grads || !grads)) return cudaSuccess;
    A.n = n;
    A.gz = gz;
    A.gy = gy;
    A.gx = gx;
    A.grads = grads;
    const size_t V1 = (size_t)n * gz * gy * gx, V2 = V1 / 8, V3 = V1 / 64, V4 = V1 / 512;
    struct Req {
        bf16 **p;
        size_t count;
    };
    std::vector<Req> req = {{&A.x0, V1 * 16},  {&A.a0, V1 * 16},   {&A.cat1, V1 * 48}, {&A.p1, V2 * 16},
                            {&A.a2, V2 * 32},  {&A.cat2, V2 * 96}, {&A.p2, V3 * 32},   {&A.a4, V3 * 64},
                            {&A.cat3, V3 * 192}, {&A.p3, V4 * 64}, {&A.a6, V4 * 128},  {&A.e4, V4 * 128},
                            {&A.a8, V3 * 64},  {&A.d3, V3 * 64},   {&A.a10, V2 * 32},  {&A.d2, V2 * 32},
                            {&A.a12, V1 * 16}, {&A.d1, V1 * 16}};
    if (grads) {
        std::vector<Req> g = {{&A.gout, V1 * 16},  {&A.g_d1, V1 * 16},   {&A.g_a12, V1 * 16}, {&A.g_cat1, V1 * 48},
                              {&A.g_d2, V2 * 32},  {&A.g_a10, V2 * 32},  {&A.g_cat2, V2 * 96}, {&A.g_d3, V3 * 64},
                              {&A.g_a8, V3 * 64},  {&A.g_cat3, V3 * 192}, {&A.g_e4, V4 * 128}, {&A.g_a6, V4 * 128},
                              {&A.g_p3, V4 * 64},  {&A.g_a4, V3 * 64},   {&A.g_p2, V3 * 32},  {&A.g_a2, V2 * 32},
                              {&A.g_p1, V2 * 16},  {&A.g_a0, V1 * 16}};
        req.insert(req.end(), g.begin(), g.end());
    }
    size_t tot = 0;
    for (auto &r : req) tot += (r.count + 127) / 128 * 128;
    A.pool.release();
    cudaError_t e = A.pool.alloc(tot);
    if (e != cudaSuccess) return e;
    size_t o = 0;
    for (auto &r : req) {
        *r.p = A.pool.p + o;
        o += (r.count + 127) / 128 * 128;
    }
    if (!grads) {
        A.gout = A.g_d1 = A.g_a12 = A.g_cat1 = A.g_d2 = A.g_a10 = A.g_cat2 = A.g_d3 = A.g_a8 = A.g_cat3 = nullptr;
        A.g_e4 = A.g_a6 = A.g_p3 = A.g_a4 = A.g_p2 = A.g_a2 = A.g_p1 = A.g_a0 = nullptr;
    }
    A.out.release();
    return A.out.alloc(V1 * 16);
}

TensorView tv(void *p, int cs, int co = 0) { return TensorView{p, cs, co}; }
TensorView none() { return TensorView{nullptr, 0, 0}; }

// ---------------------------------------------------------------------------
// residual <-> network tensors
// ---------------------------------------------------------------------------
// One density of the training set (or of the problem being preconditioned).
struct DensityDev {
    float *s32 = nullptr;   // element scales (training only)
    float *dsq = nullptr;   // D^-1/2 per node, 0 on masked nodes
    float *rhon = nullptr;  // node density (mean of the adjacent elements)
    uint8_t *mask = nullptr;
};

__global__ void node_fields_kernel(Layout L, const float *__restrict__ dinv, const double *__restrict__ rho,
                                   float *__restrict__ dsq, float *__restrict__ rhon) {
    const long long nn = L.sxy * (L.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        if (ix > L.nx) continue;
        dsq[n] = sqrtf(fmaxf(dinv[n], 0.f));
        double s = 0.0;
        int c = 0;
        for (int dz = -1; dz <= 0; ++dz)
            for (int dy = -1; dy <= 0; ++dy)
                for (int dx = -1; dx <= 0; ++dx) {
                    const int ex = ix + dx, ey = iy + dy, ez = iz + dz;
                    if (ex < 0 || ex >= L.nx || ey < 0 || ey >= L.ny || ez < 0 || ez >= L.nz) continue;
                    s += rho[elem_index(L, ex, ey, ez)];
                    ++c;
                }
        rhon[n] = c ? (float)(s / c) : 0.f;
    }
}

// per batch entry: residual (FP32 or FP64 [3][cs]), node fields, scale
struct PackSrc {
    const float *r32;
    const double *r64;
    const float *dsq, *rhon;
    const uint8_t *mask;
    double inv_scale;  // r~ = dsq r * inv_scale (FP64 input) or r32 already scaled (inv_scale = 1)
};

// x0[b][z][y][x][0:16] = (r~x, r~y, r~z, rho_node, 0...), zero outside the node grid
__global__ void pack_input_kernel(Layout L, int gz, int gy, int gx, const PackSrc *src, bf16 *x0, int nbatch) {
    const long long V = (long long)nbatch * gz * gy * gx;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        long long t = v;
        const int x = (int)(t % gx);
        t /= gx;
        const int y = (int)(t % gy);
        t /= gy;
        const int z = (int)(t % gz);
        const int b = (int)(t / gz);
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        if (x <= L.nx && y <= L.ny && z <= L.nz) {
            const PackSrc &S = src[b];
            const long long n = node_index(L, x, y, z);
            const uint8_t m = S.mask[n];
            for (int k = 0; k < 3; ++k) {
                if ((m >> k) & 1u) continue;
                c[k] = S.r32 ? S.r32[n + k * L.cs] : (float)(S.dsq[n] * S.r64[n + k * L.cs] * S.inv_scale);
            }
            c[3] = S.rhon[n];
        }
        __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(x0 + v * 16);
        o[0] = __floats2bfloat162_rn(c[0], c[1]);
        o[1] = __floats2bfloat162_rn(c[2], c[3]);
#pragma unroll
        for (int k = 2; k < 8; ++k) o[k] = __floats2bfloat162_rn(0.f, 0.f);
    }
}

// sum over free DOFs of (dsq r)^2 (FP64 input) -> *out
__global__ void scaled_norm_kernel(Layout L, const double *r, const float *dsq, const uint8_t *mask, double *out) {
    __shared__ double red[256 / 32];
    double s = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const uint8_t m = mask[n];
        for (int k = 0; k < 3; ++k) {
            if ((m >> k) & 1u) continue;
            const double v = (double)dsq[n] * r[n + k * L.cs];
            s += v * v;
        }
    }
    double v[1] = {s};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) atomicAdd(out, v[0]);
}

// z = dsq (r~ + N(r~)) * scale on free DOFs (inference); r~ recomputed from r
__global__ void apply_out_kernel(Layout L, int gz, int gy, int gx, const double *r, const float *dsq,
                                 const uint8_t *mask, const float *out, const double *nrm2, double nfree, double *z) {
    const double rms = sqrt(fmax(*nrm2, 1e-300) / fmax(nfree, 1.0));
    const long long nn = L.cs;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        const bool real = iz <= L.nz && ix <= L.nx;
        const uint8_t m = real ? mask[n] : 7;
        const long long v = ((long long)iz * gy + iy) * gx + ix;
        for (int k = 0; k < 3; ++k) {
            double val = 0.0;
            if (!((m >> k) & 1u)) {
                const double rt = (double)dsq[n] * r[n + k * L.cs] / rms;
                val = (double)dsq[n] * (rt + (double)out[v * 16 + k]) * rms;
            }
            z[n + k * L.cs] = val;
        }
    }
}

// training loss, step 1: u = dsq (r~ + N) on free DOFs
__global__ void make_u_kernel(Layout L, int gz, int gy, int gx, const float *r, const float *dsq, const uint8_t *mask,
                              const float *out, float *u) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        const bool real = iz <= L.nz && ix <= L.nx;
        const uint8_t m = real ? mask[n] : 7;
        const long long v = ((long long)iz * gy + iy) * gx + ix;
        for (int k = 0; k < 3; ++k)
            u[n + k * L.cs] = ((m >> k) & 1u) ? 0.f : dsq[n] * (r[n + k * L.cs] + out[v * 16 + k]);
    }
}

// step 2: e = dsq (K u) - r~ on free DOFs; |e|^2, |r~|^2 -> acc[0..1]; u := dsq e
__global__ void resid_kernel(Layout L, const float *r, const float *dsq, const uint8_t *mask, const float *y, float *u,
                             double *acc) {
    __shared__ double red[2 * (256 / 32)];
    double ee = 0.0, rr = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const uint8_t m = mask[n];
        for (int k = 0; k < 3; ++k) {
            const long long i = n + k * L.cs;
            float e = 0.f;
            if (!((m >> k) & 1u)) {
                e = dsq[n] * y[i] - r[i];
                rr += (double)r[i] * r[i];
            }
            ee += (double)e * e;
            u[i] = dsq[n] * e;
        }
    }
    double v[2] = {ee, rr};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        atomicAdd(acc, v[0]);
        atomicAdd(acc + 1, v[1]);
    }
}

// step 3: d loss / d N = coef * dsq (K dsq e) on free DOFs, written as BF16
// channels 0..2 of gout (the other channels stay zero)
__global__ void grad_out_kernel(Layout L, int gz, int gy, int gx, const float *dsq, const uint8_t *mask,
                                const float *y, const double *acc, double scale, bf16 *gout) {
    const double coef = 2.0 * scale / fmax(acc[1], 1e-300);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        if (iz > L.nz || ix > L.nx) continue;
        const uint8_t m = mask[n];
        const long long v = ((long long)iz * gy + iy) * gx + ix;
        for (int k = 0; k < 3; ++k) {
            const float g = ((m >> k) & 1u) ? 0.f : (float)(coef * dsq[n] * y[n + k * L.cs]);
            gout[v * 16 + k] = __float2bfloat16(g);
        }
    }
}

// harvested residual -> r~ = dsq r / rms (stored FP32 in the training set)
__global__ void scale_sample_kernel(Layout L, const float *r, const float *dsq, const uint8_t *mask, float *out,
                                    const double *nrm2, double nfree) {
    const double rms = sqrt(fmax(*nrm2, 1e-300) / fmax(nfree, 1.0));
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const uint8_t m = mask[n];
        for (int k = 0; k < 3; ++k) {
            const long long i = n + k * L.cs;
            out[i] = ((m >> k) & 1u) ? 0.f : (float)((double)dsq[n] * r[i] / rms);
        }
    }
}

// e~ = (xstar - xk) / (dsq rms) on free DOFs (the ideal network output
// r~ + N(r~) for this residual)
__global__ void scale_error_kernel(Layout L, const double *xstar, const double *xk, const float *dsq,
                                   const uint8_t *mask, float *out, const double *nrm2, double nfree) {
    const double rms = sqrt(fmax(*nrm2, 1e-300) / fmax(nfree, 1.0));
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const uint8_t m = mask[n];
        for (int k = 0; k < 3; ++k) {
            const long long i = n + k * L.cs;
            out[i] = (((m >> k) & 1u) || !(dsq[n] > 0.f)) ? 0.f
                                                          : (float)((xstar[i] - xk[i]) / ((double)dsq[n] * rms));
        }
    }
}

// energy-norm (direction) loss: a = z~.r~, b = z~.K~z~ (K~z~ = dsq y), d = e~.r~
// (= e~.K~e~) -> acc[0..2]
__global__ void energy_sums_kernel(Layout L, int gz, int gy, int gx, const float *r, const float *et,
                                   const float *dsq, const uint8_t *mask, const float *out, const float *y,
                                   double *acc) {
    __shared__ double red[3 * (256 / 32)];
    double sa = 0.0, sb = 0.0, sd = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        if (iz > L.nz || ix > L.nx) continue;
        const uint8_t m = mask[n];
        const long long v = ((long long)iz * gy + iy) * gx + ix;
        for (int k = 0; k < 3; ++k) {
            if ((m >> k) & 1u) continue;
            const long long i = n + k * L.cs;
            const double z = (double)r[i] + out[v * 16 + k];
            sa += z * r[i];
            sb += z * dsq[n] * y[i];
            sd += (double)et[i] * r[i];
        }
    }
    double w[3] = {sa, sb, sd};
    block_sum<3>(w, red);
    if (threadIdx.x == 0) {
        atomicAdd(acc, w[0]);
        atomicAdd(acc + 1, w[1]);
        atomicAdd(acc + 2, w[2]);
    }
}

// d L / d N for L = 1 - a^2 / (b d): (2a / (b d)) ((a / b) K~z~ - r~), times scale
__global__ void energy_grad_kernel(Layout L, int gz, int gy, int gx, const float *r, const float *dsq,
                                   const uint8_t *mask, const float *y, const double *acc, double scale, bf16 *gout) {
    const double a = acc[0], b = fmax(acc[1], 1e-300), d = fmax(acc[2], 1e-300);
    const double c1 = scale * 2.0 * a / (b * d), c2 = a / b;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        if (iz > L.nz || ix > L.nx) continue;
        const uint8_t m = mask[n];
        const long long v = ((long long)iz * gy + iy) * gx + ix;
        for (int k = 0; k < 3; ++k) {
            const long long i = n + k * L.cs;
            const float g = ((m >> k) & 1u) ? 0.f : (float)(c1 * (c2 * dsq[n] * y[i] - (double)r[i]));
            gout[v * 16 + k] = __float2bfloat16(g);
        }
    }
}

__global__ void scaled_norm32_kernel(Layout L, const float *r, const float *dsq, const uint8_t *mask, double *out,
                                     double *nfree) {
    __shared__ double red[2 * (256 / 32)];
    double s = 0.0, c = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int ix = (int)(rem % L.sx);
        if (iz > L.nz || ix > L.nx) continue;
        const uint8_t m = mask[n];
        for (int k = 0; k < 3; ++k) {
            if ((m >> k) & 1u) continue;
            const double v = (double)dsq[n] * r[n + k * L.cs];
            s += v * v;
            c += 1.0;
        }
    }
    double v[2] = {s, c};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        atomicAdd(out, v[0]);
        if (nfree) atomicAdd(nfree, v[1]);
    }
}

__global__ void count_free_kernel(Layout L, const uint8_t *mask, double *out) {
    __shared__ double red[256 / 32];
    double c = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int ix = (int)(rem % L.sx);
        if (iz > L.nz || ix > L.nx) continue;
        const uint8_t m = mask[n];
        c += (double)(3 - ((m & 1) + ((m >> 1) & 1) + ((m >> 2) & 1)));
    }
    double v[1] = {c};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) atomicAdd(out, v[0]);
}

// host-layout tensors (n, gz, gy, gx, c) FP32 <-> network tensors
__global__ void host_in_kernel(long long V, const float *in, int c, bf16 *x0) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < 16; ++k) x0[v * 16 + k] = __float2bfloat16(k < c ? in[v * c + k] : 0.f);
}
__global__ void host_out_kernel(long long V, const float *out16, int c, float *out) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < c; ++k) out[v * c + k] = out16[v * 16 + k];
}
__global__ void host_gout_kernel(long long V, const float *dout, int c, bf16 *g) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < 16; ++k) g[v * 16 + k] = __float2bfloat16(k < c ? dout[v * c + k] : 0.f);
}

int eb(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

int round8(int v) { return (v + 7) / 8 * 8; }

}  // namespace

struct am_precond {
    int device = 0;
    cudaStream_t st = nullptr;
    // parameters: FP32 master, Adam moments, gradient; BF16 forward and
    // flipped-transposed (backward-data) copies
    size_t off[kLayers + 1] = {};
    Buf<float> w, m, v, g;
    Buf<bf16> wb, wt;
    int adam_t = 0;
    // training set (one grid)
    bool has_grid = false;
    Layout L{};
    Modal<float> M32{};
    KuLaunch plan{};
    int gz = 0, gy = 0, gx = 0;
    long long capacity = 0, nsamples = 0;
    Buf<float> r;  // [capacity][3][cs] r~
    Buf<float> e;  // [capacity][3][cs] e~ = D^1/2 (xstar - xk) / rms (energy-norm loss)
    std::vector<int> sample_dens;
    std::vector<char> sample_err;  // 1 if e~ is stored
    std::vector<DensityDev> dens;
    double nfree_train = 0.0;
    // scratch
    Acts train, infer;
    Buf<float> u, y;
    Buf<double> acc;
    Buf<PackSrc> packsrc;
    Buf<float> hin, hout;  // host-layout tensors of the test entry points
    Buf<float> dens_scratch_dsq, dens_scratch_rhon;
    int infer_L_key[3] = {-1, -1, -1};
};

namespace {

// forward pass of the U-Net on A.x0 -> A.out
cudaError_t forward(am_precond *M, Acts &A, cudaStream_t st) {
    const Grid5 g1 = A.G(0), g2 = A.G(1), g3 = A.G(2), g4 = A.G(3);
    auto W = [&](int l) { return M->wb.p + M->off[l]; };
    auto conv = [&](int l, const Grid5 &g, TensorView x, TensorView y, TensorView yf, int relu) {
        return conv3d_fwd(g, x, kSpec[l].cin, W(l), kSpec[l].cout, y, yf, relu, st);
    };
    cudaError_t e;
#define FW(call) \
    if ((e = (call)) != cudaSuccess) return e
    FW(conv(0, g1, tv(A.x0, 16), tv(A.a0, 16), none(), 1));
    FW(conv(1, g1, tv(A.a0, 16), tv(A.cat1, 48, 32), none(), 1));
    FW(avgpool2_fwd(g2, tv(A.cat1, 48, 32), tv(A.p1, 16), 16, st));
    FW(conv(2, g2, tv(A.p1, 16), tv(A.a2, 32), none(), 1));
    FW(conv(3, g2, tv(A.a2, 32), tv(A.cat2, 96, 64), none(), 1));
    FW(avgpool2_fwd(g3, tv(A.cat2, 96, 64), tv(A.p2, 32), 32, st));
    FW(conv(4, g3, tv(A.p2, 32), tv(A.a4, 64), none(), 1));
    FW(conv(5, g3, tv(A.a4, 64), tv(A.cat3, 192, 128), none(), 1));
    FW(avgpool2_fwd(g4, tv(A.cat3, 192, 128), tv(A.p3, 64), 64, st));
    FW(conv(6, g4, tv(A.p3, 64), tv(A.a6, 128), none(), 1));
    FW(conv(7, g4, tv(A.a6, 128), tv(A.e4, 128), none(), 1));
    FW(upsample2_fwd(g3, tv(A.e4, 128), tv(A.cat3, 192, 0), 128, st));
    FW(conv(8, g3, tv(A.cat3, 192), tv(A.a8, 64), none(), 1));
    FW(conv(9, g3, tv(A.a8, 64), tv(A.d3, 64), none(), 1));
    FW(upsample2_fwd(g2, tv(A.d3, 64), tv(A.cat2, 96, 0), 64, st));
    FW(conv(10, g2, tv(A.cat2, 96), tv(A.a10, 32), none(), 1));
    FW(conv(11, g2, tv(A.a10, 32), tv(A.d2, 32), none(), 1));
    FW(upsample2_fwd(g1, tv(A.d2, 32), tv(A.cat1, 48, 0), 32, st));
    FW(conv(12, g1, tv(A.cat1, 48), tv(A.a12, 16), none(), 1));
    FW(conv(13, g1, tv(A.a12, 16), tv(A.d1, 16), none(), 1));
    FW(conv(14, g1, tv(A.d1, 16), none(), tv(A.out.p, 16), 0));
#undef FW
    return cudaSuccess;
}

// backward pass from A.gout (d loss / d out, BF16) into M->g (FP32, accumulated)
cudaError_t backward(am_precond *M, Acts &A, cudaStream_t st) {
    const Grid5 g1 = A.G(0), g2 = A.G(1), g3 = A.G(2), g4 = A.G(3);
    cudaError_t e;
#define BW(call) \
    if ((e = (call)) != cudaSuccess) return e
    // layer l: y = relu(conv(x)); dy holds d loss / d y (post-activation) unless last
    auto layer = [&](int l, const Grid5 &g, TensorView x, TensorView dy, TensorView y, TensorView dx,
                     bool relu) -> cudaError_t {
        cudaError_t e2;
        if (relu && (e2 = relu_bwd(g, dy, y, kSpec[l].cout, st)) != cudaSuccess) return e2;
        if ((e2 = conv3d_wgrad(g, x, kSpec[l].cin, dy, kSpec[l].cout, M->g.p + M->off[l], st)) != cudaSuccess)
            return e2;
        if (!dx.p) return cudaSuccess;
        return conv3d_fwd(g, dy, kSpec[l].cout, M->wt.p + M->off[l], kSpec[l].cin, dx, none(), 0, st);
    };
    BW(layer(14, g1, tv(A.d1, 16), tv(A.gout, 16), none(), tv(A.g_d1, 16), false));
    BW(layer(13, g1, tv(A.a12, 16), tv(A.g_d1, 16), tv(A.d1, 16), tv(A.g_a12, 16), true));
    BW(layer(12, g1, tv(A.cat1, 48), tv(A.g_a12, 16), tv(A.a12, 16), tv(A.g_cat1, 48), true));
    BW(upsample2_bwd(g1, tv(A.g_cat1, 48, 0), tv(A.g_d2, 32), 32, st));
    BW(layer(11, g2, tv(A.a10, 32), tv(A.g_d2, 32), tv(A.d2, 32), tv(A.g_a10, 32), true));
    BW(layer(10, g2, tv(A.cat2, 96), tv(A.g_a10, 32), tv(A.a10, 32), tv(A.g_cat2, 96), true));
    BW(upsample2_bwd(g2, tv(A.g_cat2, 96, 0), tv(A.g_d3, 64), 64, st));
    BW(layer(9, g3, tv(A.a8, 64), tv(A.g_d3, 64), tv(A.d3, 64), tv(A.g_a8, 64), true));
    BW(layer(8, g3, tv(A.cat3, 192), tv(A.g_a8, 64), tv(A.a8, 64), tv(A.g_cat3, 192), true));
    BW(upsample2_bwd(g3, tv(A.g_cat3, 192, 0), tv(A.g_e4, 128), 128, st));
    BW(layer(7, g4, tv(A.a6, 128), tv(A.g_e4, 128), tv(A.e4, 128), tv(A.g_a6, 128), true));
    BW(layer(6, g4, tv(A.p3, 64), tv(A.g_a6, 128), tv(A.a6, 128), tv(A.g_p3, 64), true));
    BW(avgpool2_bwd(g4, tv(A.g_p3, 64), tv(A.g_cat3, 192, 128), 64, 1, st));
    BW(layer(5, g3, tv(A.a4, 64), tv(A.g_cat3, 192, 128), tv(A.cat3, 192, 128), tv(A.g_a4, 64), true));
    BW(layer(4, g3, tv(A.p2, 32), tv(A.g_a4, 64), tv(A.a4, 64), tv(A.g_p2, 32), true));
    BW(avgpool2_bwd(g3, tv(A.g_p2, 32), tv(A.g_cat2, 96, 64), 32, 1, st));
    BW(layer(3, g2, tv(A.a2, 32), tv(A.g_cat2, 96, 64), tv(A.cat2, 96, 64), tv(A.g_a2, 32), true));
    BW(layer(2, g2, tv(A.p1, 16), tv(A.g_a2, 32), tv(A.a2, 32), tv(A.g_p1, 16), true));
    BW(avgpool2_bwd(g2, tv(A.g_p1, 16), tv(A.g_cat1, 48, 32), 16, 1, st));
    BW(layer(1, g1, tv(A.a0, 16), tv(A.g_cat1, 48, 32), tv(A.cat1, 48, 32), tv(A.g_a0, 16), true));
    BW(layer(0, g1, tv(A.x0, 16), tv(A.g_a0, 16), tv(A.a0, 16), none(), true));
#undef BW
    return cudaSuccess;
}

cudaError_t refresh_backward_weights(am_precond *M, cudaStream_t st) {
    for (int l = 0; l < kLayers; ++l) {
        cudaError_t e = conv3d_flip_transpose(M->wb.p + M->off[l], kSpec[l].cout, kSpec[l].cin, M->wt.p + M->off[l], st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void network_grid(const Layout &L, int &gz, int &gy, int &gx) {
    gz = round8(L.nz + 1);
    gy = round8(L.ny + 1);
    gx = round8(L.nx + 1);
}

}  // namespace

namespace amk {

am_status precond_apply(am_precond *M, const PrecondView &v, const double *r, double *z) {
    const Layout &L = v.L;
    int gz, gy, gx;
    network_grid(L, gz, gy, gx);
    PCK(ensure_acts(M->infer, 1, gz, gy, gx, false));
    PCK(M->dens_scratch_dsq.alloc((size_t)L.cs));
    PCK(M->dens_scratch_rhon.alloc((size_t)L.cs));
    PCK(M->acc.alloc(4));
    PCK(M->packsrc.alloc(1));
    float *dsq = M->dens_scratch_dsq.p, *rhon = M->dens_scratch_rhon.p;
    node_fields_kernel<<<eb(L.cs), 256, 0, v.st>>>(L, v.dinv32, v.rho, dsq, rhon);
    PCK(cudaGetLastError());
    PCK(cudaMemsetAsync(M->acc.p, 0, 4 * sizeof(double), v.st));
    scaled_norm_kernel<<<eb(L.cs), 256, 0, v.st>>>(L, r, dsq, v.mask, M->acc.p);
    count_free_kernel<<<eb(L.cs), 256, 0, v.st>>>(L, v.mask, M->acc.p + 1);
    PCK(cudaGetLastError());
    double h[2];
    PCK(cudaMemcpyAsync(h, M->acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, v.st));
    PCK(cudaStreamSynchronize(v.st));
    const double rms = std::sqrt(std::max(h[0], 1e-300) / std::max(h[1], 1.0));
    PackSrc ps{nullptr, r, dsq, rhon, v.mask, 1.0 / rms};
    PCK(cudaMemcpyAsync(M->packsrc.p, &ps, sizeof(PackSrc), cudaMemcpyHostToDevice, v.st));
    pack_input_kernel<<<eb((long long)gz * gy * gx), 256, 0, v.st>>>(L, gz, gy, gx, M->packsrc.p, M->infer.x0, 1);
    PCK(cudaGetLastError());
    PCK(forward(M, M->infer, v.st));
    apply_out_kernel<<<eb(L.cs), 256, 0, v.st>>>(L, gz, gy, gx, r, dsq, v.mask, M->infer.out.p, M->acc.p, h[1], z);
    PCK(cudaGetLastError());
    count_launches(21 + 5);
    return conv_status(v.st);
}

am_status precond_add_density(am_precond *M, const PrecondView &v, const Modal<float> &M32, const float *s32,
                              int *density_id) {
    const Layout &L = v.L;
    if (!M->has_grid) {
        M->has_grid = true;
        M->L = L;
        M->M32 = M32;
        M->plan = ku_plan(L, false, 0);
        network_grid(L, M->gz, M->gy, M->gx);
        PCK(M->r.alloc((size_t)M->capacity * 3 * (size_t)L.cs));
        PCK(M->e.alloc((size_t)M->capacity * 3 * (size_t)L.cs));
    } else if (L.nx != M->L.nx || L.ny != M->L.ny || L.nz != M->L.nz) {
        return pfail(AM_ERR_SIZE_MISMATCH, "training samples must all come from one grid size");
    }
    DensityDev d;
    PCK(cudaMalloc(&d.s32, sizeof(float) * (size_t)L.nel));
    PCK(cudaMalloc(&d.dsq, sizeof(float) * (size_t)L.cs));
    PCK(cudaMalloc(&d.rhon, sizeof(float) * (size_t)L.cs));
    PCK(cudaMalloc(&d.mask, (size_t)L.cs));
    PCK(cudaMemcpyAsync(d.s32, s32, sizeof(float) * (size_t)L.nel, cudaMemcpyDeviceToDevice, v.st));
    PCK(cudaMemcpyAsync(d.mask, v.mask, (size_t)L.cs, cudaMemcpyDeviceToDevice, v.st));
    PCK(cudaMemsetAsync(d.dsq, 0, sizeof(float) * (size_t)L.cs, v.st));
    PCK(cudaMemsetAsync(d.rhon, 0, sizeof(float) * (size_t)L.cs, v.st));
    node_fields_kernel<<<eb(L.cs), 256, 0, v.st>>>(L, v.dinv32, v.rho, d.dsq, d.rhon);
    PCK(cudaGetLastError());
    PCK(cudaStreamSynchronize(v.st));
    M->dens.push_back(d);
    *density_id = (int)M->dens.size() - 1;
    return AM_OK;
}

am_status precond_add_sample(am_precond *M, int density_id, const float *r32, const double *xk, const double *xstar,
                             cudaStream_t st) {
    if (density_id < 0 || density_id >= (int)M->dens.size()) return pfail(AM_ERR_INVALID_ARG, "bad density id");
    if (M->nsamples >= M->capacity) return pfail(AM_ERR_SIZE_MISMATCH, "training set full (capacity)");
    const Layout &L = M->L;
    const DensityDev &d = M->dens[density_id];
    PCK(M->acc.alloc(4));
    PCK(cudaMemsetAsync(M->acc.p, 0, 4 * sizeof(double), st));
    scaled_norm32_kernel<<<eb(L.cs), 256, 0, st>>>(L, r32, d.dsq, d.mask, M->acc.p, M->acc.p + 1);
    PCK(cudaGetLastError());
    double h[2];
    PCK(cudaMemcpyAsync(h, M->acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    if (!(h[0] > 0.0)) return AM_OK;  // a zero residual teaches nothing
    float *dst = M->r.p + (size_t)M->nsamples * 3 * (size_t)L.cs;
    scale_sample_kernel<<<eb(L.cs), 256, 0, st>>>(L, r32, d.dsq, d.mask, dst, M->acc.p, h[1]);
    PCK(cudaGetLastError());
    const bool has_err = xk && xstar;
    if (has_err) {
        float *edst = M->e.p + (size_t)M->nsamples * 3 * (size_t)L.cs;
        scale_error_kernel<<<eb(L.cs), 256, 0, st>>>(L, xstar, xk, d.dsq, d.mask, edst, M->acc.p, h[1]);
        PCK(cudaGetLastError());
    }
    M->sample_err.push_back(has_err ? 1 : 0);
    M->sample_dens.push_back(density_id);
    ++M->nsamples;
    return AM_OK;
}

}  // namespace amk

namespace {

// loss (and, if grad, d loss / d out into A.gout) of a batch of training samples
am_status batch_loss(am_precond *M, const std::vector<int> &ids, bool grad, int loss_kind, double *loss_sum) {
    const Layout &L = M->L;
    const int nb = (int)ids.size();
    Acts &A = M->train;
    cudaStream_t st = M->st;
    PCK(ensure_acts(A, nb, M->gz, M->gy, M->gx, grad));
    PCK(M->u.alloc(3 * (size_t)L.cs));
    PCK(M->y.alloc(3 * (size_t)L.cs));
    if (loss_kind == 1) {
        for (int id : ids)
            if (!M->sample_err[id]) return pfail(AM_ERR_INVALID_ARG, "energy-norm loss needs harvested errors");
    }
    PCK(M->acc.alloc((size_t)3 * nb + 2));
    PCK(M->packsrc.alloc((size_t)nb));
    std::vector<PackSrc> ps(nb);
    for (int b = 0; b < nb; ++b) {
        const DensityDev &d = M->dens[M->sample_dens[ids[b]]];
        ps[b] = PackSrc{M->r.p + (size_t)ids[b] * 3 * (size_t)L.cs, nullptr, d.dsq, d.rhon, d.mask, 1.0};
    }
    PCK(cudaMemcpyAsync(M->packsrc.p, ps.data(), nb * sizeof(PackSrc), cudaMemcpyHostToDevice, st));
    const long long V1 = (long long)nb * M->gz * M->gy * M->gx;
    pack_input_kernel<<<eb(V1), 256, 0, st>>>(L, M->gz, M->gy, M->gx, M->packsrc.p, A.x0, nb);
    PCK(cudaGetLastError());
    PCK(forward(M, A, st));
    PCK(cudaMemsetAsync(M->acc.p, 0, sizeof(double) * (3 * (size_t)nb + 2), st));
    if (grad) PCK(fill_zero_bf16(A.gout, V1 * 16, st));
    const long long vs = (long long)M->gz * M->gy * M->gx;
    for (int b = 0; b < nb; ++b) {
        const DensityDev &d = M->dens[M->sample_dens[ids[b]]];
        const float *r = M->r.p + (size_t)ids[b] * 3 * (size_t)L.cs;
        const float *out = A.out.p + (size_t)b * vs * 16;
        double *acc = M->acc.p + 2 * b;
        if (loss_kind == 1) {
            // 1 - (z~.r~)^2 / ((z~.K~z~)(e~.r~)): the share of the error's energy that
            // the best multiple of z~ misses (flexible CG is blind to the scale of z)
            const float *et = M->e.p + (size_t)ids[b] * 3 * (size_t)L.cs;
            make_u_kernel<<<eb(L.cs), 256, 0, st>>>(L, M->gz, M->gy, M->gx, r, d.dsq, d.mask, out, M->u.p);
            PCK(cudaGetLastError());
            PCK(ku_plain<float>(M->plan, L, M->M32, d.s32, M->u.p, M->y.p, st));
            energy_sums_kernel<<<eb(L.cs), 256, 0, st>>>(L, M->gz, M->gy, M->gx, r, et, d.dsq, d.mask, out, M->y.p,
                                                         M->acc.p + 3 * b);
            PCK(cudaGetLastError());
            if (grad) {
                energy_grad_kernel<<<eb(L.cs), 256, 0, st>>>(L, M->gz, M->gy, M->gx, r, d.dsq, d.mask, M->y.p,
                                                             M->acc.p + 3 * b, 1.0 / nb,
                                                             A.gout + (size_t)b * vs * 16);
                PCK(cudaGetLastError());
            }
            continue;
        }
        make_u_kernel<<<eb(L.cs), 256, 0, st>>>(L, M->gz, M->gy, M->gx, r, d.dsq, d.mask, out, M->u.p);
        PCK(cudaGetLastError());
        PCK(ku_plain<float>(M->plan, L, M->M32, d.s32, M->u.p, M->y.p, st));
        resid_kernel<<<eb(L.cs), 256, 0, st>>>(L, r, d.dsq, d.mask, M->y.p, M->u.p, acc);
        PCK(cudaGetLastError());
        if (grad) {
            PCK(ku_plain<float>(M->plan, L, M->M32, d.s32, M->u.p, M->y.p, st));
            grad_out_kernel<<<eb(L.cs), 256, 0, st>>>(L, M->gz, M->gy, M->gx, d.dsq, d.mask, M->y.p, acc,
                                                      1.0 / nb, A.gout + (size_t)b * vs * 16);
            PCK(cudaGetLastError());
        }
    }
    std::vector<double> h((size_t)3 * nb);
    PCK(cudaMemcpyAsync(h.data(), M->acc.p, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
        if (loss_kind == 1)
            s += 1.0 - h[3 * b] * h[3 * b] / (std::max(h[3 * b + 1], 1e-300) * std::max(h[3 * b + 2], 1e-300));
        else
            s += h[2 * b] / std::max(h[2 * b + 1], 1e-300);
    }
    *loss_sum = s;
    return AM_OK;
}

am_status check_pre(am_precond *M) {
    if (!M) return pfail(AM_ERR_INVALID_ARG, "null preconditioner");
    PCK(cudaSetDevice(M->device));
    return AM_OK;
}

}  // namespace

extern "C" {

am_status am_precond_create(uint64_t seed, long long capacity, am_precond **out) {
    if (!out) return pfail(AM_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (capacity < 0) return pfail(AM_ERR_INVALID_ARG, "capacity must be >= 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return pfail(AM_ERR_NO_DEVICE, "no CUDA device");
    am_precond *M = new am_precond();
    cudaGetDevice(&M->device);
    M->capacity = capacity;
    size_t o = 0;
    for (int l = 0; l < kLayers; ++l) {
        M->off[l] = o;
        o += 27ull * kSpec[l].cin * kSpec[l].cout;
    }
    M->off[kLayers] = o;
    cudaError_t e = cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = M->w.alloc(o);
    if (e == cudaSuccess) e = M->m.alloc(o);
    if (e == cudaSuccess) e = M->v.alloc(o);
    if (e == cudaSuccess) e = M->g.alloc(o);
    if (e == cudaSuccess) e = M->wb.alloc(o);
    if (e == cudaSuccess) e = M->wt.alloc(o);
    if (e != cudaSuccess) {
        am_precond_destroy(M);
        return pfail(e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                     std::string("preconditioner create: ") + cudaGetErrorString(e));
    }
    // He-uniform initialisation over the used input channels; the output layer
    // starts at zero (the untrained preconditioner is Jacobi)
    std::vector<float> w(o, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kLayers - 1; ++l) {
        const LayerSpec &s = kSpec[l];
        const float bound = std::sqrt(6.0f / (27.0f * s.cin_used));
        std::uniform_real_distribution<float> U(-bound, bound);
        for (int t = 0; t < 27; ++t)
            for (int co = 0; co < s.cout; ++co)
                for (int ci = 0; ci < s.cin; ++ci)
                    if (ci < s.cin_used && co < s.cout_used)
                        w[M->off[l] + ((size_t)t * s.cout + co) * s.cin + ci] = U(rng);
    }
    e = cudaMemcpy(M->w.p, w.data(), o * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = f32_to_bf16(M->w.p, M->wb.p, (long long)o, M->st);
    if (e == cudaSuccess) e = refresh_backward_weights(M, M->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e != cudaSuccess) {
        am_precond_destroy(M);
        return pfail(AM_ERR_CUDA, std::string("preconditioner init: ") + cudaGetErrorString(e));
    }
    *out = M;
    return AM_OK;
}

am_status am_precond_destroy(am_precond *M) {
    if (!M) return AM_OK;
    cudaSetDevice(M->device);
    if (M->st) cudaStreamSynchronize(M->st);
    for (auto &d : M->dens) {
        cudaFree(d.s32);
        cudaFree(d.dsq);
        cudaFree(d.rhon);
        cudaFree(d.mask);
    }
    for (auto *b : {&M->w, &M->m, &M->v, &M->g, &M->r, &M->e, &M->u, &M->y, &M->hin, &M->hout,
                    &M->dens_scratch_dsq,
                    &M->dens_scratch_rhon})
        b->release();
    M->wb.release();
    M->wt.release();
    M->acc.release();
    M->packsrc.release();
    for (Acts *A : {&M->train, &M->infer}) {
        A->pool.release();
        A->out.release();
    }
    if (M->st) cudaStreamDestroy(M->st);
    delete M;
    return AM_OK;
}

long long am_precond_num_params(am_precond *M) { return M ? (long long)M->off[kLayers] : 0; }

long long am_precond_num_samples(am_precond *M) { return M ? M->nsamples : 0; }

am_status am_precond_get_params(am_precond *M, float *w) {
    PCKS(check_pre(M));
    if (!w) return pfail(AM_ERR_INVALID_ARG, "null output");
    PCK(cudaMemcpy(w, M->w.p, M->off[kLayers] * sizeof(float), cudaMemcpyDeviceToHost));
    return AM_OK;
}

am_status am_precond_set_params(am_precond *M, const float *w) {
    PCKS(check_pre(M));
    if (!w) return pfail(AM_ERR_INVALID_ARG, "null input");
    const size_t o = M->off[kLayers];
    PCK(cudaMemcpy(M->w.p, w, o * sizeof(float), cudaMemcpyHostToDevice));
    PCK(f32_to_bf16(M->w.p, M->wb.p, (long long)o, M->st));
    PCK(refresh_backward_weights(M, M->st));
    PCK(cudaMemsetAsync(M->m.p, 0, o * sizeof(float), M->st));
    PCK(cudaMemsetAsync(M->v.p, 0, o * sizeof(float), M->st));
    M->adam_t = 0;
    PCK(cudaStreamSynchronize(M->st));
    return AM_OK;
}

am_status am_precond_forward(am_precond *M, int n, int gz, int gy, int gx, const float *in, float *out) {
    PCKS(check_pre(M));
    if (n < 1 || gz < 8 || gy < 8 || gx < 8 || gz % 8 || gy % 8 || gx % 8)
        return pfail(AM_ERR_INVALID_ARG, "grid dimensions must be positive multiples of 8");
    if (!in || !out) return pfail(AM_ERR_INVALID_ARG, "null tensor");
    const long long V = (long long)n * gz * gy * gx;
    PCK(ensure_acts(M->infer, n, gz, gy, gx, false));
    PCK(M->hin.alloc((size_t)V * 4));
    PCK(M->hout.alloc((size_t)V * 3));
    PCK(cudaMemcpyAsync(M->hin.p, in, V * 4 * sizeof(float), cudaMemcpyHostToDevice, M->st));
    host_in_kernel<<<eb(V), 256, 0, M->st>>>(V, M->hin.p, 4, M->infer.x0);
    PCK(cudaGetLastError());
    PCK(forward(M, M->infer, M->st));
    host_out_kernel<<<eb(V), 256, 0, M->st>>>(V, M->infer.out.p, 3, M->hout.p);
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(out, M->hout.p, V * 3 * sizeof(float), cudaMemcpyDeviceToHost, M->st));
    PCK(cudaStreamSynchronize(M->st));
    return conv_status(M->st);
}

am_status am_precond_param_grad(am_precond *M, int n, int gz, int gy, int gx, const float *in, const float *dout,
                                float *grad) {
    PCKS(check_pre(M));
    if (n < 1 || gz < 8 || gy < 8 || gx < 8 || gz % 8 || gy % 8 || gx % 8)
        return pfail(AM_ERR_INVALID_ARG, "grid dimensions must be positive multiples of 8");
    if (!in || !dout || !grad) return pfail(AM_ERR_INVALID_ARG, "null tensor");
    const long long V = (long long)n * gz * gy * gx;
    Acts &A = M->train;
    PCK(ensure_acts(A, n, gz, gy, gx, true));
    PCK(M->hin.alloc((size_t)V * 4));
    PCK(M->hout.alloc((size_t)V * 3));
    PCK(cudaMemcpyAsync(M->hin.p, in, V * 4 * sizeof(float), cudaMemcpyHostToDevice, M->st));
    host_in_kernel<<<eb(V), 256, 0, M->st>>>(V, M->hin.p, 4, A.x0);
    PCK(cudaGetLastError());
    PCK(forward(M, A, M->st));
    PCK(cudaMemcpyAsync(M->hout.p, dout, V * 3 * sizeof(float), cudaMemcpyHostToDevice, M->st));
    host_gout_kernel<<<eb(V), 256, 0, M->st>>>(V, M->hout.p, 3, A.gout);
    PCK(cudaGetLastError());
    PCK(cudaMemsetAsync(M->g.p, 0, M->off[kLayers] * sizeof(float), M->st));
    PCK(backward(M, A, M->st));
    PCK(cudaMemcpyAsync(grad, M->g.p, M->off[kLayers] * sizeof(float), cudaMemcpyDeviceToHost, M->st));
    PCK(cudaStreamSynchronize(M->st));
    return conv_status(M->st);
}

am_status am_precond_bench_forward(am_precond *M, int n, int gz, int gy, int gx, int reps, double *avg_ms,
                                   double *flops) {
    PCKS(check_pre(M));
    if (n < 1 || gz < 8 || gy < 8 || gx < 8 || gz % 8 || gy % 8 || gx % 8 || reps < 1)
        return pfail(AM_ERR_INVALID_ARG, "need positive multiples of 8 and reps >= 1");
    Acts &A = M->infer;
    PCK(ensure_acts(A, n, gz, gy, gx, false));
    const long long V = (long long)n * gz * gy * gx;
    PCK(fill_zero_bf16(A.x0, V * 16, M->st));
    PCK(forward(M, A, M->st));  // warm-up
    cudaEvent_t e0, e1;
    PCK(cudaEventCreate(&e0));
    PCK(cudaEventCreate(&e1));
    PCK(cudaEventRecord(e0, M->st));
    for (int r = 0; r < reps; ++r) PCK(forward(M, A, M->st));
    PCK(cudaEventRecord(e1, M->st));
    PCK(cudaEventSynchronize(e1));
    float ms = 0.f;
    PCK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    PCKS(conv_status(M->st));
    if (avg_ms) *avg_ms = ms / reps;
    if (flops) {
        // 2 * 27 * cin * cout per voxel of each layer's grid (channels as computed)
        double f = 0.0;
        const int level[kLayers] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
        for (int l = 0; l < kLayers; ++l)
            f += 2.0 * 27.0 * kSpec[l].cin * kSpec[l].cout * (double)(V >> (3 * level[l]));
        *flops = f;
    }
    count_launches(21LL * (reps + 1));
    return AM_OK;
}

am_status am_precond_train(am_precond *M, const am_train_config *cfg, float *epoch_loss) {
    PCKS(check_pre(M));
    if (!cfg) return pfail(AM_ERR_INVALID_ARG, "null training config");
    if (M->nsamples < 1) return pfail(AM_ERR_INVALID_ARG, "no training samples");
    if (cfg->epochs < 0 || cfg->batch < 1) return pfail(AM_ERR_INVALID_ARG, "need epochs >= 0, batch >= 1");
    const int nb = (int)std::min<long long>(cfg->batch, M->nsamples);
    std::mt19937_64 rng(cfg->seed);
    std::vector<int> order((size_t)M->nsamples);
    const size_t np = M->off[kLayers];
    for (int ep = 0; ep < cfg->epochs; ++ep) {
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::shuffle(order.begin(), order.end(), rng);
        double tot = 0.0;
        long long cnt = 0;
        for (size_t s = 0; s + nb <= order.size(); s += nb) {
            std::vector<int> ids(order.begin() + s, order.begin() + s + nb);
            PCK(cudaMemsetAsync(M->g.p, 0, np * sizeof(float), M->st));
            double l = 0.0;
            PCKS(batch_loss(M, ids, true, cfg->loss, &l));
            PCK(backward(M, M->train, M->st));
            ++M->adam_t;
            PCK(adam_step(M->w.p, M->m.p, M->v.p, M->g.p, M->wb.p, (long long)np, cfg->lr, cfg->beta1, cfg->beta2,
                          cfg->eps, M->adam_t, 1.0f, M->st));
            PCK(refresh_backward_weights(M, M->st));
            tot += l;
            cnt += nb;
        }
        PCKS(conv_status(M->st));
        if (epoch_loss) epoch_loss[ep] = cnt ? (float)(tot / cnt) : 0.f;
        if (cfg->verbose) std::printf("epoch %d: loss %.4e (%lld samples)\n", ep, cnt ? tot / cnt : 0.0, cnt);
    }
    PCK(cudaStreamSynchronize(M->st));
    return AM_OK;
}

am_status am_precond_eval(am_precond *M, long long first, long long count, int loss_kind, double *mean_loss) {
    PCKS(check_pre(M));
    if (!mean_loss) return pfail(AM_ERR_INVALID_ARG, "null output");
    if (first < 0 || count < 1 || first + count > M->nsamples) return pfail(AM_ERR_INVALID_ARG, "sample range");
    double tot = 0.0;
    const int chunk = 8;
    for (long long s = first; s < first + count; s += chunk) {
        std::vector<int> ids;
        for (long long i = s; i < std::min(first + count, s + chunk); ++i) ids.push_back((int)i);
        double l = 0.0;
        PCKS(batch_loss(M, ids, false, loss_kind, &l));
        tot += l;
    }
    *mean_loss = tot / count;
    return conv_status(M->st);
}

}  // extern "C"

extern "C" am_status am_precond_set_kernels(int impl) {
    if (impl != 0 && impl != 1) return pfail(AM_ERR_INVALID_ARG, "impl must be 0 (mma.sync) or 1 (tcgen05)");
    conv3d_set_impl(impl);
    return AM_OK;
}
