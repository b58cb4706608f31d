// unet.cu -- the density-predicting 3-D U-Net of the reference's am.ai module
// (TopOptUNet, src/am/ai/model.py:18-67: in_channels 4, out_channels 1,
// features (32, 64, 128, 256); a placeholder there), built on this engine's
// tensor-core convolutions (conv3d_tc.cu).
//
// Four levels of width f0, 2 f0, 4 f0, 8 f0 (two 3x3x3 convolutions + ReLU each),
// 2x2x2 mean pooling down, nearest upsampling up, skip connections by
// concatenation, a 3x3x3 output convolution and a sigmoid: the predicted density.
// Tensors are channels-last BF16 on the element grid padded to multiples of 8;
// input and output channel counts are padded to 16.  Training minimises the binary
// cross-entropy of the sigmoid output against target densities over the cells
// inside each sample's domain, with Adam on FP32 master weights, and reports the
// mean squared error.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "conv3d.cuh"
#include "kernels.cuh"

using namespace amk;

namespace {

typedef __nv_bfloat16 bf16;

am_status ufail(am_status s, const std::string &m) {
    set_last_error(m.c_str());
    return s;
}
#define UCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            return ufail(e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,                        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                               \
    } while (0)
#define UCKS(expr)                  \
    do {                            \
        am_status s_ = (expr);      \
        if (s_ != AM_OK) return s_; \
    } while (0)

constexpr int kL = 15;  // convolutions

template <typename T>
struct DBuf {
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

// activations (and gradients) of one batch shape
struct UActs {
    int n = 0, gz = 0, gy = 0, gx = 0;
    bool grads = false;
    DBuf<bf16> pool;
    DBuf<float> out;
    // forward: x0 in; a0 e1->cat1; p1 a2 e2->cat2; p2 a4 e3->cat3; p3 a6 e4; a8 d3; a10 d2; a12 d1
    bf16 *x0, *a0, *cat1, *p1, *a2, *cat2, *p2, *a4, *cat3, *p3, *a6, *e4, *a8, *d3, *a10, *d2, *a12, *d1;
    bf16 *gout, *g_d1, *g_a12, *g_cat1, *g_d2, *g_a10, *g_cat2, *g_d3, *g_a8, *g_cat3, *g_e4, *g_a6, *g_p3, *g_a4,
        *g_p2, *g_a2, *g_p1, *g_a0;
    Grid5 G(int level) const { return Grid5{n, gz >> level, gy >> level, gx >> level}; }
};

__global__ void pack_kernel(long long V, const float *__restrict__ in, int cin, bf16 *__restrict__ x0) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < 16; ++k) x0[v * 16 + k] = __float2bfloat16(k < cin ? in[v * cin + k] : 0.f);
}
__global__ void unpack_kernel(long long V, const float *__restrict__ out16, int cout, int sigm, float *__restrict__ out) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < cout; ++k) {
            const float o = out16[v * 16 + k];
            out[v * cout + k] = sigm ? 1.f / (1.f + expf(-o)) : o;
        }
}
__global__ void gout_kernel(long long V, const float *__restrict__ dout, int cout, bf16 *__restrict__ g) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < 16; ++k) g[v * 16 + k] = __float2bfloat16(k < cout ? dout[v * cout + k] : 0.f);
}
// masked squared error of y = sigmoid(out[:, 0]) against t into acc[0..1] (sum of
// squares, count); into g (BF16, other channels zero) the gradient of the binary
// cross-entropy -t log y - (1-t) log(1-y) with respect to the logit, y - t, scaled
// by `scale` -- unlike the squared error's (y - t) y (1 - y) it does not vanish
// where the sigmoid saturates, so a network pushed to all-void or all-solid
// outputs early in training still recovers
__global__ void mse_kernel(long long V, const float *__restrict__ out16, const float *__restrict__ t,
                           const uint8_t *__restrict__ m, double scale, bf16 *__restrict__ g, double *acc) {
    __shared__ double red[2 * 8];
    double se = 0.0, cnt = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
         v += (long long)gridDim.x * blockDim.x) {
        float gr = 0.f;
        if (m[v]) {
            const float y = 1.f / (1.f + expf(-out16[v * 16]));
            const float d = y - t[v];
            se += (double)d * d;
            cnt += 1.0;
            gr = (float)scale * d;
        }
        if (g) {
            g[v * 16] = __float2bfloat16(gr);
            for (int k = 1; k < 16; ++k) g[v * 16 + k] = __float2bfloat16(0.f);
        }
    }
    double w[2] = {se, cnt};
    block_sum<2>(w, red);
    if (threadIdx.x == 0) {
        atomicAdd(acc, w[0]);
        atomicAdd(acc + 1, w[1]);
    }
}

int ub(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

}  // namespace

struct am_unet {
    int device = 0;
    cudaStream_t st = nullptr;
    int cin = 4, cout = 1, f0 = 32;
    int spec[kL][2] = {};  // (cin, cout) per convolution, padded
    size_t off[kL + 1] = {};
    DBuf<float> w, m, v, g;
    DBuf<bf16> wb, wt;
    int adam_t = 0;
    UActs train, infer;
    // training set: all samples share one padded grid
    int S = 0, gz = 0, gy = 0, gx = 0;
    DBuf<bf16> xs;     // [S][V][16]
    DBuf<float> ts;    // [S][V]
    DBuf<uint8_t> ms;  // [S][V]
    DBuf<float> tbat;
    DBuf<uint8_t> mbat;
    DBuf<double> acc;
    DBuf<float> hin, hout;
};

namespace {

cudaError_t ensure_uacts(am_unet *U, UActs &A, int n, int gz, int gy, int gx, bool grads) {
    if (A.pool.p && A.n == n && A.gz == gz && A.gy == gy && A.gx == gx && (A.grads || !grads)) return cudaSuccess;
    A.n = n;
    A.gz = gz;
    A.gy = gy;
    A.gx = gx;
    A.grads = grads;
    const int f0 = U->f0, f1 = 2 * f0, f2 = 4 * f0, f3 = 8 * f0;
    const size_t V1 = (size_t)n * gz * gy * gx, V2 = V1 / 8, V3 = V1 / 64, V4 = V1 / 512;
    struct Req {
        bf16 **p;
        size_t count;
    };
    std::vector<Req> req = {{&A.x0, V1 * 16},      {&A.a0, V1 * f0},      {&A.cat1, V1 * 3 * f0}, {&A.p1, V2 * f0},
                            {&A.a2, V2 * f1},      {&A.cat2, V2 * 3 * f1}, {&A.p2, V3 * f1},      {&A.a4, V3 * f2},
                            {&A.cat3, V3 * 3 * f2}, {&A.p3, V4 * f2},      {&A.a6, V4 * f3},      {&A.e4, V4 * f3},
                            {&A.a8, V3 * f2},      {&A.d3, V3 * f2},      {&A.a10, V2 * f1},     {&A.d2, V2 * f1},
                            {&A.a12, V1 * f0},     {&A.d1, V1 * f0}};
    if (grads) {
        std::vector<Req> gq = {{&A.gout, V1 * 16},       {&A.g_d1, V1 * f0},       {&A.g_a12, V1 * f0},
                               {&A.g_cat1, V1 * 3 * f0}, {&A.g_d2, V2 * f1},       {&A.g_a10, V2 * f1},
                               {&A.g_cat2, V2 * 3 * f1}, {&A.g_d3, V3 * f2},       {&A.g_a8, V3 * f2},
                               {&A.g_cat3, V3 * 3 * f2}, {&A.g_e4, V4 * f3},       {&A.g_a6, V4 * f3},
                               {&A.g_p3, V4 * f2},       {&A.g_a4, V3 * f2},       {&A.g_p2, V3 * f1},
                               {&A.g_a2, V2 * f1},       {&A.g_p1, V2 * f0},       {&A.g_a0, V1 * f0}};
        req.insert(req.end(), gq.begin(), gq.end());
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
    A.out.release();
    return A.out.alloc(V1 * 16);
}

TensorView tvw(void *p, int cs, int co = 0) { return TensorView{p, cs, co}; }
TensorView nonev() { return TensorView{nullptr, 0, 0}; }

cudaError_t unet_forward(am_unet *U, UActs &A, cudaStream_t st) {
    const Grid5 g1 = A.G(0), g2 = A.G(1), g3 = A.G(2), g4 = A.G(3);
    const int f0 = U->f0, f1 = 2 * f0, f2 = 4 * f0, f3 = 8 * f0;
    auto conv = [&](int l, const Grid5 &g, TensorView x, TensorView y, TensorView yf, int relu) {
        return conv3d_fwd(g, x, U->spec[l][0], U->wb.p + U->off[l], U->spec[l][1], y, yf, relu, st);
    };
    cudaError_t e;
#define UF(call) \
    if ((e = (call)) != cudaSuccess) return e
    UF(conv(0, g1, tvw(A.x0, 16), tvw(A.a0, f0), nonev(), 1));
    UF(conv(1, g1, tvw(A.a0, f0), tvw(A.cat1, 3 * f0, f1), nonev(), 1));
    UF(avgpool2_fwd(g2, tvw(A.cat1, 3 * f0, f1), tvw(A.p1, f0), f0, st));
    UF(conv(2, g2, tvw(A.p1, f0), tvw(A.a2, f1), nonev(), 1));
    UF(conv(3, g2, tvw(A.a2, f1), tvw(A.cat2, 3 * f1, f2), nonev(), 1));
    UF(avgpool2_fwd(g3, tvw(A.cat2, 3 * f1, f2), tvw(A.p2, f1), f1, st));
    UF(conv(4, g3, tvw(A.p2, f1), tvw(A.a4, f2), nonev(), 1));
    UF(conv(5, g3, tvw(A.a4, f2), tvw(A.cat3, 3 * f2, f3), nonev(), 1));
    UF(avgpool2_fwd(g4, tvw(A.cat3, 3 * f2, f3), tvw(A.p3, f2), f2, st));
    UF(conv(6, g4, tvw(A.p3, f2), tvw(A.a6, f3), nonev(), 1));
    UF(conv(7, g4, tvw(A.a6, f3), tvw(A.e4, f3), nonev(), 1));
    UF(upsample2_fwd(g3, tvw(A.e4, f3), tvw(A.cat3, 3 * f2, 0), f3, st));
    UF(conv(8, g3, tvw(A.cat3, 3 * f2), tvw(A.a8, f2), nonev(), 1));
    UF(conv(9, g3, tvw(A.a8, f2), tvw(A.d3, f2), nonev(), 1));
    UF(upsample2_fwd(g2, tvw(A.d3, f2), tvw(A.cat2, 3 * f1, 0), f2, st));
    UF(conv(10, g2, tvw(A.cat2, 3 * f1), tvw(A.a10, f1), nonev(), 1));
    UF(conv(11, g2, tvw(A.a10, f1), tvw(A.d2, f1), nonev(), 1));
    UF(upsample2_fwd(g1, tvw(A.d2, f1), tvw(A.cat1, 3 * f0, 0), f1, st));
    UF(conv(12, g1, tvw(A.cat1, 3 * f0), tvw(A.a12, f0), nonev(), 1));
    UF(conv(13, g1, tvw(A.a12, f0), tvw(A.d1, f0), nonev(), 1));
    UF(conv(14, g1, tvw(A.d1, f0), nonev(), tvw(A.out.p, 16), 0));
#undef UF
    count_launches(21);
    return cudaSuccess;
}

cudaError_t unet_backward(am_unet *U, UActs &A, cudaStream_t st) {
    const Grid5 g1 = A.G(0), g2 = A.G(1), g3 = A.G(2), g4 = A.G(3);
    const int f0 = U->f0, f1 = 2 * f0, f2 = 4 * f0, f3 = 8 * f0;
    cudaError_t e;
#define UB(call) \
    if ((e = (call)) != cudaSuccess) return e
    auto layer = [&](int l, const Grid5 &g, TensorView x, TensorView dy, TensorView y, TensorView dx,
                     bool relu) -> cudaError_t {
        cudaError_t e2;
        const int ci = U->spec[l][0], co = U->spec[l][1];
        if (relu && (e2 = relu_bwd(g, dy, y, co, st)) != cudaSuccess) return e2;
        if ((e2 = conv3d_wgrad(g, x, ci, dy, co, U->g.p + U->off[l], st)) != cudaSuccess) return e2;
        if (!dx.p) return cudaSuccess;
        return conv3d_fwd(g, dy, co, U->wt.p + U->off[l], ci, dx, nonev(), 0, st);
    };
    UB(layer(14, g1, tvw(A.d1, f0), tvw(A.gout, 16), nonev(), tvw(A.g_d1, f0), false));
    UB(layer(13, g1, tvw(A.a12, f0), tvw(A.g_d1, f0), tvw(A.d1, f0), tvw(A.g_a12, f0), true));
    UB(layer(12, g1, tvw(A.cat1, 3 * f0), tvw(A.g_a12, f0), tvw(A.a12, f0), tvw(A.g_cat1, 3 * f0), true));
    UB(upsample2_bwd(g1, tvw(A.g_cat1, 3 * f0, 0), tvw(A.g_d2, f1), f1, st));
    UB(layer(11, g2, tvw(A.a10, f1), tvw(A.g_d2, f1), tvw(A.d2, f1), tvw(A.g_a10, f1), true));
    UB(layer(10, g2, tvw(A.cat2, 3 * f1), tvw(A.g_a10, f1), tvw(A.a10, f1), tvw(A.g_cat2, 3 * f1), true));
    UB(upsample2_bwd(g2, tvw(A.g_cat2, 3 * f1, 0), tvw(A.g_d3, f2), f2, st));
    UB(layer(9, g3, tvw(A.a8, f2), tvw(A.g_d3, f2), tvw(A.d3, f2), tvw(A.g_a8, f2), true));
    UB(layer(8, g3, tvw(A.cat3, 3 * f2), tvw(A.g_a8, f2), tvw(A.a8, f2), tvw(A.g_cat3, 3 * f2), true));
    UB(upsample2_bwd(g3, tvw(A.g_cat3, 3 * f2, 0), tvw(A.g_e4, f3), f3, st));
    UB(layer(7, g4, tvw(A.a6, f3), tvw(A.g_e4, f3), tvw(A.e4, f3), tvw(A.g_a6, f3), true));
    UB(layer(6, g4, tvw(A.p3, f2), tvw(A.g_a6, f3), tvw(A.a6, f3), tvw(A.g_p3, f2), true));
    UB(avgpool2_bwd(g4, tvw(A.g_p3, f2), tvw(A.g_cat3, 3 * f2, f3), f2, 1, st));
    UB(layer(5, g3, tvw(A.a4, f2), tvw(A.g_cat3, 3 * f2, f3), tvw(A.cat3, 3 * f2, f3), tvw(A.g_a4, f2), true));
    UB(layer(4, g3, tvw(A.p2, f1), tvw(A.g_a4, f2), tvw(A.a4, f2), tvw(A.g_p2, f1), true));
    UB(avgpool2_bwd(g3, tvw(A.g_p2, f1), tvw(A.g_cat2, 3 * f1, f2), f1, 1, st));
    UB(layer(3, g2, tvw(A.a2, f1), tvw(A.g_cat2, 3 * f1, f2), tvw(A.cat2, 3 * f1, f2), tvw(A.g_a2, f1), true));
    UB(layer(2, g2, tvw(A.p1, f0), tvw(A.g_a2, f1), tvw(A.a2, f1), tvw(A.g_p1, f0), true));
    UB(avgpool2_bwd(g2, tvw(A.g_p1, f0), tvw(A.g_cat1, 3 * f0, f1), f0, 1, st));
    UB(layer(1, g1, tvw(A.a0, f0), tvw(A.g_cat1, 3 * f0, f1), tvw(A.cat1, 3 * f0, f1), tvw(A.g_a0, f0), true));
    UB(layer(0, g1, tvw(A.x0, 16), tvw(A.g_a0, f0), tvw(A.a0, f0), nonev(), true));
#undef UB
    return cudaSuccess;
}

cudaError_t refresh_wt(am_unet *U, cudaStream_t st) {
    for (int l = 0; l < kL; ++l) {
        cudaError_t e = conv3d_flip_transpose(U->wb.p + U->off[l], U->spec[l][1], U->spec[l][0], U->wt.p + U->off[l], st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

am_status ucheck(am_unet *U) {
    if (!U) return ufail(AM_ERR_INVALID_ARG, "null network");
    UCK(cudaSetDevice(U->device));
    return AM_OK;
}

am_status conv_ok(cudaStream_t st) {
    int f = 0;
    UCK(conv3d_tc_error(&f, true, st));
    if (f) return ufail(AM_ERR_TIMEOUT, "a bounded copy / MMA wait of a tensor-core convolution ran out");
    return AM_OK;
}

bool grid_ok(int n, int gz, int gy, int gx) {
    return n >= 1 && gz >= 8 && gy >= 8 && gx >= 8 && gz % 8 == 0 && gy % 8 == 0 && gx % 8 == 0;
}

}  // namespace

extern "C" {

am_status am_unet_create(int in_channels, int out_channels, int f0, uint64_t seed, am_unet **out) {
    if (!out) return ufail(AM_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (in_channels < 1 || in_channels > 16 || out_channels < 1 || out_channels > 16 || (f0 != 16 && f0 != 32))
        return ufail(AM_ERR_INVALID_ARG, "need 1 <= in, out <= 16 and base width 16 or 32");
    if (!am_is_available()) return ufail(AM_ERR_NO_DEVICE, "no CUDA device");
    am_unet *U = new am_unet();
    cudaGetDevice(&U->device);
    U->cin = in_channels;
    U->cout = out_channels;
    U->f0 = f0;
    const int f1 = 2 * f0, f2 = 4 * f0, f3 = 8 * f0;
    const int sp[kL][2] = {{16, f0},     {f0, f0}, {f0, f1}, {f1, f1},     {f1, f2}, {f2, f2},
                           {f2, f3},     {f3, f3}, {3 * f2, f2}, {f2, f2}, {3 * f1, f1}, {f1, f1},
                           {3 * f0, f0}, {f0, f0}, {f0, 16}};
    size_t o = 0;
    for (int l = 0; l < kL; ++l) {
        U->spec[l][0] = sp[l][0];
        U->spec[l][1] = sp[l][1];
        U->off[l] = o;
        o += 27ull * sp[l][0] * sp[l][1];
    }
    U->off[kL] = o;
    cudaError_t e = cudaStreamCreateWithFlags(&U->st, cudaStreamNonBlocking);
    for (auto *b : {&U->w, &U->m, &U->v, &U->g})
        if (e == cudaSuccess) e = b->alloc(o);
    if (e == cudaSuccess) e = U->wb.alloc(o);
    if (e == cudaSuccess) e = U->wt.alloc(o);
    if (e == cudaSuccess) e = U->acc.alloc(4);
    if (e != cudaSuccess) {
        am_unet_destroy(U);
        return ufail(e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                     std::string("network create: ") + cudaGetErrorString(e));
    }
    // He-uniform over the channels in use; the output layer small so the first
    // prediction sits near density 0.5
    std::vector<float> w(o, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kL; ++l) {
        const int ci = sp[l][0], co = sp[l][1];
        const int ci_used = l == 0 ? in_channels : ci, co_used = l == kL - 1 ? out_channels : co;
        const float bound = std::sqrt(6.0f / (27.0f * ci_used)) * (l == kL - 1 ? 0.1f : 1.0f);
        std::uniform_real_distribution<float> Ud(-bound, bound);
        for (int t = 0; t < 27; ++t)
            for (int c = 0; c < co; ++c)
                for (int k = 0; k < ci; ++k)
                    if (k < ci_used && c < co_used) w[U->off[l] + ((size_t)t * co + c) * ci + k] = Ud(rng);
    }
    e = cudaMemcpy(U->w.p, w.data(), o * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = f32_to_bf16(U->w.p, U->wb.p, (long long)o, U->st);
    if (e == cudaSuccess) e = refresh_wt(U, U->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(U->st);
    if (e != cudaSuccess) {
        am_unet_destroy(U);
        return ufail(AM_ERR_CUDA, std::string("network init: ") + cudaGetErrorString(e));
    }
    *out = U;
    return AM_OK;
}

am_status am_unet_destroy(am_unet *U) {
    if (!U) return AM_OK;
    cudaSetDevice(U->device);
    if (U->st) cudaStreamSynchronize(U->st);
    for (auto *b : {&U->w, &U->m, &U->v, &U->g, &U->ts, &U->tbat, &U->hin, &U->hout}) b->release();
    U->wb.release();
    U->wt.release();
    U->xs.release();
    U->ms.release();
    U->mbat.release();
    U->acc.release();
    for (UActs *A : {&U->train, &U->infer}) {
        A->pool.release();
        A->out.release();
    }
    if (U->st) cudaStreamDestroy(U->st);
    delete U;
    return AM_OK;
}

long long am_unet_num_params(am_unet *U) { return U ? (long long)U->off[kL] : 0; }

am_status am_unet_get_params(am_unet *U, float *w) {
    UCKS(ucheck(U));
    if (!w) return ufail(AM_ERR_INVALID_ARG, "null output");
    UCK(cudaMemcpy(w, U->w.p, U->off[kL] * sizeof(float), cudaMemcpyDeviceToHost));
    return AM_OK;
}

am_status am_unet_set_params(am_unet *U, const float *w) {
    UCKS(ucheck(U));
    if (!w) return ufail(AM_ERR_INVALID_ARG, "null input");
    const size_t o = U->off[kL];
    UCK(cudaMemcpy(U->w.p, w, o * sizeof(float), cudaMemcpyHostToDevice));
    UCK(f32_to_bf16(U->w.p, U->wb.p, (long long)o, U->st));
    UCK(refresh_wt(U, U->st));
    UCK(cudaMemsetAsync(U->m.p, 0, o * sizeof(float), U->st));
    UCK(cudaMemsetAsync(U->v.p, 0, o * sizeof(float), U->st));
    U->adam_t = 0;
    UCK(cudaStreamSynchronize(U->st));
    return AM_OK;
}

am_status am_unet_forward(am_unet *U, int n, int gz, int gy, int gx, const float *in, float *out, int sigmoid) {
    UCKS(ucheck(U));
    if (!grid_ok(n, gz, gy, gx)) return ufail(AM_ERR_INVALID_ARG, "grid dimensions must be positive multiples of 8");
    if (!in || !out) return ufail(AM_ERR_INVALID_ARG, "null tensor");
    const long long V = (long long)n * gz * gy * gx;
    UCK(ensure_uacts(U, U->infer, n, gz, gy, gx, false));
    UCK(U->hin.alloc((size_t)V * U->cin));
    UCK(U->hout.alloc((size_t)V * U->cout));
    UCK(cudaMemcpyAsync(U->hin.p, in, V * U->cin * sizeof(float), cudaMemcpyHostToDevice, U->st));
    pack_kernel<<<ub(V), 256, 0, U->st>>>(V, U->hin.p, U->cin, U->infer.x0);
    UCK(cudaGetLastError());
    UCK(unet_forward(U, U->infer, U->st));
    unpack_kernel<<<ub(V), 256, 0, U->st>>>(V, U->infer.out.p, U->cout, sigmoid, U->hout.p);
    UCK(cudaGetLastError());
    count_launches(2);
    UCK(cudaMemcpyAsync(out, U->hout.p, V * U->cout * sizeof(float), cudaMemcpyDeviceToHost, U->st));
    UCK(cudaStreamSynchronize(U->st));
    return conv_ok(U->st);
}

am_status am_unet_param_grad(am_unet *U, int n, int gz, int gy, int gx, const float *in, const float *dout,
                             float *grad) {
    UCKS(ucheck(U));
    if (!grid_ok(n, gz, gy, gx)) return ufail(AM_ERR_INVALID_ARG, "grid dimensions must be positive multiples of 8");
    if (!in || !dout || !grad) return ufail(AM_ERR_INVALID_ARG, "null tensor");
    const long long V = (long long)n * gz * gy * gx;
    UActs &A = U->train;
    UCK(ensure_uacts(U, A, n, gz, gy, gx, true));
    UCK(U->hin.alloc((size_t)V * U->cin));
    UCK(U->hout.alloc((size_t)V * U->cout));
    UCK(cudaMemcpyAsync(U->hin.p, in, V * U->cin * sizeof(float), cudaMemcpyHostToDevice, U->st));
    pack_kernel<<<ub(V), 256, 0, U->st>>>(V, U->hin.p, U->cin, A.x0);
    UCK(cudaGetLastError());
    UCK(unet_forward(U, A, U->st));
    UCK(cudaMemcpyAsync(U->hout.p, dout, V * U->cout * sizeof(float), cudaMemcpyHostToDevice, U->st));
    gout_kernel<<<ub(V), 256, 0, U->st>>>(V, U->hout.p, U->cout, A.gout);
    UCK(cudaGetLastError());
    UCK(cudaMemsetAsync(U->g.p, 0, U->off[kL] * sizeof(float), U->st));
    UCK(unet_backward(U, A, U->st));
    UCK(cudaMemcpyAsync(grad, U->g.p, U->off[kL] * sizeof(float), cudaMemcpyDeviceToHost, U->st));
    UCK(cudaStreamSynchronize(U->st));
    return conv_ok(U->st);
}

am_status am_unet_set_data(am_unet *U, int n_samples, int gz, int gy, int gx, const float *inputs,
                           const float *targets, const uint8_t *mask) {
    UCKS(ucheck(U));
    if (!grid_ok(n_samples, gz, gy, gx)) return ufail(AM_ERR_INVALID_ARG, "grid dimensions must be positive multiples of 8");
    if (!inputs || !targets || !mask) return ufail(AM_ERR_INVALID_ARG, "null tensor");
    const long long V = (long long)gz * gy * gx, SV = V * n_samples;
    UCK(U->xs.alloc((size_t)SV * 16));
    UCK(U->ts.alloc((size_t)SV));
    UCK(U->ms.alloc((size_t)SV));
    UCK(U->hin.alloc((size_t)SV * U->cin));
    UCK(cudaMemcpyAsync(U->hin.p, inputs, SV * U->cin * sizeof(float), cudaMemcpyHostToDevice, U->st));
    pack_kernel<<<ub(SV), 256, 0, U->st>>>(SV, U->hin.p, U->cin, U->xs.p);
    UCK(cudaGetLastError());
    count_launches(1);
    UCK(cudaMemcpyAsync(U->ts.p, targets, SV * sizeof(float), cudaMemcpyHostToDevice, U->st));
    UCK(cudaMemcpyAsync(U->ms.p, mask, (size_t)SV, cudaMemcpyHostToDevice, U->st));
    UCK(cudaStreamSynchronize(U->st));
    U->S = n_samples;
    U->gz = gz;
    U->gy = gy;
    U->gx = gx;
    return AM_OK;
}

}  // extern "C"

namespace {

// loss (and gradient into A.gout) of samples ids
am_status unet_batch(am_unet *U, const std::vector<int> &ids, bool grad, double *loss_sum, double *count) {
    const int nb = (int)ids.size();
    const long long V = (long long)U->gz * U->gy * U->gx, BV = V * nb;
    UActs &A = U->train;
    UCK(ensure_uacts(U, A, nb, U->gz, U->gy, U->gx, true));
    UCK(U->tbat.alloc((size_t)BV));
    UCK(U->mbat.alloc((size_t)BV));
    for (int b = 0; b < nb; ++b) {
        UCK(cudaMemcpyAsync(A.x0 + (size_t)b * V * 16, U->xs.p + (size_t)ids[b] * V * 16, V * 16 * sizeof(bf16),
                            cudaMemcpyDeviceToDevice, U->st));
        UCK(cudaMemcpyAsync(U->tbat.p + (size_t)b * V, U->ts.p + (size_t)ids[b] * V, V * sizeof(float),
                            cudaMemcpyDeviceToDevice, U->st));
        UCK(cudaMemcpyAsync(U->mbat.p + (size_t)b * V, U->ms.p + (size_t)ids[b] * V, (size_t)V,
                            cudaMemcpyDeviceToDevice, U->st));
    }
    UCK(unet_forward(U, A, U->st));
    UCK(cudaMemsetAsync(U->acc.p, 0, 2 * sizeof(double), U->st));
    // the count of masked cells scales the gradient; take it from the data (one pass)
    double h[2] = {0.0, 0.0};
    mse_kernel<<<ub(BV), 256, 0, U->st>>>(BV, A.out.p, U->tbat.p, U->mbat.p, 0.0, nullptr, U->acc.p);
    UCK(cudaGetLastError());
    UCK(cudaMemcpyAsync(h, U->acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, U->st));
    UCK(cudaStreamSynchronize(U->st));
    count_launches(1);
    if (grad) {
        UCK(cudaMemsetAsync(U->acc.p, 0, 2 * sizeof(double), U->st));
        mse_kernel<<<ub(BV), 256, 0, U->st>>>(BV, A.out.p, U->tbat.p, U->mbat.p, 1.0 / std::max(h[1], 1.0), A.gout,
                                             U->acc.p);
        UCK(cudaGetLastError());
        count_launches(1);
    }
    *loss_sum = h[0];
    *count = h[1];
    return AM_OK;
}

}  // namespace

extern "C" {

am_status am_unet_train(am_unet *U, const am_train_config *cfg, float *epoch_loss) {
    UCKS(ucheck(U));
    if (!cfg) return ufail(AM_ERR_INVALID_ARG, "null training config");
    if (U->S < 1) return ufail(AM_ERR_INVALID_ARG, "no training data (am_unet_set_data)");
    if (cfg->epochs < 0 || cfg->batch < 1) return ufail(AM_ERR_INVALID_ARG, "need epochs >= 0, batch >= 1");
    const int nb = std::min(cfg->batch, U->S);
    std::mt19937_64 rng(cfg->seed);
    std::vector<int> order((size_t)U->S);
    const size_t np = U->off[kL];
    for (int ep = 0; ep < cfg->epochs; ++ep) {
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::shuffle(order.begin(), order.end(), rng);
        double se = 0.0, cnt = 0.0;
        for (size_t s = 0; s + nb <= order.size(); s += nb) {
            std::vector<int> ids(order.begin() + s, order.begin() + s + nb);
            UCK(cudaMemsetAsync(U->g.p, 0, np * sizeof(float), U->st));
            double l = 0.0, c = 0.0;
            UCKS(unet_batch(U, ids, true, &l, &c));
            UCK(unet_backward(U, U->train, U->st));
            ++U->adam_t;
            UCK(adam_step(U->w.p, U->m.p, U->v.p, U->g.p, U->wb.p, (long long)np, cfg->lr, cfg->beta1, cfg->beta2,
                          cfg->eps, U->adam_t, 1.0f, U->st));
            UCK(refresh_wt(U, U->st));
            se += l;
            cnt += c;
        }
        UCKS(conv_ok(U->st));
        if (epoch_loss) epoch_loss[ep] = cnt > 0 ? (float)(se / cnt) : 0.f;
        if (cfg->verbose) std::printf("epoch %d: mse %.4e\n", ep, cnt > 0 ? se / cnt : 0.0);
    }
    UCK(cudaStreamSynchronize(U->st));
    return AM_OK;
}

am_status am_unet_eval(am_unet *U, double *mse) {
    UCKS(ucheck(U));
    if (!mse) return ufail(AM_ERR_INVALID_ARG, "null output");
    if (U->S < 1) return ufail(AM_ERR_INVALID_ARG, "no data");
    double se = 0.0, cnt = 0.0;
    for (int s = 0; s < U->S; s += 4) {
        std::vector<int> ids;
        for (int i = s; i < std::min(U->S, s + 4); ++i) ids.push_back(i);
        double l = 0.0, c = 0.0;
        UCKS(unet_batch(U, ids, false, &l, &c));
        se += l;
        cnt += c;
    }
    *mse = cnt > 0 ? se / cnt : 0.0;
    return conv_ok(U->st);
}

}  // extern "C"
