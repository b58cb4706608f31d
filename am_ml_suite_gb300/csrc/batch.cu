// batch.cu -- am_batch: many independent C++-variant SIMP problems of uneven
// sizes advanced together by batched persistent kernels (batch.cuh).
//
// One SIMP step of the batch is: scales + Jacobi diagonal, warm-start clean-up,
// FP64 defect correction (FP64 residual, FP32 Jacobi PCG on it updating the FP64
// iterate) until
// every problem's |F - K u| <= tol |F|, the FP64 residual with element energies,
// then sensitivities, u.F, filter and the FP64 OC bisection.  Each of these is one
// launch for the whole batch; the FP32 PCG iterations run as CUDA-graph chunks of
// 32 iterations, and a problem that has converged (or whose SIMP loop has ended)
// is skipped by its kernels.  The reference runs one TopologyOptimizer per
// problem (topology_optimizer.cpp:391-520); the per-problem results follow those
// semantics.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "batch.cuh"
#include "batch_axes.h"
#include "host_util.h"
#include "kernels.cuh"
#include "ku3.cuh"

using namespace amk;

namespace {

am_status bfail(am_status s, const std::string &msg) {
    set_last_error(msg.c_str());
    return s;
}

#define BCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return bfail(e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,       \
                         std::string(#call) + ": " + cudaGetErrorString(e_));              \
    } while (0)
#define BCKS(expr)                   \
    do {                             \
        am_status s_ = (expr);       \
        if (s_ != AM_OK) return s_;  \
    } while (0)

template <typename T>
struct Pool {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
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

constexpr int kChunk = 32;     // FP32 PCG iterations per CUDA-graph chunk
constexpr int kMaxRounds = 30; // defect-correction rounds per solve
constexpr int kSms = 152;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct am_batch {
    int device = 0;
    cudaStream_t st = nullptr;
    int n = 0;
    std::vector<Layout> L;  // internal (axis-permuted) layouts
    // per problem: the caller's grid dimensions, and the caller's axis that each
    // internal axis holds (axes[p][a] = physical axis of internal axis a)
    std::vector<std::array<int, 3>> dims, axes;
    double h = 1, E0 = 1, nu = 0.3;
    BatchConst C{};
    // offsets (in elements of the pool type) per problem
    std::vector<size_t> eoff, noff, foff, toff, poff;
    size_t nel_tot = 0, nn_tot = 0;
    // pools
    Pool<double> rho, rho_new, s64, ce, dc, dcf, oc_a, oc_lo, oc_hi;
    Pool<float> s32;
    Pool<uint8_t> design;
    Pool<double> F, x64, r64, dinv64;
    Pool<float> r32, pa, pb, q32, dinv32, xh, xl;
    Pool<uint8_t> mask, fixed_bits;
    // the tensor-copy staged PCG K*u: padded scale / constraint copies, per-problem
    // tensor maps and arguments, (problem, tile) work list; staged = 0 runs the
    // warp-row kernel with the autotuned plan instead
    Pool<float> s32pad;
    Pool<uint8_t> maskpad;
    Pool<Ku3BatchItem> k3items;
    Pool<int2> w_k3;
    WorkList k3{};
    bool staged = true;
    Pool<long long> f_idx;
    Pool<double> f_val;
    Pool<int4> tap_d;
    Pool<double> tap_w;
    Pool<double> partial;
    Pool<Scalars> S;
    Scalars *Sh = nullptr;  // pinned mirror
    Pool<BatchItem> items_d;
    std::vector<BatchItem> items;
    // work lists
    Pool<int2> w_elem, w_vec, w_k2, w_k2b, w_k64, w_prob, w_chunk;
    WorkList elem{}, vec{}, k2{}, k2b{}, k64{}, prob{}, chunk{};
    // FP32 K*u plan (autotuner): warps per CTA (0: each problem's own, 4 or 8), z chunk
    // (0 = all planes), CTAs per SM
    int warps = 8, zchunk = 0, ctas = 2;
    bool loads_set = false;
    cudaGraphExec_t graph = nullptr;  // one chunk of batched PCG iterations
    cudaGraphExec_t loop = nullptr;   // a whole FP32 PCG round: a device-side while loop over chunks
    Pool<int> loopc;                  // [0] chunks run by the loop, [1] its cap
    bool device_loop = true;
    std::vector<long long> pcg_its;
    // SIMP state between am_batch_simp_begin and the steps
    bool begun = false;
    std::vector<am_simp_config> cfg;
    std::vector<int> frozen, iters, conv;
    int max_chunks = 0;
};

namespace {

int div_up_i(long long a, long long b) { return (int)((a + b - 1) / b); }

am_status upload_worklist(am_batch *B, Pool<int2> &pool, WorkList &wl, const std::vector<int2> &w) {
    BCK(pool.alloc(w.size()));
    BCK(cudaMemcpy(pool.p, w.data(), w.size() * sizeof(int2), cudaMemcpyHostToDevice));
    wl.w = pool.p;
    wl.n = (int)w.size();
    (void)B;
    return AM_OK;
}

// FP32 K*u tiles of every problem for the plan (warps, zchunk); work items in
// descending tile height so the persistent grid ends with the short ones.  warps 0:
// per problem the tile height (4 or 8 warps: 7 or 15 node rows) that computes
// fewer element slots on its grid; the 8-warp problems' tiles go to list k2, the
// 4-warp ones' to k2b.
am_status plan_k2(am_batch *B, int warps, int zchunk) {
    struct T {
        int p, b, h;
    };
    std::vector<T> t8, t4;
    for (int p = 0; p < B->n; ++p) {
        const Layout &L = B->L[p];
        BatchItem &it = B->items[p];
        const int planes = L.nz + 1;
        const int tz = zchunk > 0 ? std::min(zchunk, planes) : planes;
        const int tiles_z = div_up_i(planes, tz);
        int w = warps;
        if (w == 0) {
            // element slots: 32 lanes x 2w rows per tile and plane, a halo plane per z chunk
            auto slots = [&](int ww) {
                return (long long)div_up_i(L.nx + 1, 30) * div_up_i(L.ny + 1, 2 * ww - 1) * 64 * ww *
                       (planes + tiles_z);
            };
            w = slots(4) < slots(8) ? 4 : 8;
        }
        it.k2_tiles_x = div_up_i(L.nx + 1, 30);
        it.k2_tiles_y = div_up_i(L.ny + 1, 2 * w - 1);
        it.k2_tz = tz;
        it.k2_tiles_z = tiles_z;
        it.n_k2 = it.k2_tiles_x * it.k2_tiles_y * it.k2_tiles_z;
        auto &tl = (warps == 0 && w == 4) ? t4 : t8;
        for (int b = 0; b < it.n_k2; ++b) {
            const int tzi = b / (it.k2_tiles_x * it.k2_tiles_y);
            const int h = std::min(it.k2_tz, planes - tzi * it.k2_tz);
            tl.push_back(T{p, b, h});
        }
    }
    auto upload = [&](std::vector<T> &t, Pool<int2> &pool, WorkList &wl) -> am_status {
        std::stable_sort(t.begin(), t.end(), [](const T &a, const T &b) { return a.h > b.h; });
        std::vector<int2> w(t.size());
        for (size_t i = 0; i < t.size(); ++i) w[i] = make_int2(t[i].p, t[i].b);
        if (w.empty()) {
            wl.w = nullptr;
            wl.n = 0;
            return AM_OK;
        }
        return upload_worklist(B, pool, wl, w);
    };
    BCKS(upload(t8, B->w_k2, B->k2));
    BCKS(upload(t4, B->w_k2b, B->k2b));
    BCK(cudaMemcpy(B->items_d.p, B->items.data(), B->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    B->warps = warps;
    B->zchunk = zchunk;
    if (B->graph) {
        cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
    }
    if (B->loop) {
        cudaGraphExecDestroy(B->loop);
        B->loop = nullptr;
    }
    return AM_OK;
}

// The staged K*u's records and work list: per problem the tensor maps of its
// FP32 PCG vectors and padded copies, tiles of 28 x 15 nodes over all planes (one
// z chunk: long tiles amortise each tile's pipeline fill), the tiles of the
// problems with the most planes first.
am_status plan_k3(am_batch *B) {
    using Sh = Ku3Shape<8, 4>;
    std::vector<Ku3BatchItem> rec(B->n);
    std::vector<std::pair<int, int2>> w;
    for (int p = 0; p < B->n; ++p) {
        const BatchItem &it = B->items[p];
        const Layout &L = it.L;
        cudaError_t err = cudaSuccess;
        Ku3Maps *T = ku3_make_maps(L, it.r32, it.pa, it.pb, it.dinv32, it.maskpad, it.s32pad, it.q32, 8, &err);
        if (!T) return bfail(AM_ERR_CUDA, "tensor maps of problem " + std::to_string(p) + ": " + cudaGetErrorString(err));
        Ku3BatchItem &r = rec[p];
        std::memset(&r, 0, sizeof(r));
        r.T = *T;
        ku3_free_maps(T);
        r.A.M = B->C.M32;
        r.A.partial = it.partial;
        r.A.S = it.S;
        r.A.tiles_x = div_up_i(L.nx + 1, Sh::TX);
        r.A.tiles_y = div_up_i(L.ny + 1, Sh::TY);
        r.A.tz = L.nz + 1;
        r.A.nz = L.nz;
        r.ntiles = r.A.tiles_x * r.A.tiles_y;
        for (int b = 0; b < r.ntiles; ++b) w.push_back({L.nz, make_int2(p, b)});
    }
    std::stable_sort(w.begin(), w.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    std::vector<int2> wl(w.size());
    for (size_t i = 0; i < w.size(); ++i) wl[i] = w[i].second;
    BCK(B->k3items.alloc(rec.size()));
    BCK(cudaMemcpy(B->k3items.p, rec.data(), rec.size() * sizeof(Ku3BatchItem), cudaMemcpyHostToDevice));
    return upload_worklist(B, B->w_k3, B->k3, wl);
}

// one batched FP32 PCG iteration: the staged K*u over the (problem, tile) list or
// the warp-row K*u of the autotuned plan, then the bulk-copy update
cudaError_t pcg_iteration(am_batch *B) {
    if (!B->staged)
        return batch_pcg_iteration(B->items_d.p, B->k2, B->k2b, B->chunk, B->C, B->warps, kSms * B->ctas, kSms * 2,
                                   B->st);
    if (cudaError_t e = batch_ku3_pcg(B->k3items.p, B->k3, B->C.M32, B->st)) return e;
    return batch_pcg_update(B->items_d.p, B->chunk, kSms * 2, B->st);
}

// The device-side loop of a batched FP32 PCG round: a CUDA-graph while node whose
// body is one chunk followed by batch_loop_next_kernel, which keeps the loop going
// while some problem of the batch is still iterating and fewer than the cap's
// chunks have run; batch_loop_reset_kernel, upstream of the node, zeroes the count
// and opens the loop if some problem is iterating.
__device__ __forceinline__ bool batch_any_active(const Scalars *S, int n) {
    int active = 0;
    for (int p = threadIdx.x; p < n; p += blockDim.x) active |= (!S[p].frozen && !S[p].done) ? 1 : 0;
    return __syncthreads_or(active) != 0;
}
__global__ void batch_loop_reset_kernel(cudaGraphConditionalHandle h, const Scalars *S, int n, int *loopc) {
    const bool active = batch_any_active(S, n);
    if (threadIdx.x == 0) {
        loopc[0] = 0;
        cudaGraphSetConditional(h, active ? 1u : 0u);
    }
}
__global__ void batch_loop_next_kernel(cudaGraphConditionalHandle h, const Scalars *S, int n, int *loopc) {
    const bool active = batch_any_active(S, n);
    if (threadIdx.x == 0) {
        const int c = ++loopc[0];
        cudaGraphSetConditional(h, (active && c < loopc[1]) ? 1u : 0u);
    }
}

am_status build_loop_graph(am_batch *B) {
    if (B->loop) return AM_OK;
    if (!B->loopc.p) BCK(B->loopc.alloc(2));
    const long long launches_before = launch_count();
    cudaGraph_t g = nullptr;
    BCK(cudaGraphCreate(&g, 0));
    auto bail = [&](cudaError_t e, const char *what) {
        cudaGraphDestroy(g);
        return bfail(AM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return bail(e, "batch loop handle");
    e = cudaStreamBeginCaptureToGraph(B->st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bail(e, "batch loop capture");
    batch_loop_reset_kernel<<<1, 256, 0, B->st>>>(h, B->S.p, B->n, B->loopc.p);
    e = cudaGetLastError();
    cudaGraph_t gc = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(B->st, &gc);
    if (e != cudaSuccess || e2 != cudaSuccess) return bail(e != cudaSuccess ? e : e2, "batch loop capture");
    cudaGraphNode_t reset = nullptr;
    size_t nn = 1;
    e = cudaGraphGetNodes(g, &reset, &nn);
    if (e != cudaSuccess || nn != 1) return bail(e != cudaSuccess ? e : cudaErrorUnknown, "batch loop reset node");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond = nullptr;
    e = cudaGraphAddNode(&cond, g, &reset, nullptr, 1, &cp);
    if (e != cudaSuccess) return bail(e, "batch loop node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(B->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bail(e, "batch loop body capture");
    for (int k = 0; k < kChunk && e == cudaSuccess; ++k) e = pcg_iteration(B);
    if (e == cudaSuccess) {
        batch_loop_next_kernel<<<1, 256, 0, B->st>>>(h, B->S.p, B->n, B->loopc.p);
        e = cudaGetLastError();
    }
    cudaGraph_t gb = nullptr;
    const cudaError_t e3 = cudaStreamEndCapture(B->st, &gb);
    if (e != cudaSuccess || e3 != cudaSuccess) return bail(e != cudaSuccess ? e : e3, "batch loop body capture");
    count_launches(launches_before - launch_count());  // captured, not executed
    e = cudaGraphInstantiate(&B->loop, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(AM_ERR_CUDA, std::string("batch loop instantiate: ") + cudaGetErrorString(e));
    return AM_OK;
}

am_status sync_scalars(am_batch *B) {
    BCK(cudaMemcpyAsync(B->Sh, B->S.p, sizeof(Scalars) * B->n, cudaMemcpyDeviceToHost, B->st));
    BCK(cudaStreamSynchronize(B->st));
    return AM_OK;
}

am_status build_graph(am_batch *B) {
    if (B->device_loop) return build_loop_graph(B);
    if (B->graph) return AM_OK;
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kChunk && e == cudaSuccess; ++k) e = pcg_iteration(B);
    cudaError_t e2 = cudaStreamEndCapture(B->st, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(AM_ERR_CUDA, std::string("batch graph capture: ") +
                                      cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(AM_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    return AM_OK;
}

bool all_done(const am_batch *B) {
    for (int p = 0; p < B->n; ++p)
        if (!B->Sh[p].frozen && !B->Sh[p].done) return false;
    return true;
}

// FP64 defect correction around FP32 Jacobi PCG for every active problem.
am_status batch_solve(am_batch *B, int max_chunks) {
    for (int round = 0; round < kMaxRounds; ++round) {
        BCK(batch_resid(B->items_d.p, B->k64, B->C, 0, kSms * 4, B->st));
        BCK(batch_inner_start(B->items_d.p, B->vec, kSms * 8, B->st));
        BCKS(sync_scalars(B));
        for (int p = 0; p < B->n; ++p)
            if (!B->Sh[p].frozen && !std::isfinite(B->Sh[p].res_rr))
                return bfail(AM_ERR_NAN_DETECTED, "NaN in the residual of batch problem " + std::to_string(p));
        if (all_done(B)) return AM_OK;
        if (B->device_loop) {
            // the round's chunks in one graph launch, the loop decided on the device
            const int lc[2] = {0, max_chunks + 1};
            BCK(cudaMemcpyAsync(B->loopc.p, lc, sizeof(lc), cudaMemcpyHostToDevice, B->st));
            BCK(cudaGraphLaunch(B->loop, B->st));
            int ran[2] = {0, 0};
            BCK(cudaMemcpyAsync(ran, B->loopc.p, sizeof(ran), cudaMemcpyDeviceToHost, B->st));
            BCKS(sync_scalars(B));
            count_launches(1 + (2LL * kChunk + 1) * ran[0]);
            if (!all_done(B)) return bfail(AM_ERR_TIMEOUT, "batched PCG did not stop within its cap");
        } else {
            int chunks = 0;
            while (true) {
                BCK(cudaGraphLaunch(B->graph, B->st));
                count_launches(2LL * kChunk);
                BCKS(sync_scalars(B));
                ++chunks;
                if (all_done(B)) break;
                if (chunks > max_chunks) return bfail(AM_ERR_TIMEOUT, "batched PCG did not stop within its cap");
            }
        }
        BCK(batch_inner_end(B->items_d.p, B->vec, kSms * 8, B->st));
        for (int p = 0; p < B->n; ++p) {
            if (B->Sh[p].frozen) continue;
            if (B->Sh[p].status == ST_NAN)
                return bfail(AM_ERR_NAN_DETECTED, "NaN in the PCG of batch problem " + std::to_string(p));
            if (B->Sh[p].status == ST_TIMEOUT)
                return bfail(AM_ERR_TIMEOUT, "a bulk-copy wait of the batched PCG update timed out");
            B->pcg_its[p] += B->Sh[p].it;
        }
    }
    return AM_OK;  // not converged within the rounds: reported through the residuals
}

am_status check_batch(am_batch *B) {
    if (!B) return bfail(AM_ERR_INVALID_ARG, "null batch");
    BCK(cudaSetDevice(B->device));
    return AM_OK;
}

}  // namespace

extern "C" {

am_status am_batch_destroy(am_batch *B) {
    if (!B) return AM_OK;
    cudaSetDevice(B->device);
    if (B->st) cudaStreamSynchronize(B->st);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    if (B->loop) cudaGraphExecDestroy(B->loop);
    B->loopc.release();
    for (auto *q : {&B->rho, &B->rho_new, &B->s64, &B->ce, &B->dc, &B->dcf, &B->oc_a, &B->oc_lo, &B->oc_hi,
                    &B->F, &B->x64, &B->r64, &B->dinv64, &B->f_val, &B->tap_w, &B->partial})
        q->release();
    for (auto *q : {&B->s32, &B->r32, &B->pa, &B->pb, &B->q32, &B->dinv32, &B->xh, &B->xl, &B->s32pad}) q->release();
    for (auto *q : {&B->design, &B->mask, &B->fixed_bits, &B->maskpad}) q->release();
    B->k3items.release();
    B->w_k3.release();
    for (auto *q : {&B->w_elem, &B->w_vec, &B->w_k2, &B->w_k2b, &B->w_k64, &B->w_prob, &B->w_chunk}) q->release();
    B->f_idx.release();
    B->tap_d.release();
    B->S.release();
    B->items_d.release();
    if (B->Sh) cudaFreeHost(B->Sh);
    if (B->st) cudaStreamDestroy(B->st);
    delete B;
    return AM_OK;
}

am_status am_batch_create(int n, const int *shapes, double h, double E0, double nu, am_batch **out) {
    if (!out) return bfail(AM_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (n < 1 || !shapes) return bfail(AM_ERR_INVALID_ARG, "need n >= 1 problems and their shapes");
    if (!(h > 0.0) || !(E0 > 0.0) || !(nu > -1.0 && nu < 0.5))
        return bfail(AM_ERR_INVALID_ARG, "need h > 0, E0 > 0, -1 < nu < 0.5");
    for (int p = 0; p < n; ++p) {
        if (shapes[3 * p] < 1 || shapes[3 * p + 1] < 1 || shapes[3 * p + 2] < 1)
            return bfail(AM_ERR_INVALID_ARG, "problem " + std::to_string(p) + ": dimensions must be >= 1");
        // the batched warp-row K*u indexes a problem's nodes with 32-bit integers
        const std::array<int, 3> ax = best_axes(shapes + 3 * p);
        if (3 * make_layout(shapes[3 * p + ax[0]], shapes[3 * p + ax[1]], shapes[3 * p + ax[2]]).cs >= (1LL << 31))
            return bfail(AM_ERR_SIZE_MISMATCH, "problem " + std::to_string(p) + ": too large for a batch");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return bfail(AM_ERR_NO_DEVICE, "no CUDA device");
    am_batch *B = new am_batch();
    cudaGetDevice(&B->device);
    B->n = n;
    B->h = h;
    B->E0 = E0;
    B->nu = nu;
    B->C.M64 = modal_constants(E0, nu, h);
    B->C.M32 = modal_float(B->C.M64);
    B->C.d0 = element_stiffness_entry(B->C.M64, 0, 0);
    B->L.resize(n);
    B->dims.resize(n);
    B->axes.resize(n);
    B->eoff.resize(n + 1);
    B->noff.resize(n + 1);
    B->poff.resize(n + 1);
    B->items.assign(n, BatchItem{});
    B->pcg_its.assign(n, 0);
    size_t e = 0, nn = 0, pp = 0, sp = 0, mp = 0;
    std::vector<size_t> spoff(n), mpoff(n);
    for (int p = 0; p < n; ++p) {
        const int *d = shapes + 3 * p;
        B->dims[p] = {d[0], d[1], d[2]};
        B->axes[p] = best_axes(d);
        const std::array<int, 3> &ax = B->axes[p];
        const Layout L = make_layout(d[ax[0]], d[ax[1]], d[ax[2]]);
        B->L[p] = L;
        BatchItem &it = B->items[p];
        it.L = L;
        it.n_vec = std::max(1, div_up_i(L.cs, 4LL * BATCH_VEC_THREADS));
        it.n_elem = std::max(1, div_up_i(L.nel, 4LL * 256));
        it.k64_tiles_x = div_up_i(L.nx + 1, 32);
        it.k64_tiles_y = div_up_i(L.ny + 1, 4);
        it.k64_tz = L.nz + 1;
        it.k64_tiles_z = 1;
        it.n_k64 = it.k64_tiles_x * it.k64_tiles_y;
        B->eoff[p] = e;
        B->noff[p] = nn;
        B->poff[p] = pp;
        e += align_up((size_t)L.nel, 64);
        nn += (size_t)L.cs;  // multiple of 64
        // partials: 2 per K*u tile (either plan: at most 15x more tiles than 4-warp
        // ku2 tiles of 1 plane), 3 per element block, 2 per vector block
        const size_t k2max = (size_t)div_up_i(L.nx + 1, 30) * div_up_i(L.ny + 1, 7) * (L.nz + 1);
        const size_t nchunk = 3 * (size_t)div_up_i(L.cs, BATCH_UPD_CHUNK);
        const size_t k3 = (size_t)div_up_i(L.nx + 1, Ku3Shape<8, 4>::TX) * div_up_i(L.ny + 1, Ku3Shape<8, 4>::TY);
        pp += align_up(std::max({2 * k2max, 2 * k3, 2 * (size_t)it.n_k64, 3 * (size_t)it.n_elem,
                                 2 * (size_t)it.n_vec, 2 * nchunk, (size_t)16}),
                       32);
        // padded copies for the staged K*u (16-byte aligned rows; 256-byte aligned starts)
        long long se = 0, mb = 0;
        ku3_padded_sizes(L, &se, &mb);
        spoff[p] = sp;
        mpoff[p] = mp;
        sp += align_up((size_t)se, 64);
        mp += align_up((size_t)mb, 256);
    }
    B->eoff[n] = e;
    B->noff[n] = nn;
    B->poff[n] = pp;
    B->nel_tot = e;
    B->nn_tot = nn;
    cudaError_t ce = cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking);
    auto A = [&](auto &pool, size_t cnt) {
        if (ce == cudaSuccess) ce = pool.alloc(cnt);
    };
    for (auto *q : {&B->rho, &B->rho_new, &B->s64, &B->ce, &B->dc, &B->dcf, &B->oc_a, &B->oc_lo, &B->oc_hi}) A(*q, e);
    A(B->s32, e);
    A(B->design, e);
    for (auto *q : {&B->F, &B->x64, &B->r64}) A(*q, 3 * nn);
    A(B->dinv64, nn);
    for (auto *q : {&B->r32, &B->pa, &B->pb, &B->q32, &B->xh, &B->xl}) A(*q, 3 * nn);
    A(B->dinv32, nn);
    A(B->mask, nn);
    A(B->fixed_bits, nn);
    A(B->s32pad, sp);
    A(B->maskpad, mp);
    A(B->partial, pp);
    A(B->S, (size_t)n);
    A(B->items_d, (size_t)n);
    if (ce == cudaSuccess) ce = cudaMallocHost(&B->Sh, sizeof(Scalars) * n);
    if (ce != cudaSuccess) {
        am_batch_destroy(B);
        return bfail(ce == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                     std::string("batch create: ") + cudaGetErrorString(ce));
    }
    std::vector<int2> we, wv, w64, wp, wc;
    for (int p = 0; p < n; ++p) {
        BatchItem &it = B->items[p];
        const size_t eo = B->eoff[p], no = B->noff[p];
        it.rho = B->rho.p + eo;
        it.rho_new = B->rho_new.p + eo;
        it.s64 = B->s64.p + eo;
        it.ce = B->ce.p + eo;
        it.dc = B->dc.p + eo;
        it.dcf = B->dcf.p + eo;
        it.oc_a = B->oc_a.p + eo;
        it.oc_lo = B->oc_lo.p + eo;
        it.oc_hi = B->oc_hi.p + eo;
        it.s32 = B->s32.p + eo;
        it.design = B->design.p + eo;
        it.F = B->F.p + 3 * no;
        it.x64 = B->x64.p + 3 * no;
        it.r64 = B->r64.p + 3 * no;
        it.dinv64 = B->dinv64.p + no;
        it.r32 = B->r32.p + 3 * no;
        it.pa = B->pa.p + 3 * no;
        it.pb = B->pb.p + 3 * no;
        it.q32 = B->q32.p + 3 * no;
        it.xh = B->xh.p + 3 * no;
        it.xl = B->xl.p + 3 * no;
        it.dinv32 = B->dinv32.p + no;
        it.mask = B->mask.p + no;
        it.s32pad = B->s32pad.p + spoff[p];
        it.maskpad = B->maskpad.p + mpoff[p];
        it.fixed_bits = B->fixed_bits.p + no;
        it.partial = B->partial.p + B->poff[p];
        it.S = B->S.p + p;
        for (int b = 0; b < it.n_elem; ++b) we.push_back(make_int2(p, b));
        for (int b = 0; b < it.n_vec; ++b) wv.push_back(make_int2(p, b));
        for (int b = 0; b < 3 * div_up_i(it.L.cs, BATCH_UPD_CHUNK); ++b) wc.push_back(make_int2(p, b));
        for (int b = 0; b < it.n_k64; ++b) w64.push_back(make_int2(p, b));
        wp.push_back(make_int2(p, 0));
    }
    am_status s = upload_worklist(B, B->w_elem, B->elem, we);
    if (s == AM_OK) s = upload_worklist(B, B->w_vec, B->vec, wv);
    if (s == AM_OK) s = upload_worklist(B, B->w_k64, B->k64, w64);
    if (s == AM_OK) s = upload_worklist(B, B->w_prob, B->prob, wp);
    if (s == AM_OK) s = upload_worklist(B, B->w_chunk, B->chunk, wc);
    if (s == AM_OK) s = plan_k2(B, 8, 0);
    if (s == AM_OK) s = plan_k3(B);
    if (s == AM_OK && (ku_init_attributes() != cudaSuccess || batch_ku3_init_attributes() != cudaSuccess))
        s = bfail(AM_ERR_CUDA, "kernel attributes");
    if (s != AM_OK) {
        am_batch_destroy(B);
        return s;
    }
    *out = B;
    return AM_OK;
}

am_status am_batch_set_loads(am_batch *B, const double *F, const int64_t *fixed, const int64_t *n_fixed) {
    BCKS(check_batch(B));
    if (!F || !n_fixed) return bfail(AM_ERR_INVALID_ARG, "null loads");
    std::vector<double> Fd(3 * B->nn_tot, 0.0);
    std::vector<uint8_t> fb(B->nn_tot, 0);
    std::vector<long long> idx;
    std::vector<double> val;
    std::vector<size_t> foff(B->n + 1);
    size_t fo = 0, xo = 0;
    for (int p = 0; p < B->n; ++p) {
        const Layout &L = B->L[p];
        const std::array<int, 3> &ax = B->axes[p], &dm = B->dims[p];
        const long long nn = (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
        const size_t no = B->noff[p];
        // the internal node of reference node r = (i*(ny+1) + j)*(nz+1) + k (the
        // caller's dimensions and axis order)
        auto node_of = [&](long long r) {
            long long c3[3], q[3];
            c3[2] = r % (dm[2] + 1);
            const long long t = r / (dm[2] + 1);
            c3[1] = t % (dm[1] + 1);
            c3[0] = t / (dm[1] + 1);
            to_internal(ax, c3, q);
            return node_index(L, (int)q[0], (int)q[1], (int)q[2]);
        };
        foff[p] = idx.size();
        for (long long r = 0; r < nn; ++r) {
            const long long d = node_of(r);
            for (int c = 0; c < 3; ++c) {
                const double v = F[fo + 3 * r + c];
                if (!std::isfinite(v)) return bfail(AM_ERR_NAN_DETECTED, "non-finite force, problem " + std::to_string(p));
                const int ci = internal_component(ax, c);
                Fd[3 * no + (size_t)ci * L.cs + d] = v;
                if (v != 0.0) {
                    idx.push_back((long long)ci * L.cs + d);
                    val.push_back(v);
                }
            }
        }
        const int64_t nf = n_fixed[p];
        if (nf < 0) return bfail(AM_ERR_INVALID_ARG, "negative fixed-DOF count");
        if (nf > 0 && !fixed) return bfail(AM_ERR_INVALID_ARG, "null fixed DOFs");
        for (int64_t q = 0; q < nf; ++q) {
            const int64_t dof = fixed[xo + q];
            if (dof < 0 || dof >= 3 * nn)
                return bfail(AM_ERR_DOF_OUT_OF_RANGE, "fixed DOF out of range, problem " + std::to_string(p));
            const int c = internal_component(ax, (int)(dof % 3));
            fb[no + node_of(dof / 3)] |= (uint8_t)(1u << c);
        }
        fo += 3 * (size_t)nn;
        xo += (size_t)nf;
    }
    foff[B->n] = idx.size();
    BCK(B->f_idx.alloc(std::max<size_t>(idx.size(), 1)));
    BCK(B->f_val.alloc(std::max<size_t>(val.size(), 1)));
    if (!idx.empty()) {
        BCK(cudaMemcpy(B->f_idx.p, idx.data(), idx.size() * sizeof(long long), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(B->f_val.p, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    BCK(cudaMemcpy(B->F.p, Fd.data(), Fd.size() * sizeof(double), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(B->fixed_bits.p, fb.data(), fb.size(), cudaMemcpyHostToDevice));
    for (int p = 0; p < B->n; ++p) {
        BatchItem &it = B->items[p];
        it.f_idx = B->f_idx.p + foff[p];
        it.f_val = B->f_val.p + foff[p];
        it.f_nnz = (int)(foff[p + 1] - foff[p]);
    }
    BCK(cudaMemcpy(B->items_d.p, B->items.data(), B->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    B->loads_set = true;
    return AM_OK;
}

am_status am_batch_set_staged(am_batch *B, int on) {
    BCKS(check_batch(B));
    if ((on != 0) != B->staged) {
        B->staged = on != 0;
        // the chunk graphs hold the other kernel
        if (B->graph) cudaGraphExecDestroy(B->graph);
        if (B->loop) cudaGraphExecDestroy(B->loop);
        B->graph = nullptr;
        B->loop = nullptr;
        // the padded copies are refreshed with the operator at every step; a switch
        // between steps refreshes them now
        if (B->staged && B->begun) BCK(batch_ku3_pad(B->items_d.p, B->vec, kSms * 8, B->st));
    }
    return AM_OK;
}

am_status am_batch_bench_ku(am_batch *B, int reps, double *avg_ms) {
    BCKS(check_batch(B));
    if (!B->begun) return bfail(AM_ERR_INVALID_ARG, "am_batch_simp_begin not called");
    if (reps < 1 || !avg_ms) return bfail(AM_ERR_INVALID_ARG, "need reps >= 1 and an output");
    // every problem iterating, first PCG iteration (beta 0: p = D^-1 r, p_prev not
    // read), on the residual and operator the last step left; state restored after
    BCK(batch_operator(B->items_d.p, B->elem, B->vec, B->C, kSms * 8, B->st));
    if (B->staged) BCK(batch_ku3_pad(B->items_d.p, B->vec, kSms * 8, B->st));
    BCKS(sync_scalars(B));
    std::vector<Scalars> saved(B->Sh, B->Sh + B->n), run(saved);
    for (Scalars &S : run) {
        S.done = 0;
        S.frozen = 0;
        S.it = 0;
        S.beta = 0.0;
        S.rz = 1.0;
        S.cnt_ku = 0;
        S.kerr = 0;
    }
    // the timed launches; the events are destroyed and the solver state restored
    // whether or not they succeed
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double tot = 0.0;
    auto timed = [&]() -> cudaError_t {
        cudaError_t e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        for (int r = 0; r < reps + 1 && e == cudaSuccess; ++r) {  // the first launch warms up
            e = cudaMemcpyAsync(B->S.p, run.data(), sizeof(Scalars) * B->n, cudaMemcpyHostToDevice, B->st);
            if (e == cudaSuccess) e = cudaEventRecord(e0, B->st);
            if (e == cudaSuccess)
                e = B->staged ? batch_ku3_pcg(B->k3items.p, B->k3, B->C.M32, B->st)
                              : batch_pcg_ku(B->items_d.p, B->k2, B->k2b, B->C, B->warps, kSms * B->ctas, B->st);
            if (e == cudaSuccess) e = cudaEventRecord(e1, B->st);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) tot += ms;
        }
        return e;
    };
    const cudaError_t et = timed();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    BCK(cudaMemcpyAsync(B->S.p, saved.data(), sizeof(Scalars) * B->n, cudaMemcpyHostToDevice, B->st));
    BCK(cudaStreamSynchronize(B->st));
    BCK(et);
    *avg_ms = tot / reps;
    return AM_OK;
}

am_status am_batch_axes(am_batch *B, int i, int *axes) {
    BCKS(check_batch(B));
    if (i < 0 || i >= B->n || !axes) return bfail(AM_ERR_INVALID_ARG, "problem index out of range or null output");
    for (int a = 0; a < 3; ++a) axes[a] = B->axes[i][a];
    return AM_OK;
}

am_status am_batch_set_plan(am_batch *B, int warps, int z_chunk, int ctas_per_sm) {
    BCKS(check_batch(B));
    if (!(warps == 0 || warps == 4 || warps == 8) || z_chunk < 0 || ctas_per_sm < 1 || ctas_per_sm > 4)
        return bfail(AM_ERR_INVALID_ARG, "plan: warps 0, 4 or 8; z_chunk >= 0; 1-4 CTAs per SM");
    BCKS(plan_k2(B, warps, z_chunk));
    B->ctas = ctas_per_sm;
    return AM_OK;
}

am_status am_batch_autotune(am_batch *B, int reps, int *warps, int *z_chunk, int *ctas_per_sm, double *best_ms) {
    BCKS(check_batch(B));
    if (reps < 1) return bfail(AM_ERR_INVALID_ARG, "reps must be >= 1");
    struct Cand {
        int w, z, c;
    };
    // w = 0: each problem's own tile height (4 or 8 warps)
    const Cand cands[] = {{8, 0, 2}, {8, 16, 2}, {8, 8, 2}, {8, 0, 1}, {4, 0, 4}, {4, 16, 4},
                          {4, 8, 4}, {4, 0, 2}, {0, 0, 2}, {0, 16, 2}, {0, 8, 2}};
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    double best = 1e300;
    Cand bc = cands[0];
    for (const Cand &c : cands) {
        BCKS(plan_k2(B, c.w, c.z));
        BCK(batch_ku_plain(B->items_d.p, B->k2, B->k2b, B->C, c.w, kSms * c.c, B->st));  // warm-up
        BCK(cudaEventRecord(e0, B->st));
        for (int r = 0; r < reps; ++r) BCK(batch_ku_plain(B->items_d.p, B->k2, B->k2b, B->C, c.w, kSms * c.c, B->st));
        BCK(cudaEventRecord(e1, B->st));
        BCK(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        const double avg = ms / reps;
        if (avg < best) {
            best = avg;
            bc = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    BCKS(plan_k2(B, bc.w, bc.z));
    B->ctas = bc.c;
    if (warps) *warps = bc.w;
    if (z_chunk) *z_chunk = bc.z;
    if (ctas_per_sm) *ctas_per_sm = bc.c;
    if (best_ms) *best_ms = best;
    return AM_OK;
}

am_status am_batch_set_device_loop(am_batch *B, int on) {
    BCKS(check_batch(B));
    B->device_loop = on != 0;
    return AM_OK;
}

am_status am_batch_stream(am_batch *B, void **stream) {
    BCKS(check_batch(B));
    if (!stream) return bfail(AM_ERR_INVALID_ARG, "null output");
    *stream = (void *)B->st;
    return AM_OK;
}

am_status am_batch_simp_begin(am_batch *B, const am_simp_config *cfgs, const double *rho0) {
    BCKS(check_batch(B));
    if (!cfgs) return bfail(AM_ERR_INVALID_ARG, "null configs");
    if (!B->loads_set) return bfail(AM_ERR_INVALID_ARG, "loads not set");
    const int n = B->n;
    for (int p = 0; p < n; ++p) {
        const am_simp_config &c = cfgs[p];
        const std::string w = "problem " + std::to_string(p) + ": ";
        if (c.variant != AM_VARIANT_CPP) return bfail(AM_ERR_INVALID_ARG, w + "batches run the C++ variant");
        if (c.layout != AM_LAYOUT_ZFASTEST && c.layout != AM_LAYOUT_XFASTEST)
            return bfail(AM_ERR_INVALID_ARG, w + "unknown layout");
        if (!(c.volume_fraction > 0.0 && c.volume_fraction <= 1.0))
            return bfail(AM_ERR_INVALID_ARG, w + "volume_fraction must be in (0, 1]");
        if (!(c.penalty >= 1.0) || !(c.move_limit > 0.0) || !(c.rho_min >= 0.0) || !(c.E_min >= 0.0))
            return bfail(AM_ERR_INVALID_ARG, w + "need penalty >= 1, move_limit > 0, rho_min >= 0, E_min >= 0");
        if (!(c.cg_tol > 0.0)) return bfail(AM_ERR_INVALID_ARG, w + "cg_tol must be > 0");
        if (!(c.filter_radius > 0.0) || c.filter_radius > 6.0)
            return bfail(AM_ERR_INVALID_ARG, w + "filter_radius must be in (0, 6]");
        if (c.max_iterations < 0) return bfail(AM_ERR_INVALID_ARG, w + "max_iterations < 0");
    }
    B->begun = false;
    // densities, design masks, taps, parameters
    std::vector<double> r0(B->nel_tot, 0.0);
    std::vector<uint8_t> dm(B->nel_tot, 0);
    std::vector<int4> td;
    std::vector<double> tw;
    std::vector<size_t> toff(n + 1);
    size_t ho = 0;
    int max_maxit = 1;
    for (int p = 0; p < n; ++p) {
        const am_simp_config &c = cfgs[p];
        const Layout &L = B->L[p];
        const size_t eo = B->eoff[p];
        long long nd = 0;
        for (long long ez = 0; ez < L.nz; ++ez)
            for (long long ey = 0; ey < L.ny; ++ey)
                for (long long ex = 0; ex < L.nx; ++ex) {
                    const long long e = (ez * L.ny + ey) * L.nx + ex;
                    const long long hidx = host_element(B->axes[p], B->dims[p], c.layout == AM_LAYOUT_ZFASTEST, ex, ey, ez);
                    const double v = rho0 ? rho0[ho + hidx] : c.volume_fraction;
                    r0[eo + e] = v;
                    // design mask from the initial density (topology_optimizer.cpp:419-428)
                    const bool d = v > c.rho_min + 1e-6 && v < 0.99;
                    dm[eo + e] = d;
                    nd += d;
                }
        ho += (size_t)L.nel;
        std::vector<int4> d;
        std::vector<double> w;
        filter_taps(c.filter_radius, 0, d, w);
        toff[p] = td.size();
        td.insert(td.end(), d.begin(), d.end());
        tw.insert(tw.end(), w.begin(), w.end());
        BatchItem &it = B->items[p];
        it.penalty = c.penalty;
        it.emin = c.E_min;
        it.rho_min = c.rho_min;
        it.move = c.move_limit;
        it.vf = c.volume_fraction;
        it.n_design = nd == 0 ? (double)L.nel : (double)nd;
        it.tol = c.cg_tol;
        it.maxit = c.cg_max_iterations > 0 ? c.cg_max_iterations : 100000;
        max_maxit = std::max(max_maxit, it.maxit);
    }
    toff[n] = td.size();
    BCK(B->tap_d.alloc(td.size()));
    BCK(B->tap_w.alloc(tw.size()));
    BCK(cudaMemcpy(B->tap_d.p, td.data(), td.size() * sizeof(int4), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(B->tap_w.p, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice));
    for (int p = 0; p < n; ++p) {
        BatchItem &it = B->items[p];
        it.tap_d = B->tap_d.p + toff[p];
        it.tap_w = B->tap_w.p + toff[p];
        it.ntaps = (int)(toff[p + 1] - toff[p]);
    }
    BCK(cudaMemcpy(B->items_d.p, B->items.data(), B->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(B->rho.p, r0.data(), r0.size() * sizeof(double), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(B->design.p, dm.data(), dm.size(), cudaMemcpyHostToDevice));
    BCK(cudaMemset(B->x64.p, 0, sizeof(double) * B->x64.n));  // cold start; warm starts between steps
    BCK(cudaMemset(B->S.p, 0, sizeof(Scalars) * n));
    B->cfg.assign(cfgs, cfgs + n);
    B->frozen.assign(n, 0);
    B->iters.assign(n, 0);
    B->conv.assign(n, 0);
    for (int p = 0; p < n; ++p) {
        if (cfgs[p].max_iterations == 0) {
            B->frozen[p] = 1;
            BCK(cudaMemcpy(&B->S.p[p].frozen, &B->frozen[p], sizeof(int), cudaMemcpyHostToDevice));
        }
    }
    std::fill(B->pcg_its.begin(), B->pcg_its.end(), 0);
    BCKS(build_graph(B));
    B->max_chunks = max_maxit / kChunk + 2;
    B->begun = true;
    return AM_OK;
}

am_status am_batch_simp_step(am_batch *B, double *compliance, double *volume, double *change,
                             long long *pcg_iterations, int *n_active) {
    BCKS(check_batch(B));
    if (!B->begun) return bfail(AM_ERR_INVALID_ARG, "am_batch_simp_begin not called");
    BCKS(build_graph(B));  // after a re-plan by the autotuner
    const int n = B->n;
    if (std::all_of(B->frozen.begin(), B->frozen.end(), [](int f) { return f != 0; })) {
        if (n_active) *n_active = 0;
        return AM_OK;
    }
    BCK(batch_operator(B->items_d.p, B->elem, B->vec, B->C, kSms * 8, B->st));
    if (B->staged) BCK(batch_ku3_pad(B->items_d.p, B->vec, kSms * 8, B->st));
    BCK(batch_prepare_solve(B->items_d.p, B->vec, B->prob, kSms * 8, B->st));
    BCKS(batch_solve(B, B->max_chunks));
    BCK(batch_resid(B->items_d.p, B->k64, B->C, 1, kSms * 4, B->st));
    BCK(batch_update(B->items_d.p, B->elem, B->prob, kSms * 8, B->st));
    BCKS(sync_scalars(B));
    int active = 0;
    for (int p = 0; p < n; ++p) {
        if (B->frozen[p]) continue;
        const Scalars &S = B->Sh[p];
        if (compliance) compliance[p] = S.comp_fu;
        if (volume) volume[p] = S.oc_volume;
        if (change) change[p] = S.oc_change;
        B->iters[p] += 1;
        bool stop = false;
        if (S.oc_change < B->cfg[p].convergence_tol) {
            B->conv[p] = 1;
            stop = true;
        }
        if (B->iters[p] >= B->cfg[p].max_iterations) stop = true;
        if (stop) {
            B->frozen[p] = 1;
            BCK(cudaMemcpyAsync(&B->S.p[p].frozen, &B->frozen[p], sizeof(int), cudaMemcpyHostToDevice, B->st));
        } else {
            ++active;
        }
    }
    BCK(cudaStreamSynchronize(B->st));
    if (pcg_iterations)
        for (int p = 0; p < n; ++p) pcg_iterations[p] = B->pcg_its[p];
    if (n_active) *n_active = active;
    return AM_OK;
}

am_status am_batch_get_density(am_batch *B, double *rho_out) {
    BCKS(check_batch(B));
    if (!B->begun) return bfail(AM_ERR_INVALID_ARG, "am_batch_simp_begin not called");
    if (!rho_out) return bfail(AM_ERR_INVALID_ARG, "null output");
    std::vector<double> r(B->nel_tot);
    BCK(cudaMemcpy(r.data(), B->rho.p, r.size() * sizeof(double), cudaMemcpyDeviceToHost));
    size_t o = 0;
    for (int p = 0; p < B->n; ++p) {
        const Layout &L = B->L[p];
        const size_t eo = B->eoff[p];
        for (long long ez = 0; ez < L.nz; ++ez)
            for (long long ey = 0; ey < L.ny; ++ey)
                for (long long ex = 0; ex < L.nx; ++ex) {
                    const long long e = (ez * L.ny + ey) * L.nx + ex;
                    const long long hidx = host_element(B->axes[p], B->dims[p], B->cfg[p].layout == AM_LAYOUT_ZFASTEST, ex, ey, ez);
                    rho_out[o + hidx] = r[eo + e];
                }
        o += (size_t)L.nel;
    }
    return AM_OK;
}

am_status am_batch_simp_run(am_batch *B, const am_simp_config *cfgs, const double *rho0, double *rho_out,
                            double *compliance_hist, double *volume_hist, int *iterations, int *converged,
                            long long *pcg_iterations) {
    BCKS(am_batch_simp_begin(B, cfgs, rho0));
    const int n = B->n;
    int hist = 0;
    for (int p = 0; p < n; ++p) hist = std::max(hist, cfgs[p].max_iterations);
    std::vector<double> c(n), v(n);
    for (int step = 0; step < hist; ++step) {
        int active = 0;
        std::vector<int> was(B->frozen);
        BCKS(am_batch_simp_step(B, c.data(), v.data(), nullptr, nullptr, &active));
        for (int p = 0; p < n; ++p) {
            if (was[p]) continue;
            if (compliance_hist) compliance_hist[(size_t)p * hist + step] = c[p];
            if (volume_hist) volume_hist[(size_t)p * hist + step] = v[p];
        }
        if (active == 0) break;
    }
    if (rho_out) BCKS(am_batch_get_density(B, rho_out));
    for (int p = 0; p < n; ++p) {
        if (iterations) iterations[p] = B->iters[p];
        if (converged) converged[p] = B->conv[p];
        if (pcg_iterations) pcg_iterations[p] = B->pcg_its[p];
    }
    return AM_OK;
}

}  // extern "C"
