// am_gpu.cu -- host side of the GB300 SIMP engine: problem handles, the PCG /
// defect-correction drivers (CUDA-graph chunks of device-driven iterations), the
// SIMP loop of both reference variants, and the extern "C" ABI of include/am_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "host_util.h"
#include "kernels.cuh"
#include "defl.h"
#include "mg.h"
#include "ku.cuh"
#include "precond.h"

using namespace amk;

namespace {

thread_local std::string g_last_error;

am_status fail(am_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

}  // namespace

void amk::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

namespace {

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            return fail(e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,         \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
        }                                                                                   \
    } while (0)

#define CKS(expr)                        \
    do {                                 \
        am_status s_ = (expr);           \
        if (s_ != AM_OK) return s_;      \
    } while (0)

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device array of n elements at p, zero-filled, with `pad` zero elements of
// slack before and after it (vectors read by the unpredicated K*u kernel).
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    T *base = nullptr;
    size_t pad = 0;
    cudaError_t alloc(size_t count, size_t slack = 0) {
        if (p && n >= count && pad >= slack) return cudaSuccess;
        release();
        const size_t total = std::max<size_t>(count + 2 * slack, 1);
        cudaError_t e = cudaMalloc(&base, total * sizeof(T));
        if (e == cudaSuccess) {
            p = base + slack;
            n = count;
            pad = slack;
            e = cudaMemset(base, 0, total * sizeof(T));
        } else {
            base = nullptr;
        }
        return e;
    }
    void release() {
        if (base) cudaFree(base);
        p = base = nullptr;
        n = pad = 0;
    }
};

struct LoadCaseDev {
    DevBuf<double> F;           // device layout [3][cs]
    DevBuf<uint8_t> fixed_bits; // per node
    DevBuf<long long> f_idx;    // nonzero entries of F (device index) for u.F
    DevBuf<double> f_val;
    int f_nnz = 0;
    double bnorm2_all = 0.0;    // ||F||^2 over all DOFs (free-DOF norm is computed per solve)
    DevBuf<double> x64;         // warm-start displacement (device layout)
    bool have_x = false;
};

}  // namespace

struct am_problem {
    int nx, ny, nz;
    double h, E0, nu;
    Layout L;
    long long nn_ref;   // (nx+1)(ny+1)(nz+1)
    long long N;        // 3 nn_ref
    int device = 0;
    cudaStream_t st = nullptr;
    double ke00 = 0.0;  // KE[0][0] of the unit-modulus element (all diagonal entries equal)
    Modal<double> M64;
    Modal<float> M32;
    KuLaunch plan32, plan64;
    KuLaunch plan3;           // TMA-staged FP32 PCG K*u (ku3): 7- or 8-warp tiles
    int ku3_stages = 4;
    // the solver's K*u: 0 = ku3_kernel (tensor-store output tiles, ku3_stages
    // stages; the faster on GB300), 1 = ku3b_kernel (no CTA barrier per plane)
    int ku3_variant = 0;
    Ku3Maps *maps3 = nullptr;  // tensor maps of the FP32 PCG vectors (built on first use)
    bool pad_dirty = true;     // scales or constraint bits changed since the padded copies were made
    int nblocks_vec = 0;

    std::vector<int8_t> grid_host;  // internal layout, empty = all design
    DevBuf<int8_t> grid;

    std::vector<LoadCaseDev> cases;

    // element arrays
    DevBuf<double> rho, rho_new, rho_f, s64, ce, dc, dcf, estage;
    DevBuf<float> s32;
    DevBuf<double> oc_a64, oc_lo64, oc_hi64;  // OC terms (FP64 mode)
    DevBuf<float2> oc_a32, oc_lo32, oc_hi32;  // OC terms (double-float, mixed mode)
    DevBuf<uint8_t> design;
    // node arrays
    DevBuf<double> dinv64;
    DevBuf<float> dinv32;
    DevBuf<uint8_t> mask, nofix;
    // padded copies read by the ku3 tensor maps: element scales (rows of
    // round_up(nx, 4)) and constraint bits (rows of round_up(nx+1, 16))
    DevBuf<float> s32pad;
    DevBuf<uint8_t> maskpad;
    // vectors
    DevBuf<double> r64, xw64, p64a, p64b, q64v, vstage;
    DevBuf<float> x32, r32, p32a, p32b, q32v;
    DevBuf<double> xi64;  // FP64 result z of an FP32 inner PCG (for the flexible CG)
    // the inner PCG's iterate during the solve: the double-float pair x32 + xl32
    DevBuf<float> xl32;
    DevBuf<double> partial;
    Scalars *S = nullptr;    // device
    Scalars *Sh = nullptr;   // pinned host mirror
    // filter taps
    DevBuf<int4> tap_d;
    DevBuf<double> tap_w;
    int ntaps = 0;
    double taps_r = -1.0;
    int taps_variant = -1;
    // CUDA graphs of PCG chunks (host-driven loop) and of whole inner solves
    // (device-side while loop over chunks)
    cudaGraphExec_t g32 = nullptr, g64 = nullptr, gl32 = nullptr, gl64 = nullptr;
    int chunk = 32;
    bool device_loop = true;
    bool resid_df = true;  // mixed solvers: residuals in double-float (false: FP64 kernel)

    // SIMP state
    bool simp_begun = false;
    am_precond *pre = nullptr;       // learned preconditioner (AM_PRECOND_LEARNED)
    // multigrid preconditioner (AM_PRECOND_MG): built on first use; nullptr if
    // the grid does not coarsen far enough
    Mg *mg = nullptr;
    bool mg_tried = false;
    bool mg_dirty = true;  // operator or constraints changed since the last set-up
    int mg_lc = -1;        // load case whose fixed DOFs the coarse levels carry
    // rigid-body deflation of the passive solid inclusions around the V-cycle:
    // built on first use after the design mask is known; nullptr if there is none
    Defl *defl = nullptr;
    bool defl_tried = false;
    bool defl_set = false;  // set up for the current operator and load case
    const double *rho_op = nullptr;  // element densities of the current operator
    am_simp_config cfg{};
    double n_design = 0.0;
    int iter = 0;
    // self-test only: the next PCG run starts with Scalars::kerr set, as if a
    // kernel's bounded copy wait had run out (am_selftest_solve_timeout)
    bool inject_kerr = false;
};

namespace {

am_status sync_scalars(am_problem *P) {
    CK(cudaMemcpyAsync(P->Sh, P->S, sizeof(Scalars), cudaMemcpyDeviceToHost, P->st));
    CK(cudaStreamSynchronize(P->st));
    return AM_OK;
}

am_status ensure_vectors(am_problem *P, bool fp64) {
    const size_t nv = 3 * (size_t)P->L.cs;
    CK(P->r64.alloc(nv));
    CK(P->xw64.alloc(nv));
    CK(P->vstage.alloc(std::max<size_t>(nv, (size_t)P->N)));
    CK(P->dinv64.alloc(P->L.cs));
    const size_t slack = (size_t)ku2_slack(P->L);  // PCG vectors of the unpredicated K*u
    CK(P->dinv32.alloc(P->L.cs, slack));
    CK(P->mask.alloc(P->L.cs));
    CK(P->nofix.alloc(P->L.cs));
    if (fp64) {
        CK(P->p64a.alloc(nv));
        CK(P->p64b.alloc(nv));
        CK(P->q64v.alloc(nv));
    } else {
        CK(P->x32.alloc(nv));
        CK(P->xl32.alloc(nv));
        CK(P->xi64.alloc(nv));
        CK(P->r32.alloc(nv, slack));
        CK(P->p32a.alloc(nv, slack));
        CK(P->p32b.alloc(nv, slack));
        CK(P->q32v.alloc(nv));
        long long se = 0, mb = 0;
        ku3_padded_sizes(P->L, &se, &mb);
        CK(P->s32pad.alloc((size_t)se));
        CK(P->maskpad.alloc((size_t)mb));
    }
    // the staged K*u's partials for either tile height (am_problem_set_ku_plan)
    const size_t np = 3 * (size_t)std::max({P->plan32.ntiles(), P->plan64.ntiles(), ku3_plan(P->L, 7).ntiles(),
                                            ku3_plan(P->L, 8).ntiles(), P->nblocks_vec, 152 * 16});
    CK(P->partial.alloc(np));
    return AM_OK;
}

am_status ensure_elements(am_problem *P) {
    const size_t ne = (size_t)P->L.nel;
    CK(P->rho.alloc(ne));
    CK(P->rho_new.alloc(ne));
    CK(P->rho_f.alloc(ne));
    CK(P->s64.alloc(ne));
    CK(P->s32.alloc(ne));
    CK(P->ce.alloc(ne));
    CK(P->dc.alloc(ne));
    CK(P->dcf.alloc(ne));
    CK(P->design.alloc(ne));
    CK(P->estage.alloc(ne));
    return AM_OK;
}

// Uploads a host element array (host layout) into dst (internal layout).
am_status upload_elem(am_problem *P, const double *host, double *dst, int layout) {
    CK(cudaMemcpyAsync(P->estage.p, host, sizeof(double) * P->L.nel, cudaMemcpyHostToDevice, P->st));
    CK(elem_to_dev<double>(P->L, P->estage.p, dst, layout, P->st));
    return AM_OK;
}
am_status download_elem(am_problem *P, const double *src, double *host, int layout) {
    CK(elem_from_dev<double>(P->L, src, P->estage.p, layout, P->st));
    CK(cudaMemcpyAsync(host, P->estage.p, sizeof(double) * P->L.nel, cudaMemcpyDeviceToHost, P->st));
    CK(cudaStreamSynchronize(P->st));
    return AM_OK;
}

am_status build_taps(am_problem *P, double r, int variant) {
    if (P->taps_r == r && P->taps_variant == variant) return AM_OK;
    if (!(r > 0.0) || r > 6.0) return fail(AM_ERR_INVALID_ARG, "filter_radius must be in (0, 6]");
    std::vector<int4> d;
    std::vector<double> w;
    filter_taps(r, variant, d, w);
    CK(P->tap_d.alloc(d.size()));
    CK(P->tap_w.alloc(w.size()));
    CK(cudaMemcpyAsync(P->tap_d.p, d.data(), d.size() * sizeof(int4), cudaMemcpyHostToDevice, P->st));
    CK(cudaMemcpyAsync(P->tap_w.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, P->st));
    CK(cudaStreamSynchronize(P->st));
    P->ntaps = (int)d.size();
    P->taps_r = r;
    P->taps_variant = variant;
    return AM_OK;
}

Taps taps_of(am_problem *P) { return Taps{P->tap_d.p, P->tap_w.p, P->ntaps, (int)std::ceil(P->taps_r)}; }

// Element scales + Jacobi diagonal for the density currently in `rho_dev`.
am_status setup_operator(am_problem *P, const am_simp_config &c, const double *rho_dev) {
    P->rho_op = rho_dev;
    const int variant = c.variant;
    const int8_t *g = (variant == AM_VARIANT_PY && !P->grid_host.empty()) ? P->grid.p : nullptr;
    const int d1 = (variant == AM_VARIANT_CPP && c.cpp_assembly_index) ? 1 : 0;
    CK(scales(P->L, rho_dev, g, variant, c.penalty, c.E_min, c.rho_min, P->E0, P->s64.p, P->s32.p, P->st, d1));
    P->pad_dirty = true;
    P->mg_dirty = true;
    return AM_OK;
}

am_status setup_mask(am_problem *P, int lc) {
    const uint8_t *fb = (lc >= 0 && lc < (int)P->cases.size()) ? P->cases[lc].fixed_bits.p : nullptr;
    CK(diag_mask(P->L, P->s64.p, P->ke00, fb, P->dinv64.p, P->dinv32.p, P->mask.p, P->st));
    P->pad_dirty = true;
    P->mg_dirty = true;
    return AM_OK;
}

// The ku3 K*u reads its inputs through tensor maps: builds them once (the FP32
// vectors keep their addresses for the problem's lifetime) and refreshes the
// padded scale and constraint-bit copies after the operator or mask changed.
am_status ku3_ready(am_problem *P) {
    if (!P->maps3) {
        cudaError_t e = cudaSuccess;
        P->maps3 = ku3_make_maps(P->L, P->r32.p, P->p32a.p, P->p32b.p, P->dinv32.p, P->maskpad.p, P->s32pad.p,
                                 P->q32v.p, P->plan3.warps, &e);
        if (!P->maps3) return fail(AM_ERR_CUDA, std::string("tensor maps of the PCG vectors: ") + cudaGetErrorString(e));
    }
    if (P->pad_dirty) {
        CK(ku3_pad(P->L, P->s32.p, P->mask.p, P->s32pad.p, P->maskpad.p, P->st));
        P->pad_dirty = false;
    }
    return AM_OK;
}

// one FP32 PCG K*u step: p = D^-1 r + beta p_prev, q = mask(K p), p.q -> alpha
cudaError_t pcg_ku32(am_problem *P) {
    if (P->ku3_variant == 1)
        return ku3b_pcg(P->maps3, P->plan3, P->L, P->M32, P->q32v.p, P->p32a.p, P->p32b.p, P->partial.p, P->S, 5,
                        P->st);
    return ku3_pcg(P->maps3, P->plan3, P->L, P->M32, P->partial.p, P->S, P->ku3_stages, P->st);
}

// r = mask(f - K x) (+ element energies into ce): the residual replacements and
// the acceptance test of the mixed-precision solvers.  Double-float on the FP32
// pipes by default (kudf.cuh); the FP64 kernel when `native` (FP64 precision) or
// the problem's residual arithmetic is set to FP64.
cudaError_t solver_resid(am_problem *P, bool native, const double *x, const double *f, double *ce) {
    if (P->resid_df && !native)
        return ku_resid_df(P->plan64, P->L, P->M64, P->s64.p, x, f, P->dinv64.p, P->mask.p, P->r64.p, ce,
                           P->partial.p, P->S, P->st);
    return ku_resid(P->plan64, P->L, P->M64, P->s64.p, x, f, P->dinv64.p, P->mask.p, P->r64.p, ce, P->partial.p,
                    P->S, P->st);
}

// ||F||^2 over the free DOFs of case lc (mask already built)
am_status free_rhs_norm(am_problem *P, int lc, double *bnorm2) {
    const LoadCaseDev &C = P->cases[lc];
    CK(masked_sqnorm(C.f_idx.p, C.f_val.p, C.f_nnz, P->L.cs, P->mask.p, &P->S->res_rr, P->st));
    CKS(sync_scalars(P));
    *bnorm2 = P->Sh->res_rr;
    return AM_OK;
}

// The device-side loop of an inner solve: a CUDA-graph while node whose body is
// one chunk of PCG iterations followed by pcg_loop_next_kernel, which keeps the
// loop going while the solve runs and fewer than maxit / chunk + 4 chunks have run
// (every chunk either advances the iteration count or ends the solve, so the cap
// only catches a state that stops advancing).  pcg_loop_reset_kernel, upstream of
// the while node, zeroes the chunk count and opens the loop unless the solve has
// already ended.
__global__ void pcg_loop_reset_kernel(cudaGraphConditionalHandle h, Scalars *S) {
    S->loops = 0;
    cudaGraphSetConditional(h, S->done ? 0u : 1u);
}
__global__ void pcg_loop_next_kernel(cudaGraphConditionalHandle h, Scalars *S, int chunk) {
    const int n = ++S->loops;
    const int cap = S->maxit / chunk + 4;
    cudaGraphSetConditional(h, (!S->done && n < cap) ? 1u : 0u);
}

// captures one chunk of PCG iterations into the stream's capture
template <typename T>
cudaError_t capture_pcg_chunk(am_problem *P) {
    const KuLaunch &K = std::is_same<T, float>::value ? P->plan32 : P->plan64;
    double *x = nullptr;
    T *r, *pa, *pb, *q;
    const T *dinv, *s;
    Modal<T> M;
    if constexpr (std::is_same<T, float>::value) {
        r = P->r32.p; pa = P->p32a.p; pb = P->p32b.p; q = P->q32v.p;
        dinv = P->dinv32.p; s = P->s32.p; M = P->M32;
    } else {
        x = P->xw64.p; r = P->r64.p; pa = P->p64a.p; pb = P->p64b.p; q = P->q64v.p;
        dinv = P->dinv64.p; s = P->s64.p; M = P->M64;
    }
    for (int k = 0; k < P->chunk; ++k) {
        // the p ping-pong member is chosen on the device from the parity of S->it
        cudaError_t e;
        if constexpr (std::is_same<T, float>::value) {
            e = pcg_ku32(P);
            if (e == cudaSuccess)
                e = pcg_update_df(P->L, P->x32.p, P->xl32.p, r, pa, pb, q, dinv, P->partial.p, P->S, P->st);
        } else {
            e = ku_pcg<T>(K, P->L, M, s, pa, pb, r, dinv, P->mask.p, q, P->partial.p, P->S, P->st);
            if (e == cudaSuccess)
                e = pcg_update<T>(P->L, x, r, pa, pb, q, dinv, P->partial.p, P->S, P->nblocks_vec, P->st);
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T>
am_status build_pcg_loop_graph(am_problem *P, cudaGraphExec_t *out) {
    const long long launches_before = launch_count();
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    auto bail = [&](cudaError_t e, const char *what) {
        cudaGraphDestroy(g);
        return fail(AM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return bail(e, "PCG loop handle");
    e = cudaStreamBeginCaptureToGraph(P->st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bail(e, "PCG loop capture");
    pcg_loop_reset_kernel<<<1, 1, 0, P->st>>>(h, P->S);
    e = cudaGetLastError();
    cudaGraph_t gc = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(P->st, &gc);
    if (e != cudaSuccess || e2 != cudaSuccess) return bail(e != cudaSuccess ? e : e2, "PCG loop capture");
    cudaGraphNode_t reset = nullptr;
    size_t nn = 1;
    e = cudaGraphGetNodes(g, &reset, &nn);
    if (e != cudaSuccess || nn != 1) return bail(e != cudaSuccess ? e : cudaErrorUnknown, "PCG loop reset node");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond = nullptr;
    e = cudaGraphAddNode(&cond, g, &reset, nullptr, 1, &cp);
    if (e != cudaSuccess) return bail(e, "PCG loop node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(P->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bail(e, "PCG loop body capture");
    e = capture_pcg_chunk<T>(P);
    if (e == cudaSuccess) {
        pcg_loop_next_kernel<<<1, 1, 0, P->st>>>(h, P->S, P->chunk);
        e = cudaGetLastError();
    }
    cudaGraph_t gb = nullptr;
    const cudaError_t e3 = cudaStreamEndCapture(P->st, &gb);
    if (e != cudaSuccess || e3 != cudaSuccess) return bail(e != cudaSuccess ? e : e3, "PCG loop body capture");
    count_launches(launches_before - launch_count());  // captured, not executed
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(AM_ERR_CUDA, std::string("PCG loop instantiate: ") + cudaGetErrorString(e));
    return AM_OK;
}

template <typename T>
am_status build_pcg_graph(am_problem *P, cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    const long long launches_before = launch_count();
    CK(cudaStreamBeginCapture(P->st, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e1 = capture_pcg_chunk<T>(P);
    const cudaError_t e2 = cudaStreamEndCapture(P->st, &g);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(AM_ERR_CUDA, std::string("PCG capture: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    }
    count_launches(launches_before - launch_count());  // captured, not executed
    cudaError_t e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(AM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return AM_OK;
}

// Runs PCG chunks until S->done.  Returns the iteration count in *its.
template <typename T>
am_status run_pcg(am_problem *P, int *its, int *status) {
    cudaGraphExec_t *gx = std::is_same<T, float>::value ? &P->g32 : &P->g64;
    if constexpr (std::is_same<T, float>::value) CKS(ku3_ready(P));
    if (!P->device_loop && !*gx) CKS(build_pcg_graph<T>(P, gx));
    if (P->inject_kerr) {
        static const int kOne = 1;
        P->inject_kerr = false;
        CK(cudaMemcpyAsync(&P->S->kerr, &kOne, sizeof(int), cudaMemcpyHostToDevice, P->st));
    }
    if (P->device_loop) {
        // the whole inner solve in one graph launch, the loop decided on the device
        cudaGraphExec_t *gl = std::is_same<T, float>::value ? &P->gl32 : &P->gl64;
        if (!*gl) CKS(build_pcg_loop_graph<T>(P, gl));
        CK(cudaGraphLaunch(*gl, P->st));
        CKS(sync_scalars(P));
        count_launches(1 + (2LL * P->chunk + 1) * P->Sh->loops);
        if (!P->Sh->done) return fail(AM_ERR_TIMEOUT, "PCG did not terminate within its iteration cap");
    } else {
        CKS(sync_scalars(P));
        // every chunk either advances the iteration count or ends the solve; the
        // host bound below only catches a solver state that stops advancing
        const long long max_chunks = (long long)P->Sh->maxit / P->chunk + 4;
        long long chunks = 0;
        while (!P->Sh->done) {
            if (++chunks > max_chunks) return fail(AM_ERR_TIMEOUT, "PCG did not terminate within its iteration cap");
            CK(cudaGraphLaunch(*gx, P->st));
            count_launches(2LL * P->chunk);
            CKS(sync_scalars(P));
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        // the iterate folds every second iteration: pay the term a solve that
        // stopped after an even iteration still owes
        if (P->Sh->it & 1)
            CK(pcg_df_settle(3 * P->L.cs, P->x32.p, P->xl32.p, P->p32a.p, P->p32b.p, P->S, P->nblocks_vec, P->st));
    }
    *its = P->Sh->it;
    *status = P->Sh->status;
    if (P->Sh->status == ST_TIMEOUT) return fail(AM_ERR_TIMEOUT, "a bulk-copy wait of the PCG timed out");
    return AM_OK;
}

// The FP32 inner PCG iterates on the double-float pair (x32, xl32); these move
// it to and from the FP64 vector xi64 that the flexible CG uses.
am_status inner_iterate_zero(am_problem *P) {
    CK(cudaMemsetAsync(P->x32.p, 0, sizeof(float) * 3 * P->L.cs, P->st));
    CK(cudaMemsetAsync(P->xl32.p, 0, sizeof(float) * 3 * P->L.cs, P->st));
    return AM_OK;
}
am_status inner_iterate_to_fp64(am_problem *P) {
    CK(df_compose(P->x32.p, P->xl32.p, P->xi64.p, 3 * P->L.cs, P->nblocks_vec, P->st));
    return AM_OK;
}

// The multigrid hierarchy for the current operator and load case lc: true when
// it is ready, false when the grid does not coarsen far enough (the solve then
// uses the Jacobi path).
// Passive solid elements: CPP elements outside the design mask at density >= 0.99
// (their scale is rho^p = 1 for the whole run); PY and outside a SIMP run, grid == 1
// (scale 1 whatever the density, fem.py:175-248).
am_status passive_solid(am_problem *P, std::vector<uint8_t> &solid) {
    const size_t nel = (size_t)P->L.nel;
    solid.assign(nel, 0);
    if (P->simp_begun && P->cfg.variant == AM_VARIANT_CPP) {
        std::vector<uint8_t> dm(nel);
        std::vector<double> rho(nel);
        CK(cudaMemcpyAsync(dm.data(), P->design.p, nel, cudaMemcpyDeviceToHost, P->st));
        CK(cudaMemcpyAsync(rho.data(), P->rho.p, sizeof(double) * nel, cudaMemcpyDeviceToHost, P->st));
        CK(cudaStreamSynchronize(P->st));
        for (size_t e = 0; e < nel; ++e) solid[e] = !dm[e] && rho[e] >= 0.99;
    } else if (!P->grid_host.empty()) {
        for (size_t e = 0; e < nel; ++e) solid[e] = P->grid_host[e] == 1;
    }
    return AM_OK;
}

am_status mg_ready(am_problem *P, int lc, bool deflate, bool *ok) {
    *ok = false;
    if (!P->mg_tried) {
        P->mg_tried = true;
        cudaError_t e = cudaSuccess;
        P->mg = mg_create(P->L, P->E0, P->nu, P->h, &e);
        if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                                          std::string("multigrid levels: ") + cudaGetErrorString(e));
    }
    if (!P->mg) return AM_OK;
    if (P->mg_dirty || P->mg_lc != lc) {
        CKS(ensure_vectors(P, false));
        const cudaError_t e = mg_setup(P->mg, P->s64.p, P->s32.p, P->dinv32.p, P->mask.p, P->cases[lc].fixed_bits.p,
                                       P->st);
        if (e == cudaErrorInvalidValue) return fail(AM_ERR_SINGULAR, "multigrid coarsest matrix is not positive definite");
        CK(e);
        P->mg_dirty = false;
        P->mg_lc = lc;
        P->defl_set = false;
    }
    if (deflate && !P->defl_tried) {
        P->defl_tried = true;
        std::vector<uint8_t> solid;
        CKS(passive_solid(P, solid));
        cudaError_t e = cudaSuccess;
        P->defl = defl_create(P->L, solid.data(), &e);
        if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                                          std::string("deflation space: ") + cudaGetErrorString(e));
        P->defl_set = false;
    }
    if (deflate && P->defl && !P->defl_set) {
        CKS(ensure_vectors(P, true));
        CK(defl_setup(P->defl, P->plan64, P->M64, P->s64.p, P->mask.p, P->p64a.p, P->q64v.p, P->st));
        P->defl_set = true;
    }
    *ok = true;
    return AM_OK;
}

struct SolveOut {
    int iterations = 0, outer = 0, converged = 0, learned = 0;
    double residual = 0.0, time_s = 0.0;
};

// Solves K(s) u = F_lc on the free DOFs.  Operator (s64/s32, dinv, mask) must be
// set up.  Result in P->cases[lc].x64; ce filled when want_ce.
am_status solve_case(am_problem *P, const am_simp_config &c, int lc, bool want_ce, SolveOut &o) {
    const double t0 = now_s();
    LoadCaseDev &C = P->cases[lc];
    const bool fp64 = c.precision == AM_PREC_FP64;
    CKS(ensure_vectors(P, fp64));
    CK(C.x64.alloc(3 * (size_t)P->L.cs));
    if (!c.warm_start || !C.have_x) CK(cudaMemsetAsync(C.x64.p, 0, sizeof(double) * 3 * P->L.cs, P->st));
    else CK(zero_masked(P->L, P->mask.p, C.x64.p, P->nblocks_vec, P->st));  // DOFs orphaned since the last solve
    C.have_x = true;
    double bnorm2 = 0.0;
    CKS(free_rhs_norm(P, lc, &bnorm2));
    o = SolveOut{};
    if (!(bnorm2 > 0.0)) {
        // rhs is zero on the free DOFs: u = 0 (Eigen returns x = 0 for b = 0)
        CK(cudaMemsetAsync(C.x64.p, 0, sizeof(double) * 3 * P->L.cs, P->st));
        if (want_ce) CK(cudaMemsetAsync(P->ce.p, 0, sizeof(double) * P->L.nel, P->st));
        o.converged = 1;
        o.time_s = now_s() - t0;
        return AM_OK;
    }
    const double tol = c.cg_tol;
    const int maxit = c.cg_max_iterations > 0 ? c.cg_max_iterations : 100000;
    const bool learned0 = c.preconditioner == AM_PRECOND_LEARNED && P->pre;
    bool mg0 = false;
    if (c.preconditioner == AM_PRECOND_MG) CKS(mg_ready(P, lc, c.mg_deflation != 0, &mg0));
    Defl *defl = (mg0 && c.mg_deflation) ? P->defl : nullptr;
    if (fp64 && !learned0 && !mg0) {
        CK(cudaMemcpyAsync(P->xw64.p, C.x64.p, sizeof(double) * 3 * P->L.cs, cudaMemcpyDeviceToDevice, P->st));
        CK(ku_resid(P->plan64, P->L, P->M64, P->s64.p, P->xw64.p, C.F.p, P->dinv64.p, P->mask.p,
                    P->r64.p, nullptr, P->partial.p, P->S, P->st));
        CK(pcg_start<double>(P->L, P->r64.p, P->dinv64.p, tol * tol * bnorm2, 0.0, maxit, 0, P->partial.p, P->S,
                             P->nblocks_vec, P->st));
        int its = 0, stt = 0;
        CKS(run_pcg<double>(P, &its, &stt));
        CK(cudaMemcpyAsync(C.x64.p, P->xw64.p, sizeof(double) * 3 * P->L.cs, cudaMemcpyDeviceToDevice, P->st));
        // true FP64 residual (+ element energies) at the accepted solution
        CK(ku_resid(P->plan64, P->L, P->M64, P->s64.p, C.x64.p, C.F.p, P->dinv64.p, P->mask.p, P->r64.p,
                    want_ce ? P->ce.p : nullptr, P->partial.p, P->S, P->st));
        CKS(sync_scalars(P));
        o.iterations = its;
        o.outer = 1;
        o.residual = std::sqrt(P->Sh->res_rr / bnorm2);
        o.converged = (stt == ST_CONVERGED) ? 1 : 0;
        if (stt == ST_NAN) return fail(AM_ERR_NAN_DETECTED, "NaN in the PCG iteration");
    } else if (!learned0 && !mg0 && c.mixed_solver == AM_MIXED_RELIABLE) {
        // Mixed precision, one FP32 Jacobi-PCG sequence with reliable updates
        // (residual replacement, van der Vorst and Ye): the FP32 iteration runs
        // until its recursive residual has fallen by inner_tol; then the
        // double-float iterate is added to the FP64 displacement, the residual is
        // recomputed in FP64 and replaces the recursive one, and the sequence
        // continues along its last search direction (beta from the replaced
        // residual) instead of restarting, so the Krylov space built so far is kept.
        // The solve is accepted on the recomputed FP64 residual.
        CKS(ensure_vectors(P, true));
        const int max_rounds = c.max_outer > 0 ? c.max_outer : 200;
        const double red = (c.inner_tol > 0.0 && c.inner_tol < 1.0) ? c.inner_tol : 0.1;
        CK(solver_resid(P, fp64, C.x64.p, C.F.p, want_ce ? P->ce.p : nullptr));
        CKS(sync_scalars(P));
        double rel = std::sqrt(P->Sh->res_rr / bnorm2);
        int total = 0, rounds = 0, restart = 0, stt = ST_RUNNING;
        bool nan = !std::isfinite(rel);
        while (!nan && rel > tol && rounds < max_rounds && total < maxit) {
            CK(dc_inner_init(P->L, P->r64.p, P->r32.p, nullptr, P->S, P->nblocks_vec, P->st));
            CKS(inner_iterate_zero(P));
            // stop the FP32 sequence at half the goal (the recursive residual runs
            // ahead of the true one) or after a reduction by inner_tol
            CK(pcg_start<float>(P->L, P->r32.p, P->dinv32.p, 0.25 * tol * tol * bnorm2, red * red,
                                maxit, restart, P->partial.p, P->S, P->nblocks_vec, P->st));
            int its = 0;
            CKS(run_pcg<float>(P, &its, &stt));
            total = its;  // S->it runs on across replacements
            ++rounds;
            if (stt == ST_NAN) {
                nan = true;
                break;
            }
            CK(df_accumulate(P->x32.p, P->xl32.p, C.x64.p, 3 * P->L.cs, P->nblocks_vec, P->st));
            CK(solver_resid(P, fp64, C.x64.p, C.F.p, want_ce ? P->ce.p : nullptr));
            CKS(sync_scalars(P));
            rel = std::sqrt(P->Sh->res_rr / bnorm2);
            nan = !std::isfinite(rel);
            if (c.verbose >= 2)
                std::printf("  round %d: PCG iterations %d, status %d, rel-res %.3e\n", rounds, total, stt, rel);
            if (stt == ST_MAXIT) break;
            // continue the sequence along p (residual replacement); after a
            // breakdown take a fresh direction from the replaced residual
            restart = (stt == ST_BREAKDOWN) ? 2 : 1;
        }
        if (nan) return fail(AM_ERR_NAN_DETECTED, "NaN in the mixed-precision solve");
        o.iterations = total;
        o.outer = rounds;
        o.residual = rel;
        o.converged = rel <= tol ? 1 : 0;
    } else {
        // Mixed precision: flexible CG in FP64 (FP64 K*u, vectors and dot
        // products, so the accepted iterate has the energy-norm quality of FP64 CG
        // at the same residual) preconditioned by an FP32 Jacobi-PCG inner solve
        // z = M(r) that reduces its residual by inner_tol (or stops at its cap).
        CKS(ensure_vectors(P, false));
        CKS(ensure_vectors(P, true));
        // learned preconditioner: the network's z starts each inner Jacobi-PCG
        // solve; if the outer residual stops falling (< 10 % over 5 outer
        // iterations) the solve continues with Jacobi PCG alone
        bool learned = learned0;
        // multigrid likewise: a V-cycle whose coarse grids do not represent the
        // operator (rediscretisation of a rough density field) stops helping; the
        // solve then continues with Jacobi-PCG inner solves
        bool mg_on = mg0;
        // with the V-cycle the outer product K p runs in FP32 until the FP32
        // rounding of K p stalls the residual (near 1e-7 relative), then in FP64
        bool mg_f32 = mg0;
        std::vector<double> hist;
        const int max_outer = c.max_outer > 0 ? c.max_outer : 200;
        const double inner_red = (c.inner_tol > 0.0 && c.inner_tol < 1.0) ? c.inner_tol : 0.01;
        const int inner_cap = std::max(50, maxit / 4);
        CK(cudaMemsetAsync(&P->S->o_status, 0, sizeof(int), P->st));
        CK(solver_resid(P, fp64, C.x64.p, C.F.p, want_ce ? P->ce.p : nullptr));
        CKS(sync_scalars(P));
        double rel = std::sqrt(P->Sh->res_rr / bnorm2);
        int total = 0, outer = 0;
        bool nan = !std::isfinite(rel);
        while (!nan && rel > tol && outer < max_outer && total < maxit) {
            int its = 0;
            if (learned) {
                // z = M(r) from the network, refined by FP32 Jacobi PCG on the
                // residual it leaves (r - K z) to the same inner tolerance
                const PrecondView view{P->L, P->dinv32.p, P->mask.p, P->rho_op, P->st};
                CKS(precond_apply(P->pre, view, P->r64.p, P->xi64.p));
                if (!(c.inner_tol >= 1.0)) {  // inner_tol >= 1: the network alone
                    CK(df_split(P->xi64.p, P->x32.p, P->xl32.p, 3 * P->L.cs, P->nblocks_vec, P->st));
                    CK(ku_plain<float>(P->plan32, P->L, P->M32, P->s32.p, P->x32.p, P->q32v.p, P->st));
                    CK(inner_resid(P->L, P->r64.p, P->q32v.p, P->mask.p, P->r32.p, P->nblocks_vec, P->st));
                    const double tgt = std::max(inner_red * rel, 0.3 * tol);
                    const double thr = tgt * tgt * bnorm2;
                    CK(pcg_start<float>(P->L, P->r32.p, P->dinv32.p, thr, 0.0, std::min(inner_cap, maxit - total),
                                        0, P->partial.p, P->S, P->nblocks_vec, P->st));
                    int stt = 0;
                    CKS(run_pcg<float>(P, &its, &stt));
                    if (stt == ST_NAN) {
                        nan = true;
                        break;
                    }
                    CKS(inner_iterate_to_fp64(P));
                    total += its;
                }
            } else if (mg_on) {
                // z = M(r): one FP32 multigrid V-cycle, balanced by the rigid-body
                // modes of the passive solid inclusions when there are any
                if (defl) CK(defl_apply(defl, P->mg, P->r64.p, P->xi64.p, P->st));
                else CK(mg_apply(P->mg, P->r64.p, P->xi64.p, P->st));
                its = 1;
                total += its;
            } else {
                // z = M(r): FP32 PCG (FP64 iterate) on K z = r from zero, to
                // inner_tol of |r| but not below 0.3 tol |f| (the overall goal)
                CK(dc_inner_init(P->L, P->r64.p, P->r32.p, nullptr, P->S, P->nblocks_vec, P->st));
                CKS(inner_iterate_zero(P));
                const double tgt = std::max(inner_red * rel, 0.3 * tol);
                CK(pcg_start<float>(P->L, P->r32.p, P->dinv32.p, tgt * tgt * bnorm2, 0.0,
                                    std::min(inner_cap, maxit - total), 0, P->partial.p, P->S, P->nblocks_vec,
                                    P->st));
                int stt = 0;
                CKS(run_pcg<float>(P, &its, &stt));
                if (stt == ST_NAN) {
                    nan = true;
                    break;
                }
                CKS(inner_iterate_to_fp64(P));
                total += its;
            }
            // outer step
            CK(fcg_dots(P->L, P->xi64.p, P->r64.p, P->q64v.p, outer == 0 ? 1 : 0, P->partial.p, P->S,
                        P->nblocks_vec, P->st));
            CK(fcg_direction(P->L, P->xi64.p, P->p64a.p, P->S, P->nblocks_vec, P->st));
            if (mg_on && mg_f32)  // the V-cycle is FP32: its outer product need not be FP64 either
                CK(ku_dot_f32(P->plan32, P->L, P->M32, P->s32.p, P->p64a.p, P->mask.p, P->x32.p, P->q32v.p,
                              P->q64v.p, P->partial.p, P->S, P->nblocks_vec, P->st));
            else if (P->resid_df && !fp64)  // the FP64-accurate outer product in double-float
                CK(ku_dot_df(P->plan64, P->L, P->M64, P->s64.p, P->p64a.p, P->mask.p, P->q64v.p, P->partial.p,
                             P->S, P->st));
            else
                CK(ku_dot(P->plan64, P->L, P->M64, P->s64.p, P->p64a.p, P->mask.p, P->q64v.p, P->partial.p, P->S,
                          P->st));
            CK(fcg_update(P->L, C.x64.p, P->r64.p, P->p64a.p, P->q64v.p, P->partial.p, P->S, P->nblocks_vec,
                          P->st));
            CKS(sync_scalars(P));
            ++outer;
            if (P->Sh->o_status == ST_NAN || !std::isfinite(P->Sh->o_rr)) {
                nan = true;
                break;
            }
            rel = std::sqrt(P->Sh->o_rr / bnorm2);
            if (c.verbose >= 2)
                std::printf("  outer %d: %s %d (total %d) rel-res %.3e\n", outer,
                            learned  ? "learned"
                            : mg_on ? (mg_f32 ? "v-cycle, fp32 K p" : "v-cycle, fp64 K p")
                                     : "inner",
                            its, total, rel);
            if (learned) {
                ++o.learned;
                hist.push_back(rel);
                if (hist.size() > 5 && rel > 0.9 * hist[hist.size() - 6]) learned = false;  // Jacobi from here
            } else if (mg_on) {
                hist.push_back(rel);
                if (hist.size() > 5 && rel > 0.9 * hist[hist.size() - 6]) {
                    if (mg_f32)
                        mg_f32 = false;  // FP64 outer product from here
                    else
                        mg_on = false;  // Jacobi from here
                    hist.clear();
                }
            }
            if (rel <= tol) {
                // accept on the recomputed FP64 residual (and element energies)
                CK(solver_resid(P, fp64, C.x64.p, C.F.p, want_ce ? P->ce.p : nullptr));
                CKS(sync_scalars(P));
                rel = std::sqrt(P->Sh->res_rr / bnorm2);
            }
        }
        if (nan) return fail(AM_ERR_NAN_DETECTED, "NaN in the mixed-precision solve");
        if (want_ce && rel > tol) {
            // not converged: element energies of the returned iterate
            CK(solver_resid(P, fp64, C.x64.p, C.F.p, P->ce.p));
            CKS(sync_scalars(P));
            rel = std::sqrt(P->Sh->res_rr / bnorm2);
        }
        o.iterations = total;
        o.outer = outer;
        o.residual = rel;
        o.converged = rel <= tol ? 1 : 0;
    }
    o.time_s = now_s() - t0;
    return AM_OK;
}

// OC update of P->rho (design mask P->design / `design`) with filtered
// sensitivities `dcf` into P->rho_new; results in P->Sh after the sync.
am_status run_oc(am_problem *P, bool f64, int variant, double move, double rho_min, double vf, double n_design,
                 const double *rho, const double *dcf, const uint8_t *design, double *rho_new) {
    const size_t ne = (size_t)P->L.nel;
    if (f64) {
        CK(P->oc_a64.alloc(ne)); CK(P->oc_lo64.alloc(ne)); CK(P->oc_hi64.alloc(ne));
    } else {
        CK(P->oc_a32.alloc(ne)); CK(P->oc_lo32.alloc(ne)); CK(P->oc_hi32.alloc(ne));
    }
    OcBuffers B{P->L.nel, P->oc_a64.p, P->oc_lo64.p, P->oc_hi64.p, P->oc_a32.p, P->oc_lo32.p, P->oc_hi32.p};
    CK(oc_prepare(B, rho, dcf, move, f64, variant, P->S, P->st));
    for (int k = 0; k < 100; ++k)
        CK(oc_pass(B, design, f64, variant, rho_min, vf, n_design, P->partial.p, P->S, P->nblocks_vec, P->st));
    CK(oc_final(B, design, f64, variant, rho_min, rho, dcf, move, rho_new, P->partial.p, P->S, P->nblocks_vec,
                P->st));
    CKS(sync_scalars(P));
    return AM_OK;
}

am_status check_problem(am_problem *P) {
    if (!P) return fail(AM_ERR_INVALID_ARG, "null problem");
    CK(cudaSetDevice(P->device));
    return AM_OK;
}

am_status check_cfg(am_problem *P, const am_simp_config *c) {
    if (!c) return fail(AM_ERR_INVALID_ARG, "null config");
    if (c->variant != AM_VARIANT_CPP && c->variant != AM_VARIANT_PY)
        return fail(AM_ERR_INVALID_ARG, "unknown variant");
    if (c->precision != AM_PREC_FP64 && c->precision != AM_PREC_MIXED)
        return fail(AM_ERR_INVALID_ARG, "unknown precision");
    if (c->mixed_solver != AM_MIXED_RELIABLE && c->mixed_solver != AM_MIXED_FLEXIBLE)
        return fail(AM_ERR_INVALID_ARG, "unknown mixed_solver");
    if (c->layout != AM_LAYOUT_ZFASTEST && c->layout != AM_LAYOUT_XFASTEST)
        return fail(AM_ERR_INVALID_ARG, "unknown layout");
    if (c->preconditioner != AM_PRECOND_JACOBI && c->preconditioner != AM_PRECOND_LEARNED &&
        c->preconditioner != AM_PRECOND_MG)
        return fail(AM_ERR_INVALID_ARG, "unknown preconditioner");
    if (c->preconditioner == AM_PRECOND_LEARNED && !P->pre)
        return fail(AM_ERR_INVALID_ARG, "AM_PRECOND_LEARNED needs am_problem_set_preconditioner");
    if (!(c->volume_fraction > 0.0 && c->volume_fraction <= 1.0))
        return fail(AM_ERR_INVALID_ARG, "volume_fraction must be in (0, 1]");
    if (!(c->penalty >= 1.0) || !(c->move_limit > 0.0) || !(c->rho_min >= 0.0) || !(c->E_min >= 0.0))
        return fail(AM_ERR_INVALID_ARG, "need penalty >= 1, move_limit > 0, rho_min >= 0, E_min >= 0");
    if (!(c->cg_tol > 0.0)) return fail(AM_ERR_INVALID_ARG, "cg_tol must be > 0");
    (void)P;
    return AM_OK;
}

}  // namespace

// ============================================================================
// extern "C" ABI
// ============================================================================
extern "C" {

const char *am_status_string(am_status s) {
    switch (s) {
        case AM_OK: return "AM_OK";
        case AM_ERR_INVALID_ARG: return "AM_ERR_INVALID_ARG";
        case AM_ERR_SIZE_MISMATCH: return "AM_ERR_SIZE_MISMATCH";
        case AM_ERR_DOF_OUT_OF_RANGE: return "AM_ERR_DOF_OUT_OF_RANGE";
        case AM_ERR_NOT_CONVERGED: return "AM_ERR_NOT_CONVERGED";
        case AM_ERR_NAN_DETECTED: return "AM_ERR_NAN_DETECTED";
        case AM_ERR_SINGULAR: return "AM_ERR_SINGULAR";
        case AM_ERR_CUDA: return "AM_ERR_CUDA";
        case AM_ERR_TIMEOUT: return "AM_ERR_TIMEOUT";
        case AM_ERR_OOM: return "AM_ERR_OOM";
        case AM_ERR_NO_DEVICE: return "AM_ERR_NO_DEVICE";
    }
    return "AM_ERR_UNKNOWN";
}

const char *am_last_error(void) { return g_last_error.c_str(); }

int am_is_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n > 0;
}

am_status am_device_info(int *sm_count, size_t *free_bytes, size_t *total_bytes) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, dev));
    if (sm_count) *sm_count = prop.multiProcessorCount;
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return AM_OK;
}

void am_simp_config_default(am_simp_config *c, int variant) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->variant = variant;
    c->volume_fraction = 0.25;
    c->penalty = 3.0;
    c->filter_radius = 2.0;
    c->move_limit = 0.2;
    c->rho_min = 0.01;
    c->E_min = variant == AM_VARIANT_CPP ? 1e-6 : 1e-9;
    c->convergence_tol = 0.01;
    c->max_iterations = 100;
    c->precision = AM_PREC_MIXED;
    c->preconditioner = AM_PRECOND_JACOBI;
    c->cg_tol = 1e-6;
    c->cg_max_iterations = 100000;
    c->warm_start = 1;
    c->inner_tol = 0.0;  // the solver's own default: 0.1 (reliable updates), 0.01 (flexible CG)
    c->max_outer = 200;
    c->layout = AM_LAYOUT_ZFASTEST;
    c->verbose = 0;
    c->mg_deflation = 1;
}

am_status am_element_stiffness(double E, double nu, double h, double *ke) {
    if (!ke) return fail(AM_ERR_INVALID_ARG, "null output");
    if (!(h > 0.0) || !(E > 0.0) || !(nu > -1.0 && nu < 0.5))
        return fail(AM_ERR_INVALID_ARG, "need h > 0, E > 0, -1 < nu < 0.5");
    const Modal<double> M = modal_constants(E, nu, h);
    for (int col = 0; col < 24; ++col) {
        double u[3][8] = {}, y[3][8];
        u[col % 3][col / 3] = 1.0;
        hex8_apply<double>(u, y, M, 1.0, nullptr);
        for (int row = 0; row < 24; ++row) ke[row * 24 + col] = y[row % 3][row / 3];
    }
    return AM_OK;
}

am_status am_problem_create(int nx, int ny, int nz, double h, double E0, double nu,
                            const int8_t *grid, int layout, am_problem **out) {
    if (!out) return fail(AM_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (nx < 1 || ny < 1 || nz < 1) return fail(AM_ERR_INVALID_ARG, "grid dimensions must be >= 1");
    if (!(h > 0.0) || !(E0 > 0.0) || !(nu > -1.0 && nu < 0.5))
        return fail(AM_ERR_INVALID_ARG, "need h > 0, E0 > 0, -1 < nu < 0.5");
    if (layout != AM_LAYOUT_ZFASTEST && layout != AM_LAYOUT_XFASTEST)
        return fail(AM_ERR_INVALID_ARG, "unknown layout");
    if (!am_is_available()) return fail(AM_ERR_NO_DEVICE, "no CUDA device");
    am_problem *P = new am_problem();
    P->nx = nx; P->ny = ny; P->nz = nz;
    P->h = h; P->E0 = E0; P->nu = nu;
    cudaGetDevice(&P->device);
    Layout &L = P->L;
    L = make_layout(nx, ny, nz);
    P->nn_ref = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    P->N = 3 * P->nn_ref;
    // Lame parameters of the unit-modulus material; K scales linearly with E0
    // and the element scales carry E/E0, so the operator uses E = E0.
    P->M64 = modal_constants(E0, nu, h);
    const Modal<double> &M = P->M64;
    P->M32 = modal_float(M);
    // every diagonal entry of the cube KE equals KE[0][0]
    P->ke00 = element_stiffness_entry(M, 0, 0);
    P->plan32 = ku_plan(L, false, 0);
    P->plan64 = ku_plan(L, true, 0);
    P->plan3 = ku3_plan(L);
    P->nblocks_vec = (int)std::max<long long>(1, std::min<long long>((3 * L.cs + 255) / 256, 152LL * 8));
    cudaError_t e = ku_init_attributes();
    if (e == cudaSuccess) e = ku3_init_attributes();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&P->S, sizeof(Scalars));
    if (e == cudaSuccess) e = cudaMemset(P->S, 0, sizeof(Scalars));
    if (e == cudaSuccess) e = cudaMallocHost(&P->Sh, sizeof(Scalars));
    if (e != cudaSuccess) {
        am_problem_destroy(P);
        return fail(e == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,
                    std::string("problem create: ") + cudaGetErrorString(e));
    }
    if (grid) {
        std::vector<int8_t> g((size_t)L.nel);
        for (long long ez = 0; ez < nz; ++ez)
            for (long long ey = 0; ey < ny; ++ey)
                for (long long ex = 0; ex < nx; ++ex) {
                    const long long hidx = layout == AM_LAYOUT_ZFASTEST ? (ex * ny + ey) * nz + ez
                                                                        : (ez * ny + ey) * nx + ex;
                    const int8_t v = grid[hidx];
                    if (v < -1 || v > 1) {
                        am_problem_destroy(P);
                        return fail(AM_ERR_INVALID_ARG, "grid values must be -1, 0 or 1");
                    }
                    g[(size_t)((ez * ny + ey) * nx + ex)] = v;
                }
        P->grid_host = g;
        e = P->grid.alloc(g.size());
        if (e == cudaSuccess) e = cudaMemcpy(P->grid.p, g.data(), g.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            am_problem_destroy(P);
            return fail(AM_ERR_CUDA, std::string("grid upload: ") + cudaGetErrorString(e));
        }
    }
    *out = P;
    return AM_OK;
}

am_status am_problem_destroy(am_problem *P) {
    if (!P) return AM_OK;
    cudaSetDevice(P->device);
    if (P->st) cudaStreamSynchronize(P->st);
    for (cudaGraphExec_t g : {P->g32, P->g64, P->gl32, P->gl64})
        if (g) cudaGraphExecDestroy(g);
    for (auto &c : P->cases) {
        c.F.release(); c.fixed_bits.release(); c.f_idx.release(); c.f_val.release(); c.x64.release();
    }
    DevBuf<double> *d64[] = {&P->rho, &P->rho_new, &P->rho_f, &P->s64, &P->ce, &P->dc, &P->dcf, &P->oc_a64, &P->oc_lo64, &P->oc_hi64,
                             &P->estage, &P->dinv64, &P->r64, &P->xw64, &P->p64a, &P->p64b, &P->q64v,
                             &P->vstage, &P->partial, &P->tap_w};
    for (auto *b : d64) b->release();
    P->oc_a32.release(); P->oc_lo32.release(); P->oc_hi32.release();
    DevBuf<float> *d32[] = {&P->s32, &P->dinv32, &P->x32, &P->xl32, &P->r32, &P->p32a, &P->p32b, &P->q32v, &P->s32pad};
    P->maskpad.release();
    mg_destroy(P->mg);
    defl_destroy(P->defl);
    P->mg = nullptr;
    ku3_free_maps(P->maps3);
    P->maps3 = nullptr;
    P->xi64.release();
    for (auto *b : d32) b->release();
    P->design.release(); P->mask.release(); P->nofix.release(); P->grid.release(); P->tap_d.release();
    if (P->S) cudaFree(P->S);
    if (P->Sh) cudaFreeHost(P->Sh);
    if (P->st) cudaStreamDestroy(P->st);
    delete P;
    return AM_OK;
}

am_status am_problem_set_loads(am_problem *P, int n_cases, const double *F, const int64_t *fixed,
                               const int64_t *n_fixed) {
    CKS(check_problem(P));
    if (n_cases < 1 || !F) return fail(AM_ERR_INVALID_ARG, "need n_cases >= 1 and F");
    if (!n_fixed) return fail(AM_ERR_INVALID_ARG, "need n_fixed");
    for (auto &c : P->cases) {
        c.F.release(); c.fixed_bits.release(); c.f_idx.release(); c.f_val.release(); c.x64.release();
    }
    P->cases.clear();
    P->cases.resize(n_cases);
    const long long N = P->N;
    const Layout &L = P->L;
    long long off = 0;
    std::vector<uint8_t> bits((size_t)L.cs);
    CK(P->vstage.alloc(std::max<size_t>(3 * (size_t)L.cs, (size_t)N)));
    for (int c = 0; c < n_cases; ++c) {
        LoadCaseDev &C = P->cases[c];
        std::fill(bits.begin(), bits.end(), 0);
        for (long long t = 0; t < n_fixed[c]; ++t) {
            const long long d = fixed[off + t];
            if (d < 0 || d >= N) return fail(AM_ERR_DOF_OUT_OF_RANGE, "Fixed DOF index out of range: " + std::to_string(d));
            const long long n = d / 3;
            const int comp = (int)(d % 3);
            const int k = (int)(n % (P->nz + 1));
            const long long tt = n / (P->nz + 1);
            const int j = (int)(tt % (P->ny + 1)), i = (int)(tt / (P->ny + 1));
            bits[(size_t)node_index(L, i, j, k)] |= (uint8_t)(1u << comp);
        }
        off += n_fixed[c];
        const double *Fc = F + (size_t)c * N;
        std::vector<long long> idx;
        std::vector<double> val;
        double b2 = 0.0;
        for (long long d = 0; d < N; ++d) {
            const double v = Fc[d];
            if (!std::isfinite(v)) return fail(AM_ERR_NAN_DETECTED, "non-finite load entry");
            if (v != 0.0) {
                const long long n = d / 3;
                const int comp = (int)(d % 3);
                const int k = (int)(n % (P->nz + 1));
                const long long tt = n / (P->nz + 1);
                const int j = (int)(tt % (P->ny + 1)), i = (int)(tt / (P->ny + 1));
                idx.push_back(comp * L.cs + node_index(L, i, j, k));
                val.push_back(v);
                b2 += v * v;
            }
        }
        C.bnorm2_all = b2;
        CK(C.F.alloc(3 * (size_t)L.cs));
        CK(C.fixed_bits.alloc((size_t)L.cs));
        CK(cudaMemcpyAsync(C.fixed_bits.p, bits.data(), bits.size(), cudaMemcpyHostToDevice, P->st));
        CK(cudaMemcpyAsync(P->vstage.p, Fc, sizeof(double) * N, cudaMemcpyHostToDevice, P->st));
        CK(dof_to_dev(L, P->vstage.p, C.F.p, P->st));
        C.f_nnz = (int)idx.size();
        CK(C.f_idx.alloc(std::max<size_t>(idx.size(), 1)));
        CK(C.f_val.alloc(std::max<size_t>(val.size(), 1)));
        if (!idx.empty()) {
            CK(cudaMemcpyAsync(C.f_idx.p, idx.data(), idx.size() * sizeof(long long), cudaMemcpyHostToDevice, P->st));
            CK(cudaMemcpyAsync(C.f_val.p, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice, P->st));
        }
        CK(cudaStreamSynchronize(P->st));
    }
    return AM_OK;
}

am_status am_ku_apply(am_problem *P, const am_simp_config *cfg, const double *rho, const double *u,
                      double *y, int precision) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!rho || !u || !y) return fail(AM_ERR_INVALID_ARG, "null array");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, precision == AM_PREC_FP64));
    CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    CKS(setup_operator(P, *cfg, P->rho.p));
    CK(cudaMemcpyAsync(P->vstage.p, u, sizeof(double) * P->N, cudaMemcpyHostToDevice, P->st));
    if (precision == AM_PREC_FP64) {
        CK(dof_to_dev(P->L, P->vstage.p, P->xw64.p, P->st));
        CK(ku_plain<double>(P->plan64, P->L, P->M64, P->s64.p, P->xw64.p, P->r64.p, P->st));
        CK(dev_to_dof(P->L, P->r64.p, P->vstage.p, P->st));
    } else {
        CK(dof_to_dev_t<float>(P->L, P->vstage.p, P->x32.p, P->st));
        CK(ku_plain<float>(P->plan32, P->L, P->M32, P->s32.p, P->x32.p, P->r32.p, P->st));
        CK(dev_to_dof_t<float>(P->L, P->r32.p, P->vstage.p, P->st));
    }
    CK(cudaMemcpyAsync(y, P->vstage.p, sizeof(double) * P->N, cudaMemcpyDeviceToHost, P->st));
    CK(cudaStreamSynchronize(P->st));
    return AM_OK;
}

am_status am_ku_pcg_step(am_problem *P, const am_simp_config *cfg, const double *rho, int load_case,
                         const double *r, const double *p_prev, double beta, int impl, double *p_out,
                         double *q_out, double *pq) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!rho || !r || !p_prev) return fail(AM_ERR_INVALID_ARG, "null array");
    if (impl < 2 || impl > 4) return fail(AM_ERR_INVALID_ARG, "impl must be 2, 3 or 4");
    if (!std::isfinite(beta)) return fail(AM_ERR_INVALID_ARG, "beta must be finite");
    if (load_case < 0 || load_case >= (int)P->cases.size()) return fail(AM_ERR_INVALID_ARG, "load case not set");
    if (impl == 2 && P->plan32.warps != 8) return fail(AM_ERR_INVALID_ARG, "grid too large for the impl-2 kernel");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, false));
    CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    CKS(setup_operator(P, *cfg, P->rho.p));
    CKS(setup_mask(P, load_case));
    CKS(ku3_ready(P));
    CK(cudaMemcpyAsync(P->vstage.p, r, sizeof(double) * P->N, cudaMemcpyHostToDevice, P->st));
    CK(dof_to_dev_t<float>(P->L, P->vstage.p, P->r32.p, P->st));
    CK(cudaMemcpyAsync(P->vstage.p, p_prev, sizeof(double) * P->N, cudaMemcpyHostToDevice, P->st));
    CK(dof_to_dev_t<float>(P->L, P->vstage.p, P->p32a.p, P->st));
    CKS(sync_scalars(P));
    Scalars run = *P->Sh;
    run.done = 0;
    run.it = 0;  // reads p32a, writes p32b
    run.beta = beta;
    run.rz = 1.0;
    run.kerr = 0;
    run.status = ST_RUNNING;
    run.cnt_ku = 0;
    CK(cudaMemcpyAsync(P->S, &run, sizeof(Scalars), cudaMemcpyHostToDevice, P->st));
    if (impl == 3)
        CK(pcg_ku32(P));
    else if (impl == 4)
        CK(ku3b_pcg(P->maps3, P->plan3, P->L, P->M32, P->q32v.p, P->p32a.p, P->p32b.p, P->partial.p, P->S, 5,
                    P->st));
    else
        CK(ku2_pcg(P->plan32, P->L, P->M32, P->s32.p, P->p32a.p, P->p32b.p, P->r32.p, P->dinv32.p, P->mask.p,
                   P->q32v.p, P->partial.p, P->S, P->st));
    CKS(sync_scalars(P));
    if (P->Sh->kerr) return fail(AM_ERR_TIMEOUT, "a copy wait of the PCG K*u timed out");
    if (pq) *pq = P->Sh->pq;
    if (p_out) {
        CK(dev_to_dof_t<float>(P->L, P->p32b.p, P->vstage.p, P->st));
        CK(cudaMemcpyAsync(p_out, P->vstage.p, sizeof(double) * P->N, cudaMemcpyDeviceToHost, P->st));
    }
    if (q_out) {
        CK(dev_to_dof_t<float>(P->L, P->q32v.p, P->vstage.p, P->st));
        CK(cudaMemcpyAsync(q_out, P->vstage.p, sizeof(double) * P->N, cudaMemcpyDeviceToHost, P->st));
    }
    CK(cudaStreamSynchronize(P->st));
    return AM_OK;
}

am_status am_solve(am_problem *P, const am_simp_config *cfg, const double *rho, int load_case,
                   double *u_out, am_solve_stats *stats) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!rho) return fail(AM_ERR_INVALID_ARG, "null density");
    if (load_case < 0 || load_case >= (int)P->cases.size())
        return fail(AM_ERR_INVALID_ARG, "load case not set");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, cfg->precision == AM_PREC_FP64));
    CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    CKS(setup_operator(P, *cfg, P->rho.p));
    CKS(setup_mask(P, load_case));
    SolveOut o;
    CKS(solve_case(P, *cfg, load_case, false, o));
    if (u_out) {
        CK(dev_to_dof(P->L, P->cases[load_case].x64.p, P->vstage.p, P->st));
        CK(cudaMemcpyAsync(u_out, P->vstage.p, sizeof(double) * P->N, cudaMemcpyDeviceToHost, P->st));
        CK(cudaStreamSynchronize(P->st));
    }
    if (stats) {
        stats->iterations = o.iterations;
        stats->outer_iterations = o.outer;
        stats->residual = o.residual;
        stats->converged = o.converged;
        stats->solve_time_s = o.time_s;
        stats->learned_applications = o.learned;
        stats->max_displacement = 0.0;
        stats->min_displacement = 0.0;
        if (u_out) {
            double mx = -INFINITY, mn = INFINITY;
            for (long long i = 0; i < P->N; ++i) {
                mx = std::max(mx, u_out[i]);
                mn = std::min(mn, u_out[i]);
            }
            stats->max_displacement = mx;
            stats->min_displacement = mn;
        }
    }
    return AM_OK;
}

am_status am_selftest_solve_timeout(am_problem *P, const am_simp_config *cfg, const double *rho, int load_case,
                                    int *solve_status) {
    CKS(check_problem(P));
    if (!solve_status) return fail(AM_ERR_INVALID_ARG, "null solve_status");
    P->inject_kerr = true;
    am_solve_stats st{};
    const am_status s = am_solve(P, cfg, rho, load_case, nullptr, &st);
    const std::string msg = g_last_error;
    P->inject_kerr = false;
    // clear the flag so the problem stays usable
    static const int kZero = 0;
    CK(cudaMemcpyAsync(&P->S->kerr, &kZero, sizeof(int), cudaMemcpyHostToDevice, P->st));
    CK(cudaStreamSynchronize(P->st));
    *solve_status = (int)s;
    g_last_error = msg;
    return AM_OK;
}

am_status am_sensitivities(am_problem *P, const am_simp_config *cfg, const double *rho,
                           const double *u, double *dc, double *ce, double *compliance) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!rho || !u) return fail(AM_ERR_INVALID_ARG, "null array");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, true));
    CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    CKS(setup_operator(P, *cfg, P->rho.p));
    CKS(setup_mask(P, -1));
    CK(cudaMemcpyAsync(P->vstage.p, u, sizeof(double) * P->N, cudaMemcpyHostToDevice, P->st));
    CK(dof_to_dev(P->L, P->vstage.p, P->xw64.p, P->st));
    // r64 <- 0 - K u (discarded); ce filled
    CK(cudaMemsetAsync(P->p64a.p, 0, sizeof(double) * 3 * P->L.cs, P->st));
    CK(ku_resid(P->plan64, P->L, P->M64, P->s64.p, P->xw64.p, P->p64a.p, P->dinv64.p, P->mask.p, P->r64.p,
                P->ce.p, P->partial.p, P->S, P->st));
    // design mask: CPP all elements; PY grid == 0
    if (cfg->variant == AM_VARIANT_PY) {
        std::vector<uint8_t> dm((size_t)P->L.nel, 1);
        if (!P->grid_host.empty())
            for (size_t e = 0; e < dm.size(); ++e) dm[e] = P->grid_host[e] == 0;
        CK(cudaMemcpyAsync(P->design.p, dm.data(), dm.size(), cudaMemcpyHostToDevice, P->st));
        CK(cudaStreamSynchronize(P->st));
    }
    CK(sensitivities(P->L, P->rho.p, P->ce.p, P->s64.p, P->design.p, cfg->variant, cfg->penalty, P->dc.p, 0,
                     P->partial.p, P->S, P->st));
    CKS(sync_scalars(P));
    if (compliance) *compliance = P->Sh->comp_energy;
    if (dc) CKS(download_elem(P, P->dc.p, dc, cfg->layout));
    if (ce) CKS(download_elem(P, P->ce.p, ce, cfg->layout));
    return AM_OK;
}

am_status am_filter(am_problem *P, const am_simp_config *cfg, int which, const double *x,
                    const double *rho, double *out) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!x || !out || (which == 0 && !rho)) return fail(AM_ERR_INVALID_ARG, "null array");
    if (which != 0 && which != 1) return fail(AM_ERR_INVALID_ARG, "which must be 0 or 1");
    CKS(ensure_elements(P));
    CKS(build_taps(P, cfg->filter_radius, which));
    CKS(upload_elem(P, x, P->dc.p, cfg->layout));
    if (which == 0) CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    const bool f64 = cfg->precision == AM_PREC_FP64;
    if (which == 0) {
        CK(f64 ? filter_cpp<double>(P->L, taps_of(P), P->dc.p, P->rho.p, P->dcf.p, P->st)
               : filter_cpp<float>(P->L, taps_of(P), P->dc.p, P->rho.p, P->dcf.p, P->st));
    } else {
        CK(f64 ? filter_py<double>(P->L, taps_of(P), P->dc.p, nullptr, P->dcf.p, 0, 0.0, P->st)
               : filter_py<float>(P->L, taps_of(P), P->dc.p, nullptr, P->dcf.p, 0, 0.0, P->st));
    }
    CKS(download_elem(P, P->dcf.p, out, cfg->layout));
    return AM_OK;
}

am_status am_oc_update(am_problem *P, const am_simp_config *cfg, const double *rho, const double *dc,
                       const uint8_t *design, double *rho_new, double *max_change, int *passes) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (!rho || !dc || !design || !rho_new) return fail(AM_ERR_INVALID_ARG, "null array");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, true));
    CKS(upload_elem(P, rho, P->rho.p, cfg->layout));
    CKS(upload_elem(P, dc, P->dcf.p, cfg->layout));
    CK(cudaMemcpyAsync(P->estage.p, design, (size_t)P->L.nel, cudaMemcpyHostToDevice, P->st));
    CK(elem_to_dev<uint8_t>(P->L, (const uint8_t *)P->estage.p, P->design.p, cfg->layout, P->st));
    long long nd = 0;
    for (long long e = 0; e < P->L.nel; ++e) nd += design[e] ? 1 : 0;
    double n_design = (double)nd;
    if (cfg->variant == AM_VARIANT_CPP && nd == 0) n_design = (double)P->L.nel;
    const bool f64 = cfg->precision == AM_PREC_FP64;
    CKS(run_oc(P, f64, cfg->variant, cfg->move_limit, cfg->rho_min, cfg->volume_fraction, n_design, P->rho.p,
               P->dcf.p, P->design.p, P->rho_new.p));
    if (max_change) *max_change = P->Sh->oc_change;
    if (passes) *passes = P->Sh->oc_pass;
    CKS(download_elem(P, P->rho_new.p, rho_new, cfg->layout));
    return AM_OK;
}

am_status am_simp_begin(am_problem *P, const am_simp_config *cfg, const double *rho0) {
    CKS(check_problem(P));
    CKS(check_cfg(P, cfg));
    if (P->cases.empty()) return fail(AM_ERR_INVALID_ARG, "loads not set");
    if (cfg->max_iterations < 0) return fail(AM_ERR_INVALID_ARG, "max_iterations < 0");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, cfg->precision == AM_PREC_FP64));
    P->cfg = *cfg;
    const long long nel = P->L.nel;
    std::vector<double> r0((size_t)nel);
    if (rho0) {
        CKS(upload_elem(P, rho0, P->rho.p, cfg->layout));
        CK(cudaMemcpyAsync(r0.data(), P->rho.p, sizeof(double) * nel, cudaMemcpyDeviceToHost, P->st));
        CK(cudaStreamSynchronize(P->st));
    } else {
        for (long long e = 0; e < nel; ++e) {
            const int g = P->grid_host.empty() ? 0 : P->grid_host[(size_t)e];
            // PY: uniform volume_fraction (topopt.py:124); CPP: am_topopt.cpp:562-572
            if (cfg->variant == AM_VARIANT_PY || g == 0) r0[(size_t)e] = cfg->volume_fraction;
            else r0[(size_t)e] = g == 1 ? 1.0 : cfg->rho_min;
        }
        CK(cudaMemcpyAsync(P->rho.p, r0.data(), sizeof(double) * nel, cudaMemcpyHostToDevice, P->st));
    }
    // design mask: CPP from the initial density (topology_optimizer.cpp:419-428),
    // PY grid == 0 (topopt.py:127)
    std::vector<uint8_t> dm((size_t)nel);
    long long nd = 0;
    for (long long e = 0; e < nel; ++e) {
        bool d;
        if (cfg->variant == AM_VARIANT_CPP) d = r0[(size_t)e] > cfg->rho_min + 1e-6 && r0[(size_t)e] < 0.99;
        else d = P->grid_host.empty() ? true : P->grid_host[(size_t)e] == 0;
        dm[(size_t)e] = d;
        nd += d;
    }
    P->n_design = (cfg->variant == AM_VARIANT_CPP && nd == 0) ? (double)nel : (double)nd;
    CK(cudaMemcpyAsync(P->design.p, dm.data(), dm.size(), cudaMemcpyHostToDevice, P->st));
    CKS(build_taps(P, cfg->filter_radius, cfg->variant == AM_VARIANT_CPP ? 0 : 1));
    for (auto &c : P->cases) c.have_x = false;
    CK(cudaStreamSynchronize(P->st));
    // a new design mask: the passive solid inclusions are found again on first use
    defl_destroy(P->defl);
    P->defl = nullptr;
    P->defl_tried = false;
    P->simp_begun = true;
    P->iter = 0;
    return AM_OK;
}

am_status am_simp_step(am_problem *P, am_iteration_result *res) {
    CKS(check_problem(P));
    if (!P->simp_begun) return fail(AM_ERR_INVALID_ARG, "am_simp_begin not called");
    const am_simp_config &c = P->cfg;
    const bool f64 = c.precision == AM_PREC_FP64;
    am_iteration_result R{};
    double t0 = now_s();
    const double *rho_asm = P->rho.p;
    if (c.variant == AM_VARIANT_PY) {
        // density pre-filter + clip (topopt.py:302-303)
        CK(filter_py<double>(P->L, taps_of(P), P->rho.p, nullptr, P->rho_f.p, 1, c.rho_min, P->st));
        rho_asm = P->rho_f.p;
    }
    CKS(setup_operator(P, c, rho_asm));
    CK(cudaStreamSynchronize(P->st));
    double t1 = now_s();
    R.assembly_time_s = t1 - t0;
    double comp = 0.0;
    int total_its = 0, total_outer = 0, total_learned = 0, conv = 1;
    double worst_res = 0.0;
    double t_solve = 0.0, t_sens = 0.0;
    for (int lc = 0; lc < (int)P->cases.size(); ++lc) {
        if (c.variant == AM_VARIANT_CPP && lc > 0) break;  // the C++ loop takes one F
        double ts = now_s();
        CKS(setup_mask(P, lc));
        SolveOut o;
        CKS(solve_case(P, c, lc, true, o));
        total_its += o.iterations;
        total_outer += o.outer;
        total_learned += o.learned;
        conv = conv && o.converged;
        worst_res = std::max(worst_res, o.residual);
        double te = now_s();
        t_solve += te - ts;
        CK(sensitivities(P->L, rho_asm, P->ce.p, P->s64.p, P->design.p, c.variant, c.penalty, P->dc.p,
                         lc > 0 ? 1 : 0, P->partial.p, P->S, P->st));
        CK(sparse_dot(P->cases[lc].f_idx.p, P->cases[lc].f_val.p, P->cases[lc].f_nnz, P->cases[lc].x64.p,
                      &P->S->comp_fu, P->st));
        CKS(sync_scalars(P));
        if (c.variant == AM_VARIANT_CPP) comp = P->Sh->comp_fu;
        t_sens += now_s() - te;
    }
    if (c.variant == AM_VARIANT_PY) comp = P->Sh->comp_energy;
    R.compliance = comp;
    R.compliance_energy = P->Sh->comp_energy;
    R.solve_time_s = t_solve;
    R.sensitivity_time_s = t_sens;
    R.solver_iterations = total_its;
    R.solver_outer_iterations = total_outer;
    R.solver_residual = worst_res;
    R.solver_converged = conv;
    R.solver_learned_applications = total_learned;
    double tu = now_s();
    // filter (topology_optimizer.cpp:351 / topopt.py:363), FP64 in every mode: the
    // OC bisection is discrete, so an FP32 filter's rounding can flip one of its
    // late branch decisions and move the density by ~1e-4 relative; the filter is
    // well under 1% of a step.
    if (c.variant == AM_VARIANT_CPP) {
        CK(filter_cpp<double>(P->L, taps_of(P), P->dc.p, P->rho.p, P->dcf.p, P->st));
    } else {
        CK(filter_py<double>(P->L, taps_of(P), P->dc.p, P->rho.p, P->dcf.p, 2, 0.0, P->st));
    }
    // OC update
    CKS(run_oc(P, f64, c.variant, c.move_limit, c.rho_min, c.volume_fraction, P->n_design, P->rho.p, P->dcf.p,
               P->design.p, P->rho_new.p));
    std::swap(P->rho, P->rho_new);
    R.update_time_s = now_s() - tu;
    R.max_density_change = P->Sh->oc_change;
    R.volume_fraction = P->Sh->oc_volume;
    R.oc_passes = P->Sh->oc_pass;
    ++P->iter;
    if (res) *res = R;
    return AM_OK;
}

long long am_launch_count(void) { return launch_count(); }

am_status am_bench_kernel(am_problem *P, int which, int reps, int flush_l2, double *avg_ms, double *min_ms) {
    CKS(check_problem(P));
    if (!P->simp_begun) return fail(AM_ERR_INVALID_ARG, "am_simp_begin not called");
    if (reps < 1) return fail(AM_ERR_INVALID_ARG, "reps must be >= 1");
    if (P->cases.empty()) return fail(AM_ERR_INVALID_ARG, "no load case set");
    CKS(ensure_vectors(P, false));
    if (P->iter < 1) {
        // no step ran yet: operator and mask of the current density, zero vectors
        CKS(setup_operator(P, P->cfg, P->rho.p));
        CKS(setup_mask(P, 0));
        CK(P->cases[0].x64.alloc(3 * (size_t)P->L.cs));
    }
    CKS(sync_scalars(P));
    const Scalars saved = *P->Sh;
    Scalars run = saved;
    run.done = 0;
    run.beta = 0.5;
    run.alpha = 1e-3;
    run.thr = 0.0;
    run.maxit = 1 << 30;
    run.it = 0;
    CK(cudaMemcpyAsync(P->S, &run, sizeof(Scalars), cudaMemcpyHostToDevice, P->st));
    CKS(ku3_ready(P));
    // filter (8) and OC pass (9) time the mixed-precision forms on the state the
    // last SIMP step left (densities, sensitivities, design mask, filter taps)
    const am_simp_config &cf = P->cfg;
    OcBuffers ocb{P->L.nel, P->oc_a64.p, P->oc_lo64.p, P->oc_hi64.p, P->oc_a32.p, P->oc_lo32.p, P->oc_hi32.p};
    if (which == 8 || which == 9) {
        if (P->iter < 1) return fail(AM_ERR_INVALID_ARG, "the filter / OC probes need a SIMP step first");
        CKS(build_taps(P, cf.filter_radius, cf.variant));
    }
    if (which == 9) {
        const size_t ne = (size_t)P->L.nel;
        CK(P->oc_a32.alloc(ne)); CK(P->oc_lo32.alloc(ne)); CK(P->oc_hi32.alloc(ne));
        ocb = OcBuffers{P->L.nel, P->oc_a64.p, P->oc_lo64.p, P->oc_hi64.p, P->oc_a32.p, P->oc_lo32.p, P->oc_hi32.p};
        CK(oc_prepare(ocb, P->rho.p, P->dcf.p, cf.move_limit, 0, cf.variant, P->S, P->st));
    }
    if (which == 10 || which == 11) {
        // one V-cycle (10) or the V-cycle balanced by the passive inclusions'
        // rigid-body modes (11) on the residual vector
        bool ok = false;
        CKS(mg_ready(P, 0, which == 11, &ok));
        if (!ok) return fail(AM_ERR_INVALID_ARG, "the grid does not coarsen for multigrid");
        if (which == 11 && !P->defl) return fail(AM_ERR_INVALID_ARG, "no passive solid inclusion to deflate");
    }
    DevBuf<uint8_t> flush;
    const size_t flush_bytes = 512ull << 20;
    if (flush_l2) CK(flush.alloc(flush_bytes));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double tot = 0.0, mn = 1e30;
    for (int k = 0; k < reps; ++k) {
        if (flush_l2) {
            // write a 512 MB buffer (evicts the problem's data from the 129 MB L2),
            // then read it back so the lines the write left dirty are written back
            // before the timed launch rather than during it
            CK(cudaMemsetAsync(flush.p, k & 0xff, flush_bytes, P->st));
            CK(l2_flush_read(flush.p, flush_bytes, P->st));
        }
        CK(cudaMemcpyAsync(&P->S->done, &run.done, sizeof(int), cudaMemcpyHostToDevice, P->st));
        if (which == 6 || which == 7) {
            // the update of an even (6: r only) or odd (7: r and the folded iterate) iteration
            const int parity = which - 6;
            CK(cudaMemcpyAsync(&P->S->it, &parity, sizeof(int), cudaMemcpyHostToDevice, P->st));
        }
        CK(cudaEventRecord(e0, P->st));
        switch (which) {
            case 0:
                CK(pcg_ku32(P));
                break;
            case 1:
                CK(ku_resid(P->plan64, P->L, P->M64, P->s64.p, P->cases[0].x64.p, P->cases[0].F.p, P->dinv64.p,
                            P->mask.p, P->r64.p, nullptr, P->partial.p, P->S, P->st));
                break;
            case 2:
            case 6:
            case 7:
                CK(pcg_update_df(P->L, P->x32.p, P->xl32.p, P->r32.p, P->p32a.p, P->p32b.p, P->q32v.p,
                                 P->dinv32.p, P->partial.p, P->S, P->st));
                break;
            case 3:
                CK(ku_plain<float>(P->plan32, P->L, P->M32, P->s32.p, P->p32a.p, P->q32v.p, P->st));
                break;
            case 4:
                CK(ku2_pcg(P->plan32, P->L, P->M32, P->s32.p, P->p32a.p, P->p32b.p, P->r32.p, P->dinv32.p,
                           P->mask.p, P->q32v.p, P->partial.p, P->S, P->st));
                break;
            case 5:
                CK(ku3_pcg(P->maps3, P->plan3, P->L, P->M32, P->partial.p, P->S, 3, P->st));
                break;
            case 12:
                CK(ku3_pcg(P->maps3, P->plan3, P->L, P->M32, P->partial.p, P->S, 4, P->st));
                break;
            case 14:
                CK(ku_resid_df(P->plan64, P->L, P->M64, P->s64.p, P->cases[0].x64.p, P->cases[0].F.p,
                               P->dinv64.p, P->mask.p, P->r64.p, nullptr, P->partial.p, P->S, P->st));
                break;
            case 13:
                CK(ku3b_pcg(P->maps3, P->plan3, P->L, P->M32, P->q32v.p, P->p32a.p, P->p32b.p, P->partial.p, P->S,
                            4, P->st));
                break;
            case 8:  // the SIMP loop's FP64 shared-memory stencil
                CK(filter_cpp<double>(P->L, taps_of(P), P->dc.p, P->rho.p, P->dcf.p, P->st));
                break;
            case 9: {
                const int zero = 0;
                CK(cudaMemcpyAsync(&P->S->oc_done, &zero, sizeof(int), cudaMemcpyHostToDevice, P->st));
                CK(oc_pass(ocb, P->design.p, 0, cf.variant, cf.rho_min, cf.volume_fraction, P->n_design,
                           P->partial.p, P->S, P->nblocks_vec, P->st));
                break;
            }
            case 10:
                CK(mg_apply(P->mg, P->r64.p, P->xi64.p, P->st));
                break;
            case 11:
                CK(defl_apply(P->defl, P->mg, P->r64.p, P->xi64.p, P->st));
                break;
            default:
                return fail(AM_ERR_INVALID_ARG, "unknown kernel id");
        }
        CK(cudaEventRecord(e1, P->st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        tot += ms;
        mn = std::min(mn, (double)ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    flush.release();
    CK(cudaMemcpyAsync(P->S, &saved, sizeof(Scalars), cudaMemcpyHostToDevice, P->st));
    CK(cudaStreamSynchronize(P->st));
    if (avg_ms) *avg_ms = tot / reps;
    if (min_ms) *min_ms = mn;
    return AM_OK;
}

am_status am_problem_set_preconditioner(am_problem *P, am_precond *m) {
    CKS(check_problem(P));
    P->pre = m;
    return AM_OK;
}

am_status am_problem_set_residual_arithmetic(am_problem *P, int mode) {
    CKS(check_problem(P));
    if (mode != AM_RESID_DOUBLE_FLOAT && mode != AM_RESID_FP64) return fail(AM_ERR_INVALID_ARG, "unknown residual mode");
    P->resid_df = mode == AM_RESID_DOUBLE_FLOAT;
    return AM_OK;
}

am_status am_problem_set_ku_plan(am_problem *P, int warps) {
    CKS(check_problem(P));
    if (warps != 0 && warps != 7 && warps != 8) return fail(AM_ERR_INVALID_ARG, "warps must be 0, 7 or 8");
    const KuLaunch K = ku3_plan(P->L, warps);
    if (K.warps != P->plan3.warps || K.tz != P->plan3.tz) {
        CK(cudaStreamSynchronize(P->st));
        // the tensor maps' boxes and the FP32 solver graphs hold the old plan
        ku3_free_maps(P->maps3);
        P->maps3 = nullptr;
        for (cudaGraphExec_t *g : {&P->g32, &P->gl32})
            if (*g) {
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
        P->plan3 = K;
    }
    return AM_OK;
}

am_status am_problem_get_ku_plan(am_problem *P, int *warps, int *tiles, int *z_chunk) {
    CKS(check_problem(P));
    if (warps) *warps = P->plan3.warps;
    if (tiles) *tiles = P->plan3.ntiles();
    if (z_chunk) *z_chunk = P->plan3.tz;
    return AM_OK;
}

am_status am_problem_set_device_loop(am_problem *P, int on) {
    CKS(check_problem(P));
    P->device_loop = on != 0;
    return AM_OK;
}

am_status am_precond_harvest(am_precond *m, am_problem *P, const am_simp_config *cfg, const double *rho,
                             int load_case, const int *iters, int n_iters) {
    CKS(check_problem(P));
    if (!m) return fail(AM_ERR_INVALID_ARG, "null preconditioner");
    if (!cfg || !rho || !iters || n_iters < 1) return fail(AM_ERR_INVALID_ARG, "need cfg, rho and iteration counts");
    am_simp_config c = *cfg;
    c.preconditioner = AM_PRECOND_JACOBI;
    CKS(check_cfg(P, &c));
    if (load_case < 0 || load_case >= (int)P->cases.size()) return fail(AM_ERR_INVALID_ARG, "load case out of range");
    for (int i = 0; i < n_iters; ++i)
        if (iters[i] < 0 || (i > 0 && iters[i] < iters[i - 1]))
            return fail(AM_ERR_INVALID_ARG, "iteration counts must be >= 0 and ascending");
    CKS(ensure_elements(P));
    CKS(ensure_vectors(P, false));
    CKS(upload_elem(P, rho, P->rho_f.p, c.layout));
    CKS(setup_operator(P, c, P->rho_f.p));
    CKS(setup_mask(P, load_case));
    LoadCaseDev &C = P->cases[load_case];
    // r = mask(F) (the residual of u = 0), then FP32 Jacobi PCG from u = 0
    CK(cudaMemsetAsync(P->xw64.p, 0, sizeof(double) * 3 * P->L.cs, P->st));
    CK(ku_resid(P->plan64, P->L, P->M64, P->s64.p, P->xw64.p, C.F.p, P->dinv64.p, P->mask.p, P->r64.p, nullptr,
                P->partial.p, P->S, P->st));
    CK(dc_inner_init(P->L, P->r64.p, P->r32.p, nullptr, P->S, P->nblocks_vec, P->st));
    CKS(inner_iterate_zero(P));
    const PrecondView view{P->L, P->dinv32.p, P->mask.p, P->rho_f.p, P->st};
    int did = -1;
    CKS(precond_add_density(m, view, P->M32, P->s32.p, &did));
    CK(pcg_start<float>(P->L, P->r32.p, P->dinv32.p, 0.0, 0.0, std::max(iters[0], 0), 0, P->partial.p, P->S,
                        P->nblocks_vec, P->st));
    CKS(sync_scalars(P));
    // snapshots of (r_k, u_k); the errors need u*, solved after the sequence
    const size_t nv = 3 * (size_t)P->L.cs;
    DevBuf<float> snap;
    DevBuf<double> snapx;
    CK(snap.alloc(nv * (size_t)n_iters));
    CK(snapx.alloc(nv * (size_t)n_iters));
    for (int i = 0; i < n_iters; ++i) {
        if (iters[i] > P->Sh->it && P->Sh->status != ST_BREAKDOWN && P->Sh->status != ST_NAN) {
            // continue the same sequence up to iters[i]
            const int maxit = iters[i], zero = 0, running = ST_RUNNING;
            CK(cudaMemcpyAsync(&P->S->maxit, &maxit, sizeof(int), cudaMemcpyHostToDevice, P->st));
            CK(cudaMemcpyAsync(&P->S->done, &zero, sizeof(int), cudaMemcpyHostToDevice, P->st));
            CK(cudaMemcpyAsync(&P->S->status, &running, sizeof(int), cudaMemcpyHostToDevice, P->st));
            int its = 0, stt = 0;
            CKS(run_pcg<float>(P, &its, &stt));
            if (stt == ST_NAN) return fail(AM_ERR_NAN_DETECTED, "NaN in the harvesting PCG");
        }
        CK(cudaMemcpyAsync(snap.p + nv * i, P->r32.p, nv * sizeof(float), cudaMemcpyDeviceToDevice, P->st));
        CKS(inner_iterate_to_fp64(P));
        CK(cudaMemcpyAsync(snapx.p + nv * i, P->xi64.p, nv * sizeof(double), cudaMemcpyDeviceToDevice, P->st));
    }
    // u*: FP64-accepted solve to 1e-10 from zero
    am_simp_config cs = c;
    cs.precision = AM_PREC_MIXED;
    cs.cg_tol = 1e-10;
    cs.warm_start = 0;
    cs.verbose = 0;
    SolveOut o;
    CKS(solve_case(P, cs, load_case, false, o));
    for (int i = 0; i < n_iters; ++i)
        CKS(precond_add_sample(m, did, snap.p + nv * i, snapx.p + nv * i, C.x64.p, P->st));
    CK(cudaStreamSynchronize(P->st));
    return AM_OK;
}

am_status am_problem_stream(am_problem *P, void **stream) {
    CKS(check_problem(P));
    if (!stream) return fail(AM_ERR_INVALID_ARG, "null output");
    *stream = (void *)P->st;
    return AM_OK;
}

am_status am_problem_layout(am_problem *P, long long *nodes, long long *elements, long long *vector_stride,
                            int *ku_tiles) {
    CKS(check_problem(P));
    if (nodes) *nodes = P->nn_ref;
    if (elements) *elements = P->L.nel;
    if (vector_stride) *vector_stride = P->L.cs;
    if (ku_tiles) *ku_tiles = P->plan32.ntiles();
    return AM_OK;
}

am_status am_simp_get_density(am_problem *P, double *rho_out) {
    CKS(check_problem(P));
    if (!P->simp_begun) return fail(AM_ERR_INVALID_ARG, "am_simp_begin not called");
    if (!rho_out) return fail(AM_ERR_INVALID_ARG, "null output");
    return download_elem(P, P->rho.p, rho_out, P->cfg.layout);
}

am_status am_simp_run(am_problem *P, const am_simp_config *cfg, const double *rho0, double *rho_out,
                      double *compliance_hist, double *volume_hist, double *change_hist,
                      int *iterations, int *converged) {
    CKS(am_simp_begin(P, cfg, rho0));
    int it = 0;
    int conv = 0;
    for (; it < cfg->max_iterations; ++it) {
        am_iteration_result R;
        CKS(am_simp_step(P, &R));
        if (compliance_hist) compliance_hist[it] = R.compliance;
        if (volume_hist) volume_hist[it] = R.volume_fraction;
        if (change_hist) change_hist[it] = R.max_density_change;
        if (cfg->verbose)
            std::printf("%6d %14.4e %10.3f %12.2e %10d\n", it, R.compliance, R.volume_fraction,
                        R.max_density_change, R.solver_iterations);
        if (R.max_density_change < cfg->convergence_tol) {
            conv = 1;
            ++it;
            break;
        }
    }
    if (iterations) *iterations = it;
    if (converged) *converged = conv;
    if (rho_out) CKS(am_simp_get_density(P, rho_out));
    return AM_OK;
}

}  // extern "C"
