// kernels.cu -- the kernels of the GB300 SIMP engine other than the tiled K*u
// body (ku.cuh), plus the launchers declared in kernels.cuh.
#include <algorithm>
#include <atomic>

#include "batch.cuh"
#include "kernels.cuh"
#include "ku.cuh"
#include "kudf.cuh"
#include "bulk.cuh"
#include "ku2.cuh"

namespace amk {

static inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// Host-side count of kernel launches issued by this library (graph launches add
// the kernel nodes they contain, see count_launches).
static std::atomic<long long> g_launches{0};
long long launch_count() { return g_launches.load(); }
void count_launches(long long n) { g_launches += n; }
static inline cudaError_t counted(cudaError_t e) {
    if (e == cudaSuccess) ++g_launches;
    return e;
}

// ============================================================================
// K*u launch plans and launchers
// ============================================================================
KuLaunch ku_plan_shape(const Layout &L, int tx, int ty, int warps, int ctas_per_sm, int tz_hint, int sms) {
    KuLaunch K;
    K.tx = tx;
    K.ty = ty;
    K.warps = warps;
    K.tiles_x = div_up(L.nx + 1, K.tx);
    K.tiles_y = div_up(L.ny + 1, K.ty);
    const long long cols = (long long)K.tiles_x * K.tiles_y;
    const int planes = L.nz + 1;
    int tz = tz_hint;
    if (tz <= 0) {
        // time ~ waves x (planes per tile + 1 halo layer); pick the z chunking
        // that minimises it (chunks of >= 4 planes)
        const long long slots = (long long)sms * ctas_per_sm;
        double best = 1e300;
        tz = planes;
        for (int chunks = 1; chunks <= planes; ++chunks) {
            const int t = div_up(planes, chunks);
            if (t < 4 && chunks > 1) break;
            const long long tiles = cols * div_up(planes, t);
            const double waves = (double)div_up(tiles, slots);
            const double cost = waves * (t + 1);
            if (cost < best - 1e-9) {
                best = cost;
                tz = t;
            }
        }
    }
    K.tz = std::min(std::max(tz, 1), planes);
    K.tiles_z = div_up(planes, K.tz);
    return K;
}

KuLaunch ku_plan(const Layout &L, bool fp64, int tz_hint, int sms) {
    if (fp64) return ku_plan_shape(L, 32, 4, 0, 3, tz_hint, sms);
    // warp-row kernel (32-bit indices)
    if (3 * L.cs < (1LL << 31) && L.nel < (1LL << 31))
        return ku_plan_shape(L, Ku2Shape<8>::TX, Ku2Shape<8>::TY, 8, 2, tz_hint, sms);
    return ku_plan_shape(L, 32, 8, 0, 2, tz_hint, sms);
}

template <typename T, int TX, int TY, int MODE>
static cudaError_t set_ku_attr() {
    using Sh = KuShape<TX, TY>;
    return cudaFuncSetAttribute(ku_tile_kernel<T, TX, TY, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Sh::template smem_bytes<T>());
}

cudaError_t filter_init_attributes();
cudaError_t update_init_attributes();

cudaError_t ku_init_attributes() {
    cudaError_t e;
#define AMK_ATTR(T, X, Y, M) \
    if ((e = set_ku_attr<T, X, Y, M>()) != cudaSuccess) return e;
    AMK_ATTR(float, 32, 8, KU_PLAIN)
    AMK_ATTR(float, 32, 8, KU_PCG)
    AMK_ATTR(float, 32, 4, KU_PLAIN)
    AMK_ATTR(float, 32, 4, KU_PCG)
    AMK_ATTR(double, 32, 8, KU_PLAIN)
    AMK_ATTR(double, 32, 8, KU_PCG)
    AMK_ATTR(double, 32, 8, KU_RESID)
    AMK_ATTR(double, 32, 4, KU_PLAIN)
    AMK_ATTR(double, 32, 4, KU_PCG)
    AMK_ATTR(double, 32, 4, KU_RESID)
    AMK_ATTR(double, 32, 4, KU_DOT)
    AMK_ATTR(double, 32, 8, KU_DOT)
#undef AMK_ATTR
    if ((e = cudaFuncSetAttribute(ku_df_kernel<32, 4, KU_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)KuShape<32, 4>::smem_bytes<double>())) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(ku_df_kernel<32, 4, KU_DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)KuShape<32, 4>::smem_bytes<double>())) != cudaSuccess)
        return e;
    if ((e = update_init_attributes()) != cudaSuccess) return e;
    return filter_init_attributes();
}

template <typename T, int TX, int TY, int MODE>
static cudaError_t launch_ku(const KuLaunch &K, KuArgs<T> &a, cudaStream_t st) {
    using Sh = KuShape<TX, TY>;
    const size_t smem = Sh::template smem_bytes<T>();
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tiles_z = K.tiles_z;
    a.tz = K.tz;
    ku_tile_kernel<T, TX, TY, MODE><<<K.ntiles(), Sh::NT, smem, st>>>(a);
    return counted(cudaGetLastError());
}

template <typename T, int MODE>
static cudaError_t dispatch_ku(const KuLaunch &K, KuArgs<T> &a, cudaStream_t st) {
    if (K.tx == 32 && K.ty == 8) return launch_ku<T, 32, 8, MODE>(K, a, st);
    if (K.tx == 32 && K.ty == 4) return launch_ku<T, 32, 4, MODE>(K, a, st);
    return cudaErrorInvalidValue;
}

// PCG launches come from the single-problem engine, whose PCG vectors carry
// ku2_slack(): their node loads are unpredicated
template <int MODE>
static cudaError_t launch_ku2(const KuLaunch &K, Ku2Args &a, cudaStream_t st) {
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tiles_z = K.tiles_z;
    a.tz = K.tz;
    if (K.warps == 8) {
        ku2_kernel<8, MODE, MODE == KU_PCG><<<K.ntiles(), 256, 0, st>>>(a);
        return counted(cudaGetLastError());
    }
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t ku_plain(const KuLaunch &K, const Layout &L, const Modal<T> &M, const T *s, const T *u,
                     T *y, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (K.warps > 0) {
            Ku2Args a{};
            a.L = L;
            a.M = M;
            a.s = s;
            a.u = u;
            a.y = y;
            return launch_ku2<KU_PLAIN>(K, a, st);
        }
    }
    KuArgs<T> a{};
    a.L = L;
    a.M = M;
    a.s = s;
    a.u = u;
    a.y = y;
    return dispatch_ku<T, KU_PLAIN>(K, a, st);
}

cudaError_t ku2_pcg(const KuLaunch &K, const Layout &L, const Modal<float> &M, const float *s, float *pa, float *pb,
                    const float *r, const float *dinv, const uint8_t *mask, float *q, double *partial, Scalars *S,
                    cudaStream_t st) {
    if (K.warps != 8) return cudaErrorInvalidValue;
    Ku2Args a{};
    a.L = L;
    a.M = M;
    a.s = s;
    a.pa = pa;
    a.pb = pb;
    a.r = r;
    a.dinv = dinv;
    a.mask = mask;
    a.y = q;
    a.partial = partial;
    a.S = S;
    return launch_ku2<KU_PCG>(K, a, st);
}

template <typename T>
cudaError_t ku_pcg(const KuLaunch &K, const Layout &L, const Modal<T> &M, const T *s, T *pa, T *pb,
                   const T *r, const T *dinv, const uint8_t *mask, T *q, double *partial, Scalars *S,
                   cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (K.warps > 0) {
            Ku2Args a{};
            a.L = L;
            a.M = M;
            a.s = s;
            a.pa = pa;
            a.pb = pb;
            a.r = r;
            a.dinv = dinv;
            a.mask = mask;
            a.y = q;
            a.partial = partial;
            a.S = S;
            return launch_ku2<KU_PCG>(K, a, st);
        }
    }
    KuArgs<T> a{};
    a.L = L;
    a.M = M;
    a.s = s;
    a.pa = pa;
    a.pb = pb;
    a.r = r;
    a.dinv = dinv;
    a.mask = mask;
    a.y = q;
    a.partial = partial;
    a.S = S;
    return dispatch_ku<T, KU_PCG>(K, a, st);
}

cudaError_t ku_resid(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s,
                     const double *x, const double *f, const double *dinv, const uint8_t *mask,
                     double *r, double *ce, double *partial, Scalars *S, cudaStream_t st) {
    KuArgs<double> a{};
    a.L = L;
    a.M = M;
    a.s = s;
    a.u = x;
    a.f = f;
    a.dinv = dinv;
    a.mask = mask;
    a.y = r;
    a.ce = ce;
    a.energy = ce != nullptr;
    a.partial = partial;
    a.S = S;
    return dispatch_ku<double, KU_RESID>(K, a, st);
}

cudaError_t ku_resid_df(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s,
                        const double *x, const double *f, const double *dinv, const uint8_t *mask, double *r,
                        double *ce, double *partial, Scalars *S, cudaStream_t st) {
    if (!(K.tx == 32 && K.ty == 4) || K.warps > 0) return cudaErrorInvalidValue;
    KuArgs<double> a{};
    a.L = L;
    a.s = s;
    a.u = x;
    a.f = f;
    a.dinv = dinv;
    a.mask = mask;
    a.y = r;
    a.ce = ce;
    a.energy = ce != nullptr;
    a.partial = partial;
    a.S = S;
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tiles_z = K.tiles_z;
    a.tz = K.tz;
    using Sh = KuShape<32, 4>;
    ku_df_kernel<32, 4, KU_RESID><<<K.ntiles(), Sh::NT, Sh::smem_bytes<double>(), st>>>(a, modal_dflt(M));
    return counted(cudaGetLastError());
}

cudaError_t ku_dot_df(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s, const double *p,
                      const uint8_t *mask, double *q, double *partial, Scalars *S, cudaStream_t st) {
    if (!(K.tx == 32 && K.ty == 4) || K.warps > 0) return cudaErrorInvalidValue;
    KuArgs<double> a{};
    a.L = L;
    a.s = s;
    a.u = p;
    a.mask = mask;
    a.y = q;
    a.partial = partial;
    a.S = S;
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tiles_z = K.tiles_z;
    a.tz = K.tz;
    using Sh = KuShape<32, 4>;
    ku_df_kernel<32, 4, KU_DOT><<<K.ntiles(), Sh::NT, Sh::smem_bytes<double>(), st>>>(a, modal_dflt(M));
    return counted(cudaGetLastError());
}

cudaError_t ku_dot(const KuLaunch &K, const Layout &L, const Modal<double> &M, const double *s, const double *p,
                   const uint8_t *mask, double *q, double *partial, Scalars *S, cudaStream_t st) {
    KuArgs<double> a{};
    a.L = L;
    a.M = M;
    a.s = s;
    a.u = p;
    a.mask = mask;
    a.y = q;
    a.partial = partial;
    a.S = S;
    return dispatch_ku<double, KU_DOT>(K, a, st);
}

// q = mask(q32) in FP64 and p.q -> S->o_pq, S->o_alpha (the finish of KU_DOT)
__global__ void __launch_bounds__(256) dot_from_f32_kernel(Layout L, const double *__restrict__ p,
                                                          const float *__restrict__ q32,
                                                          const uint8_t *__restrict__ mask, double *__restrict__ q,
                                                          double *partial, Scalars *S) {
    __shared__ double red[8];
    __shared__ int last_flag;
    double acc = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const unsigned m = mask[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long i = n + c * L.cs;
            const double v = ((m >> c) & 1u) ? 0.0 : (double)q32[i];
            q[i] = v;
            acc = fma(p[i], v, acc);
        }
    }
    double v[1] = {acc};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partial[2 * blockIdx.x] = v[0];
    if (!arrive_last(&S->cnt_ku, &last_flag)) return;
    double tot[1];
    reduce_partials<1>(partial, gridDim.x, 2, tot, red);
    if (threadIdx.x == 0) {
        const double pq = tot[0];
        S->o_pq = pq;
        if (!(pq > 0.0) || !isfinite(pq)) {
            S->o_status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
            S->o_alpha = 0.0;
        } else {
            S->o_alpha = S->o_zr / pq;
        }
        S->cnt_ku = 0;
    }
}
__global__ void f64_to_f32_kernel(const double *__restrict__ a, float *__restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
cudaError_t ku_dot_f32(const KuLaunch &K32, const Layout &L, const Modal<float> &M, const float *s32, const double *p,
                       const uint8_t *mask, float *p32, float *q32, double *q, double *partial, Scalars *S,
                       int nblocks, cudaStream_t st) {
    f64_to_f32_kernel<<<nblocks, 256, 0, st>>>(p, p32, 3 * L.cs);
    cudaError_t e = counted(cudaGetLastError());
    if (e == cudaSuccess) e = ku_plain<float>(K32, L, M, s32, p32, q32, st);
    if (e != cudaSuccess) return e;
    dot_from_f32_kernel<<<nblocks, 256, 0, st>>>(L, p, q32, mask, q, partial, S);
    return counted(cudaGetLastError());
}

template cudaError_t ku_plain<float>(const KuLaunch &, const Layout &, const Modal<float> &,
                                     const float *, const float *, float *, cudaStream_t);
template cudaError_t ku_plain<double>(const KuLaunch &, const Layout &, const Modal<double> &,
                                      const double *, const double *, double *, cudaStream_t);
template cudaError_t ku_pcg<float>(const KuLaunch &, const Layout &, const Modal<float> &, const float *,
                                   float *, float *, const float *, const float *, const uint8_t *, float *,
                                   double *, Scalars *, cudaStream_t);
template cudaError_t ku_pcg<double>(const KuLaunch &, const Layout &, const Modal<double> &, const double *,
                                    double *, double *, const double *, const double *, const uint8_t *,
                                    double *, double *, Scalars *, cudaStream_t);

// ============================================================================
// PCG vector kernels
// ============================================================================
constexpr int VEC_THREADS = 256;

// Last block of a PCG update: the iteration's r.r and r.z -> beta and the stop tests.
__device__ __forceinline__ void pcg_update_finish(Scalars *S, double rr, double rz) {
    S->it += 1;
    S->rr = rr;
    S->rz_prev = S->rz;
    S->beta = (S->rz != 0.0) ? rz / S->rz : 0.0;
    S->rz = rz;
    if (S->kerr) {
        S->status = ST_TIMEOUT;
        S->done = 1;
    } else if (!isfinite(rr) || !isfinite(rz)) {
        S->status = ST_NAN;
        S->done = 1;
    } else if (rr < S->thr) {
        S->status = ST_CONVERGED;
        S->done = 1;
    } else if (rr < S->thr_update) {
        S->status = ST_UPDATE;
        S->done = 1;
    } else if (S->it >= S->maxit) {
        S->status = ST_MAXIT;
        S->done = 1;
    }
    S->cnt_upd = 0;
}

// FP64 PCG: x += alpha p; r -= alpha q; r.r and r.z partials.  p is the buffer
// the K*u kernel of this iteration wrote: p[(it + 1) & 1] of the ping-pong pair.
template <typename T>
__device__ __forceinline__ void pcg_update_body(Layout L, double *__restrict__ x, T *__restrict__ r, const T *pa, const T *pb,
                      const T *__restrict__ q, const T *__restrict__ dinv, double *partial,
                      Scalars *S, const Blk B) {
    __shared__ double red[2 * (VEC_THREADS / 32)];
    __shared__ int last_flag;
    if (S->done) return;
    const T alpha = (T)S->alpha;
    const T *__restrict__ p = (S->it & 1) ? pa : pb;
    const long long cs = L.cs;
    Acc<T> a0, a1;
    // one node per thread and step, its three component planes
    for (long long n = B.b * (long long)blockDim.x + threadIdx.x; n < cs;
         n += (long long)B.n * blockDim.x) {
        const T d = dinv[n];
        T xv[3], rv[3], pv[3], qv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long i = n + c * cs;
            xv[c] = x[i];
            rv[c] = r[i];
            pv[c] = p[i];
            qv[c] = q[i];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long i = n + c * cs;
            const T xi = xv[c] + alpha * pv[c];
            const T ri = rv[c] - alpha * qv[c];
            x[i] = xi;
            r[i] = ri;
            a0.add_prod(ri, ri);
            a1.add_prod(ri, d * ri);
        }
    }
    double v[2] = {a0.value(), a1.value()};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        partial[2 * B.b] = v[0];
        partial[2 * B.b + 1] = v[1];
    }
    if (!arrive_last_n(&S->cnt_upd, &last_flag, B.n)) return;
    double tot[2];
    reduce_partials<2>(partial, B.n, 2, tot, red);
    if (threadIdx.x == 0) pcg_update_finish(S, tot[0], tot[1]);
}
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS)
    pcg_update_kernel(Layout L, double *__restrict__ x, T *__restrict__ r, const T *pa, const T *pb,
                      const T *__restrict__ q, const T *__restrict__ dinv, double *partial,
                      Scalars *S) {
    pcg_update_body<T>(L, x, r, pa, pb, q, dinv, partial, S, grid_blk());
}

template <typename T>
cudaError_t pcg_update(const Layout &L, double *x, T *r, const T *pa, const T *pb, const T *q, const T *dinv,
                       double *partial, Scalars *S, int nblocks, cudaStream_t st) {
    pcg_update_kernel<T><<<nblocks, VEC_THREADS, 0, st>>>(L, x, r, pa, pb, q, dinv, partial, S);
    return counted(cudaGetLastError());
}
template cudaError_t pcg_update<double>(const Layout &, double *, double *, const double *, const double *,
                                        const double *, const double *, double *, Scalars *, int, cudaStream_t);

// ---- FP32 PCG update with a double-float iterate, staged by bulk copies ------
// The iterate is the unevaluated sum xh + xl of two FP32 vectors (~48 bits, the
// same 8 bytes per DOF as FP64).  x += alpha p is an exact product (the FMA
// error term) and a TwoSum (Knuth) on the FP32 pipes, because GB300's FP64 pipe
// (2 DFMA per clock and SM) would take ~19 us per launch for the FMAs and the
// FP32 -> FP64 conversions of a 5.4M-DOF grid.  (Adding the rounded product
// instead cost 10 % more inner iterations on the 192x96x96 bracket.)
// The iterate is folded every second iteration: an even iteration k only updates
// r and owes alpha_k p_k to x (kept in Scalars::alpha_prev); the odd iteration
// k+1 adds alpha_k p_k and alpha_{k+1} p_{k+1} in that order -- the same two
// TwoSum steps, so x is bitwise that of a per-iteration update -- and a solve
// that stops after an even iteration settles the debt with pcg_df_settle.  An
// even iteration moves 40 bytes per DOF, an odd one 112 (76 on average instead
// of 100).
// The streams are read in chunks by bulk asynchronous copies into shared memory:
// on a folding iteration 7 streams (xh, xl, r, p_prev, p, q and the node's D^-1),
// otherwise 3 (r, q, D^-1), two chunks in flight per CTA (96-112 KB of reads)
// without registers.
constexpr int UPD_K = 2048;  // DOFs per chunk of the batched update (a multiple of 64, as cs is)
constexpr int UPD_SMEM = 14 * 4 * UPD_K;  // shared memory of either update: 112 KB, two CTAs per SM
// single-problem update: two stages of chunks, 2048 DOFs x 7 streams on odd
// iterations, 4096 DOFs x 3 streams on even ones (1024-DOF chunks in 4 / 9 stages
// were slower: 40.9 / 26.2 us against 39.4 / 23.7 us on the 192x96x96 bracket)
constexpr int UPD1_ST = 2;

// (hi, lo) += a * b, the product added exactly (its FMA rounding error joins lo)
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float a, float b) {
    const float pr = a * b;
    const float pe = fmaf(a, b, -pr);
    const float s = hi + pr;
    const float v = s - hi;
    const float e = (hi - (s - v)) + (pr - v);
    const float l = lo + (e + pe);
    hi = s + l;
    lo = l - (hi - s);
}

template <bool FOLD>
__device__ __forceinline__ void pcg_update_df_body(const Layout &L, float *__restrict__ xh, float *__restrict__ xl,
                                                   float *__restrict__ r, const float *__restrict__ p_prev,
                                                   const float *__restrict__ p, const float *__restrict__ q,
                                                   const float *__restrict__ dinv, double *partial, Scalars *S,
                                                   float alpha_prev, float alpha, unsigned char *smem,
                                                   uint64_t *bar, double *red, int &last_flag, int &fail) {
    constexpr int NP = FOLD ? 7 : 3;          // streams per chunk
    constexpr int NST = UPD1_ST;              // stages
    constexpr int UPD1_K = FOLD ? 2048 : 4096;  // DOFs per chunk
    static_assert(NST * NP * 4 * UPD1_K <= UPD_SMEM, "update stages exceed the shared memory");
    // plane index of each stream within a stage
    constexpr int P_R = FOLD ? 2 : 0, P_Q = FOLD ? 5 : 1, P_D = FOLD ? 6 : 2;
    const long long cs = L.cs;
    const int nck = (int)((cs + UPD1_K - 1) / UPD1_K);
    const int nchunks = 3 * nck;
    auto plane = [&](int s, int a) {
        return reinterpret_cast<float *>(smem + ((size_t)s * NP + a) * 4 * UPD1_K);
    };
    auto chunk = [&](int g, long long &o, long long &j0, int &len) {
        const int c = g / nck;
        j0 = (long long)(g - c * nck) * UPD1_K;
        len = (int)min((long long)UPD1_K, cs - j0);
        o = c * cs + j0;
    };
    auto issue = [&](int g, int s) {
        long long o, j0;
        int len;
        chunk(g, o, j0, len);
        const unsigned b = 4u * (unsigned)len;
        bulk::bar_expect(&bar[s], (unsigned)NP * b);
        if (FOLD) {
            bulk::copy_g2s(plane(s, 0), xh + o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 1), xl + o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 3), p_prev + o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 4), p + o, b, &bar[s]);
        }
        bulk::copy_g2s(plane(s, P_R), r + o, b, &bar[s]);
        bulk::copy_g2s(plane(s, P_Q), q + o, b, &bar[s]);
        bulk::copy_g2s(plane(s, P_D), dinv + j0, b, &bar[s]);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) bulk::bar_init(&bar[s], 1);
        bulk::bar_init_fence();
        fail = 0;
    }
    __syncthreads();
    // this CTA's chunks: blockIdx.x + i * gridDim.x, i < mine
    const int mine = max(0, (nchunks - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x);
    if (threadIdx.x == 0)
        for (int i = 0; i < NST && i < mine; ++i) issue(blockIdx.x + i * gridDim.x, i);
    Acc<float> a0, a1;
    int i = 0;
    for (; i < mine; ++i) {
        const int s = i % NST;
        if (!bulk::bar_wait(&bar[s], (unsigned)(i / NST) & 1u)) fail = 1;
        __syncthreads();
        if (fail) break;
        long long o, j0;
        int len;
        chunk(blockIdx.x + i * gridDim.x, o, j0, len);
        const float4 *rs = reinterpret_cast<const float4 *>(plane(s, P_R));
        const float4 *qs = reinterpret_cast<const float4 *>(plane(s, P_Q));
        const float4 *ds = reinterpret_cast<const float4 *>(plane(s, P_D));
        for (int t = threadIdx.x; t < len / 4; t += VEC_THREADS) {
            float4 rv = rs[t];
            const float4 qv = qs[t], d = ds[t];
            if (FOLD) {
                float4 h = reinterpret_cast<const float4 *>(plane(s, 0))[t];
                float4 l = reinterpret_cast<const float4 *>(plane(s, 1))[t];
                const float4 pp = reinterpret_cast<const float4 *>(plane(s, 3))[t];
                const float4 pv = reinterpret_cast<const float4 *>(plane(s, 4))[t];
                two_sum_acc(h.x, l.x, alpha_prev, pp.x);
                two_sum_acc(h.y, l.y, alpha_prev, pp.y);
                two_sum_acc(h.z, l.z, alpha_prev, pp.z);
                two_sum_acc(h.w, l.w, alpha_prev, pp.w);
                two_sum_acc(h.x, l.x, alpha, pv.x);
                two_sum_acc(h.y, l.y, alpha, pv.y);
                two_sum_acc(h.z, l.z, alpha, pv.z);
                two_sum_acc(h.w, l.w, alpha, pv.w);
                reinterpret_cast<float4 *>(xh + o)[t] = h;
                reinterpret_cast<float4 *>(xl + o)[t] = l;
            }
            rv.x = fmaf(-alpha, qv.x, rv.x);
            rv.y = fmaf(-alpha, qv.y, rv.y);
            rv.z = fmaf(-alpha, qv.z, rv.z);
            rv.w = fmaf(-alpha, qv.w, rv.w);
            reinterpret_cast<float4 *>(r + o)[t] = rv;
            // r.r and r.D^-1 r: the four non-negative terms of a float4 summed in
            // FP32 (no cancellation: within a few ulps), the float4 sums in
            // double-float
            a0.add(fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, rv.w * rv.w))));
            a1.add(fmaf(rv.x, d.x * rv.x, fmaf(rv.y, d.y * rv.y, fmaf(rv.z, d.z * rv.z, rv.w * (d.w * rv.w)))));
        }
        __syncthreads();  // stage s read by every thread
        if (threadIdx.x == 0 && i + NST < mine) {
            bulk::proxy_fence();
            issue(blockIdx.x + (i + NST) * gridDim.x, s);
        }
    }
    if (fail) {
        // a copy did not complete within its wait: drain this CTA's outstanding
        // copies (bounded), flag the launch, and still take part in the reduction
        if (threadIdx.x == 0) {
            for (int j = i; j < mine && j < i + NST; ++j) bulk::bar_wait(&bar[j % NST], (unsigned)(j / NST) & 1u);
            atomicExch(&S->kerr, 1);
        }
    }
    double v[2] = {a0.value(), a1.value()};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = v[0];
        partial[2 * blockIdx.x + 1] = v[1];
    }
    if (!arrive_last_n(&S->cnt_upd, &last_flag, gridDim.x)) return;
    double tot[2];
    reduce_partials<2>(partial, gridDim.x, 2, tot, red);
    if (threadIdx.x == 0) {
        // an even iteration leaves alpha_k p_k owed to x; an odd one paid it
        S->alpha_prev = FOLD ? 0.0 : S->alpha;
        pcg_update_finish(S, tot[0], tot[1]);
    }
}

__global__ void __launch_bounds__(VEC_THREADS)
    pcg_update_df_kernel(Layout L, float *__restrict__ xh, float *__restrict__ xl, float *__restrict__ r,
                         const float *pa, const float *pb, const float *__restrict__ q,
                         const float *__restrict__ dinv, double *partial, Scalars *S) {
    extern __shared__ __align__(128) unsigned char upd_smem[];
    __shared__ uint64_t bar[UPD1_ST];
    __shared__ double red[2 * (VEC_THREADS / 32)];
    __shared__ int last_flag, fail;
    if (S->done) return;
    const int it = S->it;
    const float alpha = (float)S->alpha;
    // p of this iteration is the ping-pong member its K*u wrote, p_prev the other
    const float *p = (it & 1) ? pa : pb;
    const float *p_prev = (it & 1) ? pb : pa;
    if (it & 1)
        pcg_update_df_body<true>(L, xh, xl, r, p_prev, p, q, dinv, partial, S, (float)S->alpha_prev, alpha,
                                 upd_smem, bar, red, last_flag, fail);
    else
        pcg_update_df_body<false>(L, xh, xl, r, p_prev, p, q, dinv, partial, S, 0.f, alpha, upd_smem, bar, red,
                                  last_flag, fail);
}

// x += alpha_prev p_prev when the last PCG iteration left that term owed (S->it
// odd): p_prev is the ping-pong member the last K*u wrote
__global__ void __launch_bounds__(VEC_THREADS)
    pcg_df_settle_kernel(long long n, float *__restrict__ xh, float *__restrict__ xl, const float *pa,
                         const float *pb, const Scalars *S) {
    const int it = S->it;
    if (!(it & 1)) return;
    const float a = (float)S->alpha_prev;
    const float *p = (it & 1) ? pb : pa;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float h = xh[i], l = xl[i];
        two_sum_acc(h, l, a, p[i]);
        xh[i] = h;
        xl[i] = l;
    }
}
cudaError_t pcg_df_settle(long long n, float *xh, float *xl, const float *pa, const float *pb, Scalars *S,
                          int nblocks, cudaStream_t st) {
    pcg_df_settle_kernel<<<nblocks, VEC_THREADS, 0, st>>>(n, xh, xl, pa, pb, S);
    cudaError_t e = counted(cudaGetLastError());
    if (e != cudaSuccess) return e;
    // paid: a later folding iteration must not add it again
    return cudaMemsetAsync(&S->alpha_prev, 0, sizeof(double), st);
}

static int g_upd_grid = 0;
__global__ void __launch_bounds__(256) b_update_df_kernel(const BatchItem *items, WorkList W);

cudaError_t pcg_update_df(const Layout &L, float *xh, float *xl, float *r, const float *pa, const float *pb,
                          const float *q, const float *dinv, double *partial, Scalars *S, cudaStream_t st) {
    if (g_upd_grid <= 0) return cudaErrorInitializationError;
    pcg_update_df_kernel<<<g_upd_grid, VEC_THREADS, UPD_SMEM, st>>>(L, xh, xl, r, pa, pb, q, dinv, partial, S);
    return counted(cudaGetLastError());
}
int pcg_update_df_grid() { return g_upd_grid; }

// two CTAs of UPD_SMEM bytes per SM, one wave
cudaError_t update_init_attributes() {
    cudaError_t e = cudaFuncSetAttribute(pcg_update_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, UPD_SMEM);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(b_update_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, UPD_SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    g_upd_grid = 2 * std::max(sms, 1);
    return cudaSuccess;
}

// reads n bytes (a multiple of 16) through L2; the sum is kept only to keep the loads
__global__ void l2_flush_read_kernel(const uint4 *__restrict__ a, long long n16, unsigned *sink) {
    unsigned acc = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n16;
         i += (long long)gridDim.x * blockDim.x) {
        const uint4 v = __ldcg(a + i);
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (acc == 0x9e3779b9u) *sink = acc;
}
cudaError_t l2_flush_read(const void *buf, size_t bytes, cudaStream_t st) {
    // the sink is the buffer's first word: written only on an (irrelevant) hash match
    l2_flush_read_kernel<<<1216, 256, 0, st>>>(reinterpret_cast<const uint4 *>(buf), (long long)(bytes / 16),
                                               reinterpret_cast<unsigned *>(const_cast<void *>(buf)));
    return counted(cudaGetLastError());
}

// x64 = xh + xl (exact), and the split x64 -> (xh, xl) with xh = (float)x64
__global__ void df_compose_kernel(const float *__restrict__ xh, const float *__restrict__ xl,
                                  double *__restrict__ x, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        x[i] = (double)xh[i] + (double)xl[i];
}
__global__ void df_accumulate_kernel(const float *__restrict__ xh, const float *__restrict__ xl,
                                     double *__restrict__ x, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        x[i] += (double)xh[i] + (double)xl[i];
}
cudaError_t df_accumulate(const float *xh, const float *xl, double *x, long long n, int nblocks, cudaStream_t st) {
    df_accumulate_kernel<<<nblocks, 256, 0, st>>>(xh, xl, x, n);
    return counted(cudaGetLastError());
}
__global__ void df_split_kernel(const double *__restrict__ x, float *__restrict__ xh, float *__restrict__ xl,
                                long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float h = (float)x[i];
        xh[i] = h;
        xl[i] = (float)(x[i] - (double)h);
    }
}
cudaError_t df_compose(const float *xh, const float *xl, double *x, long long n, int nblocks, cudaStream_t st) {
    df_compose_kernel<<<nblocks, 256, 0, st>>>(xh, xl, x, n);
    return counted(cudaGetLastError());
}
cudaError_t df_split(const double *x, float *xh, float *xl, long long n, int nblocks, cudaStream_t st) {
    df_split_kernel<<<nblocks, 256, 0, st>>>(x, xh, xl, n);
    return counted(cudaGetLastError());
}

// (Re)start of the PCG sequence from the residual in r: r.r, r.z -> S.
// restart == 0: fresh sequence (beta = 0, it = 0).  restart == 1: the residual
// was replaced by a recomputed one; the search direction is kept and
// beta = r.z / (r.z of the previous iteration).  restart == 2: iteration count
// kept, beta = 0 (steepest-descent restart after a breakdown).  thr: |r|^2 that ends the
// sequence; upd_factor: a reliable update is requested when |r|^2 falls below
// upd_factor * (this |r|^2) (0 disables).  maxit caps S->it.
template <typename T>
__device__ __forceinline__ void pcg_start_body(Layout L, const T *__restrict__ r, const T *__restrict__ dinv, double thr,
                     double upd_factor, int maxit, int restart, double *partial, Scalars *S, const Blk B) {
    __shared__ double red[2 * (VEC_THREADS / 32)];
    __shared__ int last_flag;
    const long long cs = L.cs;
    Acc<T> a0, a1;
    for (long long n = B.b * (long long)blockDim.x + threadIdx.x; n < cs;
         n += (long long)B.n * blockDim.x) {
        const T d = dinv[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T ri = r[n + c * cs];
            a0.add_prod(ri, ri);
            a1.add_prod(ri, d * ri);
        }
    }
    double v[2] = {a0.value(), a1.value()};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        partial[2 * B.b] = v[0];
        partial[2 * B.b + 1] = v[1];
    }
    if (!arrive_last_n(&S->cnt_upd, &last_flag, B.n)) return;
    double tot[2];
    reduce_partials<2>(partial, B.n, 2, tot, red);
    if (threadIdx.x == 0) {
        S->rr = tot[0];
        if (restart == 1) {
            S->beta = (S->rz_prev > 0.0) ? tot[1] / S->rz_prev : 0.0;
        } else if (restart == 2) {
            S->beta = 0.0;
        } else {
            S->beta = 0.0;
            S->it = 0;
            S->rz_prev = 0.0;
        }
        S->rz = tot[1];
        S->thr = thr >= 0.0 ? thr : -thr * tot[0];  // negative: relative to this |r|^2
        S->thr_update = upd_factor * tot[0];
        S->alpha = 0.0;
        S->alpha_prev = 0.0;  // no iterate term owed at a (re)start
        S->maxit = maxit;
        S->status = ST_RUNNING;
        S->done = 0;
        if (!isfinite(tot[0])) {
            S->status = ST_NAN;
            S->done = 1;
        } else if (tot[0] < S->thr || tot[0] == 0.0) {
            S->status = ST_CONVERGED;
            S->done = 1;
        } else if (S->it >= maxit) {
            S->status = ST_MAXIT;
            S->done = 1;
        }
        S->cnt_upd = 0;
    }
}
template <typename T>
__global__ void __launch_bounds__(VEC_THREADS)
    pcg_start_kernel(Layout L, const T *__restrict__ r, const T *__restrict__ dinv, double thr,
                     double upd_factor, int maxit, int restart, double *partial, Scalars *S) {
    pcg_start_body<T>(L, r, dinv, thr, upd_factor, maxit, restart, partial, S, grid_blk());
}

template <typename T>
cudaError_t pcg_start(const Layout &L, const T *r, const T *dinv, double thr, double upd_factor, int maxit,
                      int restart, double *partial, Scalars *S, int nblocks, cudaStream_t st) {
    pcg_start_kernel<T><<<nblocks, VEC_THREADS, 0, st>>>(L, r, dinv, thr, upd_factor, maxit, restart, partial, S);
    return counted(cudaGetLastError());
}
template cudaError_t pcg_start<float>(const Layout &, const float *, const float *, double, double, int, int,
                                      double *, Scalars *, int, cudaStream_t);
template cudaError_t pcg_start<double>(const Layout &, const double *, const double *, double, double, int, int,
                                       double *, Scalars *, int, cudaStream_t);

// r32 = r64 and (x != nullptr) x = 0
__device__ __forceinline__ void dc_inner_init_body(Layout L, const double *__restrict__ r64, float *__restrict__ r32,
                                     double *__restrict__ x, const Scalars *S, const Blk B) {
    (void)S;
    const long long n = 3 * L.cs;
    for (long long i = B.b * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)B.n * blockDim.x) {
        r32[i] = (float)r64[i];
        if (x) x[i] = 0.0;
    }
}
__global__ void dc_inner_init_kernel(Layout L, const double *__restrict__ r64, float *__restrict__ r32,
                                     double *__restrict__ x, const Scalars *S) {
    dc_inner_init_body(L, r64, r32, x, S, grid_blk());
}
cudaError_t dc_inner_init(const Layout &L, const double *r64, float *r32, double *x,
                          const Scalars *S, int nblocks, cudaStream_t st) {
    dc_inner_init_kernel<<<nblocks, VEC_THREADS, 0, st>>>(L, r64, r32, x, S);
    return counted(cudaGetLastError());
}

__global__ void to_float_kernel(const double *__restrict__ a, float *__restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
cudaError_t to_float(const double *a, float *b, long long n, int nblocks, cudaStream_t st) {
    to_float_kernel<<<nblocks, 256, 0, st>>>(a, b, n);
    return counted(cudaGetLastError());
}

// r32 = mask(r64 - q32): the residual left by an initial guess with K x = q
__global__ void inner_resid_kernel(Layout L, const double *__restrict__ r64, const float *__restrict__ q32,
                                   const uint8_t *__restrict__ mask, float *__restrict__ r32) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const unsigned m = mask[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long i = n + c * L.cs;
            r32[i] = ((m >> c) & 1u) ? 0.f : (float)(r64[i] - (double)q32[i]);
        }
    }
}
cudaError_t inner_resid(const Layout &L, const double *r64, const float *q32, const uint8_t *mask, float *r32,
                        int nblocks, cudaStream_t st) {
    inner_resid_kernel<<<nblocks, 256, 0, st>>>(L, r64, q32, mask, r32);
    return counted(cudaGetLastError());
}

// x = 0 on the constrained / orphan components (bit c of mask[n] set)
__device__ __forceinline__ void zero_masked_body(Layout L, const uint8_t *__restrict__ mask, double *__restrict__ x, const Blk B) {
    const long long cs = L.cs;
    for (long long n = B.b * (long long)blockDim.x + threadIdx.x; n < cs;
         n += (long long)B.n * blockDim.x) {
        const unsigned m = mask[n];
        if (!m) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if ((m >> c) & 1u) x[n + c * cs] = 0.0;
    }
}
__global__ void zero_masked_kernel(Layout L, const uint8_t *__restrict__ mask, double *__restrict__ x) {
    zero_masked_body(L, mask, x, grid_blk());
}
// ---- outer flexible CG (FP64), preconditioned by an inner solve z = M(r) ------
// Flexible CG with one stored direction and the Polak-Ribiere beta
// (Notay, SIAM J. Sci. Comput. 22 (2000)): beta = z_new.(r_new - r_old) / z_old.r_old,
// and r_new - r_old = -alpha q, so beta = -alpha z_new.q / z_old.r_old.
__global__ void __launch_bounds__(VEC_THREADS)
    fcg_dots_kernel(Layout L, const double *__restrict__ z, const double *__restrict__ r,
                    const double *__restrict__ q, int first, double *partial, Scalars *S) {
    __shared__ double red[2 * (VEC_THREADS / 32)];
    __shared__ int last_flag;
    const long long n = 3 * L.cs;
    double zr = 0.0, zq = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double zi = z[i];
        zr = fma(zi, r[i], zr);
        if (!first) zq = fma(zi, q[i], zq);
    }
    double v[2] = {zr, zq};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = v[0];
        partial[2 * blockIdx.x + 1] = v[1];
    }
    if (!arrive_last(&S->cnt_fcg, &last_flag)) return;
    double tot[2];
    reduce_partials<2>(partial, gridDim.x, 2, tot, red);
    if (threadIdx.x == 0) {
        S->o_beta = (first || S->o_zr == 0.0) ? 0.0 : -S->o_alpha * tot[1] / S->o_zr;
        S->o_zr = tot[0];
        S->o_zq = tot[1];
        S->cnt_fcg = 0;
    }
}
cudaError_t fcg_dots(const Layout &L, const double *z, const double *r, const double *q, int first,
                     double *partial, Scalars *S, int nblocks, cudaStream_t st) {
    fcg_dots_kernel<<<nblocks, VEC_THREADS, 0, st>>>(L, z, r, q, first, partial, S);
    return counted(cudaGetLastError());
}

// p = z + beta p
__global__ void fcg_direction_kernel(Layout L, const double *__restrict__ z, double *__restrict__ p,
                                     const Scalars *S) {
    const double beta = S->o_beta;
    const long long n = 3 * L.cs;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p[i] = beta == 0.0 ? z[i] : fma(beta, p[i], z[i]);
}
cudaError_t fcg_direction(const Layout &L, const double *z, double *p, const Scalars *S, int nblocks,
                          cudaStream_t st) {
    fcg_direction_kernel<<<nblocks, VEC_THREADS, 0, st>>>(L, z, p, S);
    return counted(cudaGetLastError());
}

// x += alpha p; r -= alpha q; r.r -> S->o_rr
__global__ void __launch_bounds__(VEC_THREADS)
    fcg_update_kernel(Layout L, double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                      const double *__restrict__ q, double *partial, Scalars *S) {
    __shared__ double red[VEC_THREADS / 32];
    __shared__ int last_flag;
    const double alpha = S->o_alpha;
    const long long n = 3 * L.cs;
    double rr = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double pi = p[i], qi = q[i], xi = x[i], ri = r[i];
        x[i] = fma(alpha, pi, xi);
        const double rn = fma(-alpha, qi, ri);
        r[i] = rn;
        rr = fma(rn, rn, rr);
    }
    double v[1] = {rr};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = v[0];
    if (!arrive_last(&S->cnt_fcg, &last_flag)) return;
    double tot[1];
    reduce_partials<1>(partial, gridDim.x, 1, tot, red);
    if (threadIdx.x == 0) {
        S->o_rr = tot[0];
        S->cnt_fcg = 0;
    }
}
cudaError_t fcg_update(const Layout &L, double *x, double *r, const double *p, const double *q, double *partial,
                       Scalars *S, int nblocks, cudaStream_t st) {
    fcg_update_kernel<<<nblocks, VEC_THREADS, 0, st>>>(L, x, r, p, q, partial, S);
    return counted(cudaGetLastError());
}

cudaError_t zero_masked(const Layout &L, const uint8_t *mask, double *x, int nblocks, cudaStream_t st) {
    zero_masked_kernel<<<nblocks, VEC_THREADS, 0, st>>>(L, mask, x);
    return counted(cudaGetLastError());
}

// ============================================================================
// set-up kernels
// ============================================================================
__device__ __forceinline__ double pow_fast(double x, double p) {
    // integer exponents in [0, 8] by repeated multiplication, else pow
    if (p == floor(p) && p >= 0.0 && p <= 8.0) {
        const int k = (int)p;
        double r = 1.0;
        for (int i = 0; i < k; ++i) r *= x;
        return r;
    }
    return pow(x, p);
}

__device__ __forceinline__ void scales_body(Layout L, const double *__restrict__ rho, const int8_t *__restrict__ grid,
                              int variant, double p, double emin, double rho_min, double E,
                              double *__restrict__ s64, float *__restrict__ s32, int d1, const Blk B) {
    for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < L.nel;
         e += (long long)B.n * blockDim.x) {
        const int g = grid ? grid[e] : 0;
        long long src = e;
        if (d1) {
            // the reference C++ assembler's density index i*ny*nz + j*nz + k
            // applied to the optimizer's x-fastest vector (global_assembler.hpp:162-164)
            const long long ex = e % L.nx, ey = (e / L.nx) % L.ny, ez = e / ((long long)L.nx * L.ny);
            src = (ex * L.ny + ey) * L.nz + ez;
        }
        const double r = rho[src];
        double v;
        if (variant == 0) {
            if (g == -1 || r < rho_min) v = 0.0;
            else if (g == 1) v = 1.0;
            else v = emin + pow_fast(r, p) * (1.0 - emin);
        } else {
            if (g == -1) v = 0.0;
            else if (g == 1) v = 1.0;
            else v = (emin + pow_fast(r, p) * (E - emin)) / E;
        }
        if (s64) s64[e] = v;
        if (s32) s32[e] = (float)v;
    }
}
__global__ void scales_kernel(Layout L, const double *__restrict__ rho, const int8_t *__restrict__ grid,
                              int variant, double p, double emin, double rho_min, double E,
                              double *__restrict__ s64, float *__restrict__ s32, int d1) {
    scales_body(L, rho, grid, variant, p, emin, rho_min, E, s64, s32, d1, grid_blk());
}
cudaError_t scales(const Layout &L, const double *rho, const int8_t *grid, int variant, double p,
                   double emin, double rho_min, double E, double *s64, float *s32, cudaStream_t st, int d1) {
    const int nb = std::max(1, std::min(div_up(L.nel, 256), 152 * 16));
    scales_kernel<<<nb, 256, 0, st>>>(L, rho, grid, variant, p, emin, rho_min, E, s64, s32, d1);
    return counted(cudaGetLastError());
}

__device__ __forceinline__ void diag_mask_body(Layout L, const double *__restrict__ s, double d0,
                                 const uint8_t *__restrict__ fixed_bits, double *__restrict__ dinv64,
                                 float *__restrict__ dinv32, uint8_t *__restrict__ mask, const Blk B) {
    const long long nn = L.sxy * (L.nz + 1);
    for (long long n = B.b * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)B.n * blockDim.x) {
        const int iz = (int)(n / L.sxy);
        const long long rem = n - (long long)iz * L.sxy;
        const int iy = (int)(rem / L.sx), ix = (int)(rem - (long long)iy * L.sx);
        if (ix > L.nx) continue;  // padding column
        double acc = 0.0;
        for (int dz = -1; dz <= 0; ++dz) {
            const int ez = iz + dz;
            if (ez < 0 || ez >= L.nz) continue;
            for (int dy = -1; dy <= 0; ++dy) {
                const int ey = iy + dy;
                if (ey < 0 || ey >= L.ny) continue;
                for (int dx = -1; dx <= 0; ++dx) {
                    const int ex = ix + dx;
                    if (ex < 0 || ex >= L.nx) continue;
                    acc += s[elem_index(L, ex, ey, ez)];
                }
            }
        }
        const double dg = d0 * acc;
        const bool orphan = fabs(dg) < 1e-15;
        uint8_t m = fixed_bits ? fixed_bits[n] : 0;
        if (orphan) m = 7;
        mask[n] = m;
        const double di = orphan ? 0.0 : 1.0 / dg;
        if (dinv64) dinv64[n] = di;
        if (dinv32) dinv32[n] = (float)di;
    }
}
__global__ void diag_mask_kernel(Layout L, const double *__restrict__ s, double d0,
                                 const uint8_t *__restrict__ fixed_bits, double *__restrict__ dinv64,
                                 float *__restrict__ dinv32, uint8_t *__restrict__ mask) {
    diag_mask_body(L, s, d0, fixed_bits, dinv64, dinv32, mask, grid_blk());
}
cudaError_t diag_mask(const Layout &L, const double *s64, double d0, const uint8_t *fixed_bits,
                      double *dinv64, float *dinv32, uint8_t *mask, cudaStream_t st) {
    const long long nn = L.sxy * (L.nz + 1);
    const int nb = std::max(1, std::min(div_up(nn, 256), 152 * 16));
    diag_mask_kernel<<<nb, 256, 0, st>>>(L, s64, d0, fixed_bits, dinv64, dinv32, mask);
    return counted(cudaGetLastError());
}

// ============================================================================
// layout conversions
// ============================================================================
template <typename T>
__global__ void dof_to_dev_kernel(Layout L, const double *__restrict__ src, T *__restrict__ dst) {
    const long long nn = (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        // n enumerates reference node ids (i slowest, k fastest)
        const int k = (int)(n % (L.nz + 1));
        const long long t = n / (L.nz + 1);
        const int j = (int)(t % (L.ny + 1)), i = (int)(t / (L.ny + 1));
        const long long d = node_index(L, i, j, k);
        dst[d] = (T)src[3 * n];
        dst[d + L.cs] = (T)src[3 * n + 1];
        dst[d + 2 * L.cs] = (T)src[3 * n + 2];
    }
}
template <typename T>
__global__ void dev_to_dof_kernel(Layout L, const T *__restrict__ src, double *__restrict__ dst) {
    const long long nn = (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(n % (L.nz + 1));
        const long long t = n / (L.nz + 1);
        const int j = (int)(t % (L.ny + 1)), i = (int)(t / (L.ny + 1));
        const long long d = node_index(L, i, j, k);
        dst[3 * n] = (double)src[d];
        dst[3 * n + 1] = (double)src[d + L.cs];
        dst[3 * n + 2] = (double)src[d + 2 * L.cs];
    }
}
template <typename T>
cudaError_t dof_to_dev_t(const Layout &L, const double *src, T *dst, cudaStream_t st) {
    const long long nn = (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    dof_to_dev_kernel<T><<<std::max(1, std::min(div_up(nn, 256), 152 * 16)), 256, 0, st>>>(L, src, dst);
    return counted(cudaGetLastError());
}
template <typename T>
cudaError_t dev_to_dof_t(const Layout &L, const T *src, double *dst, cudaStream_t st) {
    const long long nn = (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    dev_to_dof_kernel<T><<<std::max(1, std::min(div_up(nn, 256), 152 * 16)), 256, 0, st>>>(L, src, dst);
    return counted(cudaGetLastError());
}
template cudaError_t dof_to_dev_t<float>(const Layout &, const double *, float *, cudaStream_t);
template cudaError_t dof_to_dev_t<double>(const Layout &, const double *, double *, cudaStream_t);
template cudaError_t dev_to_dof_t<float>(const Layout &, const float *, double *, cudaStream_t);
template cudaError_t dev_to_dof_t<double>(const Layout &, const double *, double *, cudaStream_t);
cudaError_t dof_to_dev(const Layout &L, const double *src, double *dst, cudaStream_t st) {
    return dof_to_dev_t<double>(L, src, dst, st);
}
cudaError_t dev_to_dof(const Layout &L, const double *src, double *dst, cudaStream_t st) {
    return dev_to_dof_t<double>(L, src, dst, st);
}

template <typename T>
__global__ void elem_conv_kernel(Layout L, const T *__restrict__ src, T *__restrict__ dst, int layout,
                                 int to_dev) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < L.nel;
         e += (long long)gridDim.x * blockDim.x) {
        // e enumerates internal (x-fastest) elements
        const int ex = (int)(e % L.nx);
        const long long t = e / L.nx;
        const int ey = (int)(t % L.ny), ez = (int)(t / L.ny);
        const long long h = layout == 0 ? ((long long)ex * L.ny + ey) * L.nz + ez : e;
        if (to_dev) dst[e] = src[h];
        else dst[h] = src[e];
    }
}
template <typename T>
cudaError_t elem_to_dev(const Layout &L, const T *src, T *dst, int layout, cudaStream_t st) {
    elem_conv_kernel<T><<<std::max(1, std::min(div_up(L.nel, 256), 152 * 16)), 256, 0, st>>>(L, src, dst,
                                                                                         layout, 1);
    return counted(cudaGetLastError());
}
template <typename T>
cudaError_t elem_from_dev(const Layout &L, const T *src, T *dst, int layout, cudaStream_t st) {
    elem_conv_kernel<T><<<std::max(1, std::min(div_up(L.nel, 256), 152 * 16)), 256, 0, st>>>(L, src, dst,
                                                                                         layout, 0);
    return counted(cudaGetLastError());
}
template cudaError_t elem_to_dev<double>(const Layout &, const double *, double *, int, cudaStream_t);
template cudaError_t elem_to_dev<int8_t>(const Layout &, const int8_t *, int8_t *, int, cudaStream_t);
template cudaError_t elem_to_dev<uint8_t>(const Layout &, const uint8_t *, uint8_t *, int, cudaStream_t);
template cudaError_t elem_from_dev<double>(const Layout &, const double *, double *, int, cudaStream_t);

// ============================================================================
// filters
// ============================================================================
template <typename T>
__device__ __forceinline__ void filter_cpp_body(Layout L, const int4 *__restrict__ td, const double *__restrict__ tw,
                                  int ntaps, const double *__restrict__ x, const double *__restrict__ rho,
                                  double *__restrict__ out, const Blk B) {
    for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < L.nel;
         e += (long long)B.n * blockDim.x) {
        const int ex = (int)(e % L.nx);
        const long long t = e / L.nx;
        const int ey = (int)(t % L.ny), ez = (int)(t / L.ny);
        T num = T(0), den = T(0);
        for (int k = 0; k < ntaps; ++k) {
            const int4 d = td[k];
            const int xx = ex + d.x, yy = ey + d.y, zz = ez + d.z;
            if (xx < 0 || xx >= L.nx || yy < 0 || yy >= L.ny || zz < 0 || zz >= L.nz) continue;
            const long long n = elem_index(L, xx, yy, zz);
            const T w = (T)tw[k];
            const T rn = (T)rho[n];
            num += w * rn * (T)x[n];
            den += w * rn;
        }
        out[e] = (den > T(1e-15)) ? (double)(num / den) : x[e];
    }
}
template <typename T>
__global__ void filter_cpp_kernel(Layout L, const int4 *__restrict__ td, const double *__restrict__ tw,
                                  int ntaps, const double *__restrict__ x, const double *__restrict__ rho,
                                  double *__restrict__ out) {
    filter_cpp_body<T>(L, td, tw, ntaps, x, rho, out, grid_blk());
}
// Shared-memory halo stencil (FP64): a CTA of 32 x 8 threads owns a tile of
// 32 x 8 x 4 elements (4 per thread along z) and first stages the tile plus a
// halo of R = ceil(rmin) elements in shared memory -- (rho, x) for the C++ rule,
// zero outside the grid (a zero term adds +0.0, so the sums equal the skipping
// loop's bit for bit), or the reflected value for the Python rule -- then every
// element sums its taps in the tap order from shared memory.
constexpr int FT_X = 32, FT_Y = 8, FT_Z = 4;
template <int R>
constexpr size_t filter_smem_bytes(int arrays) {
    return sizeof(double) * arrays * (FT_X + 2 * R) * (FT_Y + 2 * R) * (FT_Z + 2 * R);
}

__device__ __forceinline__ int reflect_idx(int i, int n);

template <int R, int VARIANT>
__global__ void __launch_bounds__(FT_X *FT_Y)
    filter_smem_kernel(Layout L, const int4 *__restrict__ td, const double *__restrict__ tw, int ntaps,
                       const double *__restrict__ x, const double *__restrict__ rho, double *__restrict__ out,
                       int mode, double lo) {
    extern __shared__ double fsm[];
    constexpr int HX = FT_X + 2 * R, HY = FT_Y + 2 * R, HZ = FT_Z + 2 * R, HN = HX * HY * HZ;
    double *sa = fsm;       // CPP: rho ; PY: the filtered quantity
    double *sb = fsm + HN;  // CPP: x
    const int tiles_x = (L.nx + FT_X - 1) / FT_X, tiles_y = (L.ny + FT_Y - 1) / FT_Y;
    int b = blockIdx.x;
    const int bx = b % tiles_x;
    b /= tiles_x;
    const int by = b % tiles_y, bz = b / tiles_y;
    const int x0 = bx * FT_X - R, y0 = by * FT_Y - R, z0 = bz * FT_Z - R;
    const int tid = threadIdx.y * FT_X + threadIdx.x;
    for (int i = tid; i < HN; i += FT_X * FT_Y) {
        const int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
        int gx = x0 + hx, gy = y0 + hy, gz = z0 + hz;
        if (VARIANT == 0) {
            double ra = 0.0, xb = 0.0;
            if (gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny && gz >= 0 && gz < L.nz) {
                const long long n = elem_index(L, gx, gy, gz);
                ra = rho[n];
                xb = x[n];
            }
            sa[i] = ra;
            sb[i] = xb;
        } else {
            const long long n = elem_index(L, reflect_idx(gx, L.nx), reflect_idx(gy, L.ny), reflect_idx(gz, L.nz));
            sa[i] = mode == 2 ? x[n] * rho[n] : x[n];
        }
    }
    __syncthreads();
    const int ex = bx * FT_X + threadIdx.x, ey = by * FT_Y + threadIdx.y;
    if (ex >= L.nx || ey >= L.ny) return;
    for (int k = 0; k < FT_Z; ++k) {
        const int ez = bz * FT_Z + k;
        if (ez >= L.nz) break;
        const int c = ((k + R) * HY + threadIdx.y + R) * HX + threadIdx.x + R;
        double num = 0.0, den = 0.0, acc = 0.0;
        for (int t = 0; t < ntaps; ++t) {
            const int4 d = __ldg(td + t);
            const double w = __ldg(tw + t);
            const int j = c + (d.z * HY + d.y) * HX + d.x;
            if (VARIANT == 0) {
                const double rn = sa[j];
                num += w * rn * sb[j];
                den += w * rn;
            } else {
                acc += w * sa[j];
            }
        }
        const long long e = elem_index(L, ex, ey, ez);
        if (VARIANT == 0) {
            out[e] = (den > 1e-15) ? num / den : x[e];
        } else {
            double o = acc;
            if (mode == 1) o = npmin(npmax(o, lo), 1.0);
            else if (mode == 2) o = o / npmax(rho[e], 1e-3);
            out[e] = o;
        }
    }
}

template <int VARIANT>
static bool launch_filter_smem(const Layout &L, const Taps &tp, const double *x, const double *rho, double *out,
                               int mode, double lo, cudaStream_t st, cudaError_t *err) {
    const int R = tp.R;
    if (R < 1 || R > 3) return false;
    const int tiles = ((L.nx + FT_X - 1) / FT_X) * ((L.ny + FT_Y - 1) / FT_Y) * ((L.nz + FT_Z - 1) / FT_Z);
    const dim3 blk(FT_X, FT_Y);
    const int arrays = VARIANT == 0 ? 2 : 1;
    switch (R) {
        case 1:
            filter_smem_kernel<1, VARIANT><<<tiles, blk, filter_smem_bytes<1>(arrays), st>>>(L, tp.d, tp.w, tp.n, x,
                                                                                            rho, out, mode, lo);
            break;
        case 2:
            filter_smem_kernel<2, VARIANT><<<tiles, blk, filter_smem_bytes<2>(arrays), st>>>(L, tp.d, tp.w, tp.n, x,
                                                                                            rho, out, mode, lo);
            break;
        default:
            filter_smem_kernel<3, VARIANT><<<tiles, blk, filter_smem_bytes<3>(arrays), st>>>(L, tp.d, tp.w, tp.n, x,
                                                                                            rho, out, mode, lo);
            break;
    }
    *err = counted(cudaGetLastError());
    return true;
}

cudaError_t filter_init_attributes() {
    cudaError_t e;
#define AMK_FATTR(R, V, A)                                                                                  \
    if ((e = cudaFuncSetAttribute(filter_smem_kernel<R, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                  (int)filter_smem_bytes<R>(A))) != cudaSuccess)                            \
        return e;
    AMK_FATTR(1, 0, 2)
    AMK_FATTR(2, 0, 2)
    AMK_FATTR(3, 0, 2)
    AMK_FATTR(1, 1, 1)
    AMK_FATTR(2, 1, 1)
    AMK_FATTR(3, 1, 1)
#undef AMK_FATTR
    return cudaSuccess;
}

template <typename T>
cudaError_t filter_cpp(const Layout &L, const Taps &tp, const double *x, const double *rho,
                       double *out, cudaStream_t st) {
    if constexpr (std::is_same<T, double>::value) {
        cudaError_t e;
        if (launch_filter_smem<0>(L, tp, x, rho, out, 0, 0.0, st, &e)) return e;
    }
    filter_cpp_kernel<T><<<std::max(1, std::min(div_up(L.nel, 256), 152 * 16)), 256, 0, st>>>(
        L, tp.d, tp.w, tp.n, x, rho, out);
    return counted(cudaGetLastError());
}
template cudaError_t filter_cpp<float>(const Layout &, const Taps &, const double *, const double *,
                                       double *, cudaStream_t);
template cudaError_t filter_cpp<double>(const Layout &, const Taps &, const double *, const double *,
                                        double *, cudaStream_t);

__device__ __forceinline__ int reflect_idx(int i, int n) {
    const int period = 2 * n;
    int m = i % period;
    if (m < 0) m += period;
    return (m >= n) ? period - 1 - m : m;
}

template <typename T>
__global__ void filter_py_kernel(Layout L, const int4 *__restrict__ td, const double *__restrict__ tw,
                                 int ntaps, const double *__restrict__ x, const double *__restrict__ rho,
                                 double *__restrict__ out, int mode, double lo) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < L.nel;
         e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(e % L.nx);
        const long long t = e / L.nx;
        const int ey = (int)(t % L.ny), ez = (int)(t / L.ny);
        T acc = T(0);
        for (int k = 0; k < ntaps; ++k) {
            const int4 d = td[k];
            const long long n = elem_index(L, reflect_idx(ex + d.x, L.nx), reflect_idx(ey + d.y, L.ny),
                                           reflect_idx(ez + d.z, L.nz));
            T v = (T)x[n];
            if (mode == 2) v = (T)(x[n] * rho[n]);
            acc += (T)tw[k] * v;
        }
        double o = (double)acc;
        if (mode == 1) o = npmin(npmax(o, lo), 1.0);
        else if (mode == 2) o = o / npmax(rho[e], 1e-3);
        out[e] = o;
    }
}
template <typename T>
cudaError_t filter_py(const Layout &L, const Taps &tp, const double *x, const double *rho,
                      double *out, int mode, double lo, cudaStream_t st) {
    if constexpr (std::is_same<T, double>::value) {
        cudaError_t e;
        if (launch_filter_smem<1>(L, tp, x, rho, out, mode, lo, st, &e)) return e;
    }
    filter_py_kernel<T><<<std::max(1, std::min(div_up(L.nel, 256), 152 * 16)), 256, 0, st>>>(
        L, tp.d, tp.w, tp.n, x, rho, out, mode, lo);
    return counted(cudaGetLastError());
}
template cudaError_t filter_py<float>(const Layout &, const Taps &, const double *, const double *,
                                      double *, int, double, cudaStream_t);
template cudaError_t filter_py<double>(const Layout &, const Taps &, const double *, const double *,
                                       double *, int, double, cudaStream_t);

// ============================================================================
// sensitivities
// ============================================================================
__device__ __forceinline__ void sens_body(Layout L, const double *__restrict__ rho, const double *__restrict__ ce,
                const double *__restrict__ s, const uint8_t *__restrict__ design, int variant,
                double p, double *__restrict__ dc, int accumulate, double *partial, Scalars *S, const Blk B) {
    __shared__ double red[256 / 32];
    __shared__ int last_flag;
    double en = 0.0;
    for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < L.nel;
         e += (long long)B.n * blockDim.x) {
        const double c = ce[e];
        en = fma(s[e], c, en);  // void elements have s = 0
        if (variant == 0) {
            dc[e] = -p * pow_fast(rho[e], p - 1.0) * c;
        } else {
            double d = design[e] ? -p * pow_fast(rho[e], p - 1.0) * c : 0.0;
            if (d != d) d = 0.0;
            dc[e] = accumulate ? dc[e] + d : d;
        }
    }
    double v[1] = {en};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) partial[B.b] = v[0];
    if (!arrive_last_n(&S->cnt_misc, &last_flag, B.n)) return;
    double tot[1];
    reduce_partials<1>(partial, B.n, 1, tot, red);
    if (threadIdx.x == 0) {
        S->comp_energy = accumulate ? S->comp_energy + tot[0] : tot[0];
        S->cnt_misc = 0;
    }
}
__global__ void __launch_bounds__(256)
    sens_kernel(Layout L, const double *__restrict__ rho, const double *__restrict__ ce,
                const double *__restrict__ s, const uint8_t *__restrict__ design, int variant,
                double p, double *__restrict__ dc, int accumulate, double *partial, Scalars *S) {
    sens_body(L, rho, ce, s, design, variant, p, dc, accumulate, partial, S, grid_blk());
}
cudaError_t sensitivities(const Layout &L, const double *rho, const double *ce, const double *s,
                          const uint8_t *design, int variant, double p, double *dc, int accumulate,
                          double *partial, Scalars *S, cudaStream_t st) {
    const int nb = std::max(1, std::min(div_up(L.nel, 256), 152 * 8));
    sens_kernel<<<nb, 256, 0, st>>>(L, rho, ce, s, design, variant, p, dc, accumulate, partial, S);
    return counted(cudaGetLastError());
}

__device__ __forceinline__ void sparse_dot_body(const long long *idx, const double *val, int n, const double *u,
                                  double *out, const Blk B) {
    __shared__ double red[256 / 32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc = fma(val[i], u[idx[i]], acc);
    double v[1] = {acc};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) *out = v[0];
}
__global__ void sparse_dot_kernel(const long long *idx, const double *val, int n, const double *u,
                                  double *out) {
    sparse_dot_body(idx, val, n, u, out, grid_blk());
}
cudaError_t sparse_dot(const long long *idx, const double *val, int n, const double *u,
                       double *out, cudaStream_t st) {
    sparse_dot_kernel<<<1, 256, 0, st>>>(idx, val, n, u, out);
    return counted(cudaGetLastError());
}

__device__ __forceinline__ void masked_sqnorm_body(const long long *idx, const double *val, int n, long long cs,
                                     const uint8_t *mask, double *out, const Blk B) {
    __shared__ double red[256 / 32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const long long d = idx[i];
        const int comp = (int)(d / cs);
        const long long node = d - comp * cs;
        if (!((mask[node] >> comp) & 1u)) acc = fma(val[i], val[i], acc);
    }
    double v[1] = {acc};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) *out = v[0];
}
__global__ void masked_sqnorm_kernel(const long long *idx, const double *val, int n, long long cs,
                                     const uint8_t *mask, double *out) {
    masked_sqnorm_body(idx, val, n, cs, mask, out, grid_blk());
}
cudaError_t masked_sqnorm(const long long *idx, const double *val, int n, long long cs,
                          const uint8_t *mask, double *out, cudaStream_t st) {
    masked_sqnorm_kernel<<<1, 256, 0, st>>>(idx, val, n, cs, mask, out);
    return counted(cudaGetLastError());
}

// ============================================================================
// OC bisection (topology_optimizer.cpp:205-287 / topopt.py:200-264)
//
// Per element the update is max(rmin, max(rho - m, min(1, min(rho + m, rho Be))))
// with Be = sqrt(-dc / (lmid + eps)).  It is evaluated as a * t with
// a = rho sqrt(-dc) (once per update) and t = 1/sqrt(lmid + eps) (once per pass),
// and the bounds rho -/+ m are precomputed, so a pass reads 3 values per element
// and writes nothing; the density is written once with the last pass's t.
// FP64 mode does the pass in FP64.  Mixed mode does it in double-float
// arithmetic on the FP32 pipes (FP64 is ~1/64 of FP32 on GB300): an FP32 pass
// shifts the bisection volume enough to flip its branch decisions, a
// double-float pass keeps ~48 significant bits like the FP64 reference.
// ============================================================================
__device__ __forceinline__ float2 df_of(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = p + e;
    return make_float2(s, e - (s - p));
}
__device__ __forceinline__ bool df_lt(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
__device__ __forceinline__ bool df_nan(float2 a) { return a.x != a.x; }

struct OcPrepArgs {
    long long nel;
    const double *rho, *dc;
    double *a64, *lo64, *hi64;
    float2 *a32, *lo32, *hi32;
    double move;
    int fp64, variant;
    Scalars *S;
};

__device__ __forceinline__ void oc_prepare_body(OcPrepArgs A, const Blk B) {
    for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < A.nel;
         e += (long long)B.n * blockDim.x) {
        const double r = A.rho[e];
        const double a = r * sqrt(-A.dc[e]);
        const double lo = r - A.move, hi = r + A.move;
        if (A.fp64) {
            A.a64[e] = a;
            A.lo64[e] = lo;
            A.hi64[e] = hi;
        } else {
            A.a32[e] = df_of(a);
            A.lo32[e] = df_of(lo);
            A.hi32[e] = df_of(hi);
        }
    }
    if (B.b == 0 && threadIdx.x == 0) {
        Scalars *S = A.S;
        const double l1 = A.variant == 0 ? 1e-20 : 1e-9;
        const double l2 = A.variant == 0 ? 1e20 : 1e9;
        const double eps = A.variant == 0 ? 1e-20 : 1e-10;
        S->l1 = l1;
        S->l2 = l2;
        S->oc_t = 1.0 / sqrt(0.5 * (l1 + l2) + eps);
        S->oc_t_last = S->oc_t;
        S->oc_pass = 0;
        S->oc_done = 0;
        S->oc_variant = A.variant;
    }
}
__global__ void oc_prepare_kernel(OcPrepArgs A) {
    oc_prepare_body(A, grid_blk());
}
cudaError_t oc_prepare(const OcBuffers &B, const double *rho, const double *dc, double move, int fp64,
                       int variant, Scalars *S, cudaStream_t st) {
    OcPrepArgs a{B.nel, rho, dc, B.a64, B.lo64, B.hi64, B.a32, B.lo32, B.hi32, move, fp64, variant, S};
    oc_prepare_kernel<<<std::max(1, std::min(div_up(B.nel, 256), 152 * 16)), 256, 0, st>>>(a);
    return counted(cudaGetLastError());
}

template <typename T>
__device__ __forceinline__ T oc_clamp(T c, T lo, T hi, T rmin, int variant) {
    if (variant == 0) return cmax<T>(rmin, cmax<T>(lo, cmin<T>(T(1), cmin<T>(hi, c))));
    return npmax<T>(rmin, npmax<T>(lo, npmin<T>(T(1), npmin<T>(hi, c))));
}

// the same chain on double-float values
__device__ __forceinline__ float2 oc_clamp_df(float2 c, float2 lo, float2 hi, float2 rmin, int variant) {
    const float2 one = make_float2(1.f, 0.f);
    if (variant == 0) {
        float2 m = df_lt(c, hi) ? c : hi;       // std::min(hi, c)
        m = df_lt(m, one) ? m : one;             // std::min(1, m)
        m = df_lt(lo, m) ? m : lo;               // std::max(lo, m)
        return df_lt(rmin, m) ? m : rmin;        // std::max(rmin, m)
    }
    if (df_nan(c) || df_nan(lo) || df_nan(hi)) return make_float2(__int_as_float(0x7fc00000), 0.f);
    float2 m = df_lt(c, hi) ? c : hi;
    m = df_lt(m, one) ? m : one;
    m = df_lt(m, lo) ? lo : m;
    return df_lt(m, rmin) ? rmin : m;
}

__device__ __forceinline__ void oc_stop_check(Scalars *S, double cur, double vf, int variant) {
    const double lmid = 0.5 * (S->l1 + S->l2);
    S->oc_cur = cur;
    S->oc_t_last = S->oc_t;
    if (cur > vf) S->l1 = lmid;
    else S->l2 = lmid;
    S->oc_pass += 1;
    const double l1 = S->l1, l2 = S->l2;
    bool stop;
    if (variant == 0) {
        stop = (l2 - l1) / (l1 + l2) < 1e-4;
    } else {
        const double den = (l1 + l2) > 1e-10 ? (l1 + l2) : 1e-10;
        stop = (l1 + l2 < 1e-12) || ((l2 - l1) / den <= 1e-3);
    }
    if (stop || S->oc_pass >= 100) S->oc_done = 1;
    const double eps = variant == 0 ? 1e-20 : 1e-10;
    S->oc_t = 1.0 / sqrt(0.5 * (l1 + l2) + eps);
}

struct OcPassArgs {
    OcBuffers B;
    const uint8_t *design;
    int fp64, variant;
    double rho_min, vf, n_design;
    double *partial;
    Scalars *S;
};

// One bisection pass: volume of the design elements at the current t.
__device__ __forceinline__ void oc_pass_body(OcPassArgs A, const Blk B) {
    __shared__ double red[256 / 32];
    __shared__ int last_flag;
    Scalars *S = A.S;
    if (S->oc_done) return;
    const double t = S->oc_t;
    double vol64 = 0.0;
    DF vol{0.f, 0.f};
    if (A.fp64) {
        for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < A.B.nel;
             e += (long long)B.n * blockDim.x) {
            if (!A.design[e]) continue;
            vol64 += oc_clamp<double>(A.B.a64[e] * t, A.B.lo64[e], A.B.hi64[e], A.rho_min, A.variant);
        }
    } else {
        const float2 tdf = df_of(t), rmin = df_of(A.rho_min);
        for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < A.B.nel;
             e += (long long)B.n * blockDim.x) {
            if (!A.design[e]) continue;
            const float2 v = oc_clamp_df(df_mul(A.B.a32[e], tdf), A.B.lo32[e], A.B.hi32[e], rmin, A.variant);
            df_add(vol, v.x);
            vol.lo += v.y;
        }
        vol64 = df_value(vol);
    }
    double v[1] = {vol64};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) A.partial[B.b] = v[0];
    if (!arrive_last_n(&S->cnt_oc, &last_flag, B.n)) return;
    double tot[1];
    reduce_partials<1>(A.partial, B.n, 1, tot, red);
    if (threadIdx.x == 0) {
        oc_stop_check(S, tot[0] / A.n_design, A.vf, A.variant);
        S->cnt_oc = 0;
    }
}
__global__ void __launch_bounds__(256) oc_pass_kernel(OcPassArgs A) {
    oc_pass_body(A, grid_blk());
}
cudaError_t oc_pass(const OcBuffers &B, const uint8_t *design, int fp64, int variant, double rho_min, double vf,
                    double n_design, double *partial, Scalars *S, int nblocks, cudaStream_t st) {
    OcPassArgs a{B, design, fp64, variant, rho_min, vf, n_design, partial, S};
    oc_pass_kernel<<<nblocks, 256, 0, st>>>(a);
    return counted(cudaGetLastError());
}

// Density of the last executed pass, max |change| and the design-mask mean.
// The density is always formed in FP64 from rho and dc (the same a = rho sqrt(-dc)
// and bounds as oc_prepare's FP64 terms): the clamped values rho_min, rho -/+ move
// and 1 must come out exact, because the next stiffness skips elements with
// rho < rho_min -- a double-float rho_min (48 bits) lands one ulp below it.  Only
// the multiplier t comes from the (double-float or FP64) bisection passes.
__device__ __forceinline__ void oc_final_body(OcPassArgs A, const double *__restrict__ rho,
                                                       const double *__restrict__ dc, double move,
                                                       double *__restrict__ rho_new, const Blk B) {
    __shared__ double red[2 * (256 / 32)];
    __shared__ int last_flag;
    Scalars *S = A.S;
    const double t = S->oc_t_last;
    double mc = 0.0, vs = 0.0, cnt = 0.0;
    for (long long e = B.b * (long long)blockDim.x + threadIdx.x; e < A.B.nel;
         e += (long long)B.n * blockDim.x) {
        const double r0 = rho[e];
        double v = r0;
        if (A.design[e]) {
            if (S->oc_pass > 0) {  // no pass ran: unchanged (cannot happen with the reference bounds)
                const double a = r0 * sqrt(-dc[e]);
                v = oc_clamp<double>(a * t, r0 - move, r0 + move, A.rho_min, A.variant);
            }
            vs += v;
            cnt += 1.0;
        }
        rho_new[e] = v;
        mc = fmax(mc, fabs(v - r0));
    }
    const double m = block_max(mc, red);
    double s2[2] = {vs, cnt};
    block_sum<2>(s2, red);
    if (threadIdx.x == 0) {
        A.partial[3 * B.b] = m;
        A.partial[3 * B.b + 1] = s2[0];
        A.partial[3 * B.b + 2] = s2[1];
    }
    if (!arrive_last_n(&S->cnt_oc, &last_flag, B.n)) return;
    if (threadIdx.x == 0) {
        double mm = 0.0, ss = 0.0, cc = 0.0;
        for (unsigned b = 0; b < B.n; ++b) {
            mm = fmax(mm, __ldcg(A.partial + 3 * b));
            ss += __ldcg(A.partial + 3 * b + 1);
            cc += __ldcg(A.partial + 3 * b + 2);
        }
        S->oc_change = mm;
        S->oc_volume = cc > 0.0 ? ss / cc : ss / (double)A.B.nel;
        S->cnt_oc = 0;
    }
}
__global__ void __launch_bounds__(256) oc_final_kernel(OcPassArgs A, const double *__restrict__ rho,
                                                       const double *__restrict__ dc, double move,
                                                       double *__restrict__ rho_new) {
    oc_final_body(A, rho, dc, move, rho_new, grid_blk());
}
cudaError_t oc_final(const OcBuffers &B, const uint8_t *design, int fp64, int variant, double rho_min,
                     const double *rho, const double *dc, double move, double *rho_new, double *partial, Scalars *S,
                     int nblocks, cudaStream_t st) {
    OcPassArgs a{B, design, fp64, variant, rho_min, 0.0, 1.0, partial, S};
    oc_final_kernel<<<nblocks, 256, 0, st>>>(a, rho, dc, move, rho_new);
    return counted(cudaGetLastError());
}


// ============================================================================
// Batched persistent kernels (batch.cuh).  Each CTA loops over the work items of
// its family; an item runs the single-problem body with the item's block index
// and its problem's block count.  Frozen problems are skipped by every family,
// problems whose PCG is done by the PCG bodies themselves.
// ============================================================================
#define AMK_BATCH_LOOP(WL)                                  \
    for (int _w = blockIdx.x; _w < (WL).n; _w += gridDim.x) \
        if (const int2 _k = (WL).w[_w]; true)

__global__ void __launch_bounds__(256) b_scales_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        scales_body(it.L, it.rho, nullptr, 0, it.penalty, it.emin, it.rho_min, 1.0, it.s64, it.s32, 0,
                    Blk{_k.y, it.n_elem});
    }
}
__global__ void __launch_bounds__(256) b_diag_kernel(const BatchItem *items, WorkList W, double d0) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        diag_mask_body(it.L, it.s64, d0, it.fixed_bits, it.dinv64, it.dinv32, it.mask, Blk{_k.y, it.n_vec});
    }
}
cudaError_t batch_operator(const BatchItem *it, WorkList elem, WorkList vec, const BatchConst &C, int grid,
                           cudaStream_t st) {
    b_scales_kernel<<<std::max(1, std::min(grid, elem.n)), 256, 0, st>>>(it, elem);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_diag_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(it, vec, C.d0);
    return counted(cudaGetLastError());
}

__global__ void __launch_bounds__(256) b_zero_masked_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        zero_masked_body(it.L, it.mask, it.x64, Blk{_k.y, it.n_vec});
    }
}
__global__ void __launch_bounds__(256) b_sqnorm_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        masked_sqnorm_body(it.f_idx, it.f_val, it.f_nnz, it.L.cs, it.mask, &it.S->b2, Blk{0, 1});
        __syncthreads();
    }
}
cudaError_t batch_prepare_solve(const BatchItem *it, WorkList vec, WorkList prob, int grid, cudaStream_t st) {
    b_zero_masked_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(it, vec);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_sqnorm_kernel<<<std::max(1, std::min(grid, prob.n)), 256, 0, st>>>(it, prob);
    return counted(cudaGetLastError());
}

__global__ void __launch_bounds__(KuShape<32, 4>::NT) b_resid_kernel(const BatchItem *items, WorkList W,
                                                                     Modal<dflt> Mdf, int energy) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        KuArgs<double> a{};
        a.L = it.L;
        a.s = it.s64;
        a.u = it.x64;
        a.f = it.F;
        a.dinv = it.dinv64;
        a.mask = it.mask;
        a.y = it.r64;
        a.ce = energy ? it.ce : nullptr;
        a.energy = energy;
        a.partial = it.partial;
        a.S = it.S;
        a.tiles_x = it.k64_tiles_x;
        a.tiles_y = it.k64_tiles_y;
        a.tiles_z = it.k64_tiles_z;
        a.tz = it.k64_tz;
        ku_df_body<32, 4, KU_RESID>(a, Mdf, Blk{_k.y, it.n_k64});
        __syncthreads();
    }
}
// the batch's residuals (FP64 defect correction) in double-float, as the
// single-problem mixed solver's (kudf.cuh)
cudaError_t batch_resid(const BatchItem *it, WorkList k64, const BatchConst &C, int energy, int grid,
                        cudaStream_t st) {
    using Sh = KuShape<32, 4>;
    const size_t smem = Sh::template smem_bytes<double>();
    b_resid_kernel<<<std::max(1, std::min(grid, k64.n)), Sh::NT, smem, st>>>(it, k64, modal_dflt(C.M64), energy);
    return counted(cudaGetLastError());
}

__global__ void __launch_bounds__(256) b_inner_init_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        // the FP32 sequence continues the FP64 iterate x64 (no zeroing), held as the
        // double-float pair (xh, xl) while it runs
        dc_inner_init_body(it.L, it.r64, it.r32, nullptr, it.S, Blk{_k.y, it.n_vec});
        const long long n = 3 * it.L.cs;
        for (long long i = _k.y * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)it.n_vec * blockDim.x) {
            const double x = it.x64[i];
            const float h = (float)x;
            it.xh[i] = h;
            it.xl[i] = (float)(x - (double)h);
        }
    }
}
// FP32 PCG on K x32 = r32 to |r| <= tol/2 |F| (but at most 1e-6 below its start);
// a problem whose FP64 residual already meets tol starts done.
__global__ void __launch_bounds__(256) b_inner_start_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        const double b2 = it.S->b2, rr = it.S->res_rr;
        const double tol2 = it.tol * it.tol;
        const double thr = (rr <= tol2 * b2) ? 1e300 : fmax(0.25 * tol2 * b2, 1e-12 * rr);
        pcg_start_body<float>(it.L, it.r32, it.dinv32, thr, 0.0, it.maxit, 0, it.partial, it.S,
                              Blk{_k.y, it.n_vec});
        __syncthreads();
    }
}
cudaError_t batch_inner_start(const BatchItem *it, WorkList vec, int grid, cudaStream_t st) {
    b_inner_init_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(it, vec);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_inner_start_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(it, vec);
    return counted(cudaGetLastError());
}

template <int W_, int MODE>
__global__ void __launch_bounds__(32 * W_, 2) b_ku2_kernel(const BatchItem *items, WorkList W, Modal<float> M) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        Ku2Args a{};
        a.L = it.L;
        a.M = M;
        a.s = it.s32;
        a.u = it.pa;
        a.pa = it.pa;
        a.pb = it.pb;
        a.r = it.r32;
        a.dinv = it.dinv32;
        a.mask = it.mask;
        a.y = it.q32;
        a.partial = it.partial;
        a.S = it.S;
        a.tiles_x = it.k2_tiles_x;
        a.tiles_y = it.k2_tiles_y;
        a.tiles_z = it.k2_tiles_z;
        a.tz = it.k2_tz;
        ku2_body<W_, MODE>(a, Blk{_k.y, it.n_k2});
        __syncthreads();
    }
}
// The batched form of pcg_update_df_kernel: work items are (problem, chunk of
// UPD_K DOFs), listed problem by problem.  Each CTA takes a contiguous range of
// items and runs a two-stage bulk-copy pipeline over it; the r.r / r.z partials
// of a run of consecutive items of one problem are reduced once and published in
// the run's first slot (zeros in the others), and the CTA arrives for the whole
// run, so a CTA synchronises once per problem it touches rather than per chunk.
// Items of frozen or converged problems are skipped without a copy (their state
// cannot change during the launch: only a problem's own last run ends it).
constexpr int UPD_ST = 2;  // batched update: stages of 7 chunk planes (xh, xl, r, p_prev, p, q, D^-1)
__global__ void __launch_bounds__(256) b_update_df_kernel(const BatchItem *items, WorkList W) {
    extern __shared__ __align__(128) unsigned char upd_smem[];
    __shared__ uint64_t bar[UPD_ST];
    __shared__ double red[2 * (VEC_THREADS / 32)];
    __shared__ int last_flag, fail;
    auto plane = [&](int s, int a) {
        return reinterpret_cast<float *>(upd_smem + (size_t)s * 28 * UPD_K + (size_t)4 * UPD_K * a);
    };
    struct Chunk {
        long long o, j0;
        int len, nck;
    };
    auto chunk = [&](const BatchItem &it, int g) {
        Chunk c;
        c.nck = (int)((it.L.cs + UPD_K - 1) / UPD_K);
        const int comp = g / c.nck;
        c.j0 = (long long)(g - comp * c.nck) * UPD_K;
        c.len = (int)min((long long)UPD_K, it.L.cs - c.j0);
        c.o = comp * it.L.cs + c.j0;
        return c;
    };
    const int lo = (int)((long long)W.n * blockIdx.x / gridDim.x);
    const int hi = (int)((long long)W.n * (blockIdx.x + 1) / gridDim.x);
    auto active = [&](int i) {
        const Scalars *S = items[W.w[i].x].S;
        return !S->frozen && !S->done;
    };
    // an odd iteration of a problem folds its iterate (x += alpha_prev p_prev +
    // alpha p, as the single-problem update): 7 streams; an even one 3 (r, q, D^-1)
    auto issue = [&](int i, int s) {
        const int2 k = W.w[i];
        const BatchItem &it = items[k.x];
        const Chunk c = chunk(it, k.y);
        const bool fold = (it.S->it & 1) != 0;
        const unsigned b = 4u * (unsigned)c.len;
        bulk::bar_expect(&bar[s], (fold ? 7u : 3u) * b);
        if (fold) {
            const float *p = it.pa, *pp = it.pb;  // it odd: this iteration's K*u wrote pa
            bulk::copy_g2s(plane(s, 0), it.xh + c.o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 1), it.xl + c.o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 3), pp + c.o, b, &bar[s]);
            bulk::copy_g2s(plane(s, 4), p + c.o, b, &bar[s]);
        }
        bulk::copy_g2s(plane(s, 2), it.r32 + c.o, b, &bar[s]);
        bulk::copy_g2s(plane(s, 5), it.q32 + c.o, b, &bar[s]);
        bulk::copy_g2s(plane(s, 6), it.dinv32 + c.j0, b, &bar[s]);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < UPD_ST; ++s) bulk::bar_init(&bar[s], 1);
        bulk::bar_init_fence();
        fail = 0;
    }
    __syncthreads();
    // bit s: stage s holds issued copies / the parity stage s waits for next
    unsigned issued = 0u, phase = 0u;
#pragma unroll
    for (int j = 0; j < UPD_ST; ++j) {
        if (lo + j < hi && active(lo + j)) {
            issued |= 1u << j;
            if (threadIdx.x == 0) issue(lo + j, j);
        }
    }
    // the current run: problem, first and last chunk index, and its partial sums
    int run_p = -1, run_first = 0, run_last = 0;
    Acc<float> a0, a1;
    auto flush_run = [&]() {
        const BatchItem &it = items[run_p];
        double v[2] = {a0.value(), a1.value()};
        block_sum<2>(v, red);
        if (threadIdx.x == 0) {
            it.partial[2 * run_first] = v[0];
            it.partial[2 * run_first + 1] = v[1];
        }
        for (int g = run_first + 1 + (int)threadIdx.x; g <= run_last; g += blockDim.x) {
            it.partial[2 * g] = 0.0;
            it.partial[2 * g + 1] = 0.0;
        }
        const int nb = 3 * chunk(it, 0).nck;
        if (arrive_last_weighted(&it.S->cnt_upd, &last_flag, run_last - run_first + 1, nb)) {
            double tot[2];
            reduce_partials<2>(it.partial, nb, 2, tot, red);
            if (threadIdx.x == 0) {
                // an even iteration leaves alpha_k p_k owed to the iterate; an odd one paid it
                it.S->alpha_prev = (it.S->it & 1) ? 0.0 : it.S->alpha;
                pcg_update_finish(it.S, tot[0], tot[1]);
            }
        }
        a0 = Acc<float>();
        a1 = Acc<float>();
        run_p = -1;
    };
    for (int i = lo; i < hi; ++i) {
        const int s = (i - lo) % UPD_ST;
        if (issued & (1u << s)) {
            if (!fail) {
                if (!bulk::bar_wait(&bar[s], (phase >> s) & 1u)) fail = 1;
            }
            phase ^= 1u << s;
            __syncthreads();
            const int2 k = W.w[i];
            // a new problem (or a gap in this one's chunks) closes the current run
            if (run_p >= 0 && (run_p != k.x || k.y != run_last + 1)) flush_run();
            if (run_p < 0) {
                run_p = k.x;
                run_first = k.y;
            }
            run_last = k.y;
            const BatchItem &it = items[k.x];
            const Chunk c = chunk(it, k.y);
            const float alpha = (float)it.S->alpha;
            const bool fold = (it.S->it & 1) != 0;
            const float alpha_prev = (float)it.S->alpha_prev;
            if (!fail) {
                const float4 *hs = reinterpret_cast<const float4 *>(plane(s, 0));
                const float4 *ls = reinterpret_cast<const float4 *>(plane(s, 1));
                const float4 *rs = reinterpret_cast<const float4 *>(plane(s, 2));
                const float4 *pps = reinterpret_cast<const float4 *>(plane(s, 3));
                const float4 *ps = reinterpret_cast<const float4 *>(plane(s, 4));
                const float4 *qs = reinterpret_cast<const float4 *>(plane(s, 5));
                const float4 *ds = reinterpret_cast<const float4 *>(plane(s, 6));
                for (int t = threadIdx.x; t < c.len / 4; t += VEC_THREADS) {
                    float4 rv = rs[t];
                    const float4 qv = qs[t], d = ds[t];
                    if (fold) {
                        float4 h = hs[t], l = ls[t];
                        const float4 pp = pps[t], pv = ps[t];
                        two_sum_acc(h.x, l.x, alpha_prev, pp.x);
                        two_sum_acc(h.y, l.y, alpha_prev, pp.y);
                        two_sum_acc(h.z, l.z, alpha_prev, pp.z);
                        two_sum_acc(h.w, l.w, alpha_prev, pp.w);
                        two_sum_acc(h.x, l.x, alpha, pv.x);
                        two_sum_acc(h.y, l.y, alpha, pv.y);
                        two_sum_acc(h.z, l.z, alpha, pv.z);
                        two_sum_acc(h.w, l.w, alpha, pv.w);
                        reinterpret_cast<float4 *>(it.xh + c.o)[t] = h;
                        reinterpret_cast<float4 *>(it.xl + c.o)[t] = l;
                    }
                    rv.x = fmaf(-alpha, qv.x, rv.x);
                    rv.y = fmaf(-alpha, qv.y, rv.y);
                    rv.z = fmaf(-alpha, qv.z, rv.z);
                    rv.w = fmaf(-alpha, qv.w, rv.w);
                    reinterpret_cast<float4 *>(it.r32 + c.o)[t] = rv;
                    a0.add(fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, rv.w * rv.w))));
                    a1.add(fmaf(rv.x, d.x * rv.x,
                                fmaf(rv.y, d.y * rv.y, fmaf(rv.z, d.z * rv.z, rv.w * (d.w * rv.w)))));
                }
            } else if (threadIdx.x == 0) {
                atomicExch(&it.S->kerr, 1);
            }
            __syncthreads();  // stage s read by every thread
            issued &= ~(1u << s);
        }
        // refill stage s with item i + UPD_ST (fail is uniform here: read after a barrier)
        if (i + UPD_ST < hi && !fail && active(i + UPD_ST)) {
            issued |= 1u << s;
            if (threadIdx.x == 0) {
                bulk::proxy_fence();
                issue(i + UPD_ST, s);
            }
        }
    }
    if (run_p >= 0) flush_run();
    if (fail && threadIdx.x == 0) {
        // drain what this CTA issued and did not consume (bounded waits)
        for (int s = 0; s < UPD_ST; ++s)
            if (issued & (1u << s)) bulk::bar_wait(&bar[s], (phase >> s) & 1u);
    }
}
// x64 = xh + xl for every active problem (end of an FP32 PCG round), after the
// term alpha_prev p an even last iteration left owed (the next round's start
// clears alpha_prev)
__global__ void __launch_bounds__(256) b_compose_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        const long long n = 3 * it.L.cs;
        const bool owed = (it.S->it & 1) != 0;
        const float a = (float)it.S->alpha_prev;
        const float *p = it.pb;  // it odd: the last K*u wrote pb
        for (long long i = _k.y * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)it.n_vec * blockDim.x) {
            float h = it.xh[i], l = it.xl[i];
            if (owed) two_sum_acc(h, l, a, p[i]);
            it.x64[i] = (double)h + (double)l;
        }
    }
}
cudaError_t batch_inner_end(const BatchItem *it, WorkList vec, int grid, cudaStream_t st) {
    b_compose_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(it, vec);
    return counted(cudaGetLastError());
}
static_assert(BATCH_UPD_CHUNK == UPD_K, "batched update chunk");
// The batched FP32 K*u of one plan: warps 8 or 4 for every problem (list k2), or
// 0 -- each problem's own tile height, list k2 holding the 8-warp problems' tiles
// and k2b the 4-warp ones (two launches).
template <int MODE>
static cudaError_t batch_ku_launch(const BatchItem *it, WorkList k2, WorkList k2b, const BatchConst &C, int warps,
                                   int grid, cudaStream_t st) {
    if (warps == 8 || (warps == 0 && k2.n > 0))
        b_ku2_kernel<8, MODE><<<std::max(1, std::min(grid, k2.n)), 256, 0, st>>>(it, k2, C.M32);
    else if (warps == 4)
        b_ku2_kernel<4, MODE><<<std::max(1, std::min(grid, k2.n)), 128, 0, st>>>(it, k2, C.M32);
    else if (warps != 0)
        return cudaErrorInvalidValue;
    if (warps != 0 || k2.n > 0)
        if (cudaError_t e = counted(cudaGetLastError())) return e;
    if (warps == 0 && k2b.n > 0) {
        // a 4-warp CTA holds half the threads: twice the CTAs in the persistent grid
        b_ku2_kernel<4, MODE><<<std::max(1, std::min(2 * grid, k2b.n)), 128, 0, st>>>(it, k2b, C.M32);
        if (cudaError_t e = counted(cudaGetLastError())) return e;
    }
    return cudaSuccess;
}
cudaError_t batch_pcg_iteration(const BatchItem *it, WorkList k2, WorkList k2b, WorkList vec, const BatchConst &C,
                                int warps, int grid_k2, int grid_vec, cudaStream_t st) {
    if (cudaError_t e = batch_ku_launch<KU_PCG>(it, k2, k2b, C, warps, grid_k2, st)) return e;
    b_update_df_kernel<<<std::max(1, std::min(grid_vec, vec.n)), 256, UPD_SMEM, st>>>(it, vec);
    return counted(cudaGetLastError());
}
cudaError_t batch_pcg_ku(const BatchItem *it, WorkList k2, WorkList k2b, const BatchConst &C, int warps, int grid,
                         cudaStream_t st) {
    return batch_ku_launch<KU_PCG>(it, k2, k2b, C, warps, grid, st);
}
cudaError_t batch_pcg_update(const BatchItem *it, WorkList chunks, int grid_vec, cudaStream_t st) {
    b_update_df_kernel<<<std::max(1, std::min(grid_vec, chunks.n)), 256, UPD_SMEM, st>>>(it, chunks);
    return counted(cudaGetLastError());
}
cudaError_t batch_ku_plain(const BatchItem *it, WorkList k2, WorkList k2b, const BatchConst &C, int warps, int grid,
                           cudaStream_t st) {
    return batch_ku_launch<KU_PLAIN>(it, k2, k2b, C, warps, grid, st);
}

__global__ void __launch_bounds__(256) b_sens_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        sens_body(it.L, it.rho, it.ce, it.s64, it.design, 0, it.penalty, it.dc, 0, it.partial, it.S,
                  Blk{_k.y, it.n_elem});
        __syncthreads();
    }
}
__global__ void __launch_bounds__(256) b_fu_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        sparse_dot_body(it.f_idx, it.f_val, it.f_nnz, it.x64, &it.S->comp_fu, Blk{0, 1});
        __syncthreads();
    }
}
__global__ void __launch_bounds__(256) b_filter_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        filter_cpp_body<double>(it.L, it.tap_d, it.tap_w, it.ntaps, it.dc, it.rho, it.dcf, Blk{_k.y, it.n_elem});
    }
}
__device__ __forceinline__ OcPassArgs batch_oc_args(const BatchItem &it) {
    OcPassArgs a{};
    a.B.nel = it.L.nel;
    a.B.a64 = it.oc_a;
    a.B.lo64 = it.oc_lo;
    a.B.hi64 = it.oc_hi;
    a.design = it.design;
    a.fp64 = 1;
    a.variant = 0;
    a.rho_min = it.rho_min;
    a.vf = it.vf;
    a.n_design = it.n_design;
    a.partial = it.partial;
    a.S = it.S;
    return a;
}
__global__ void __launch_bounds__(256) b_oc_prepare_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        OcPrepArgs a{it.L.nel, it.rho, it.dcf, it.oc_a, it.oc_lo, it.oc_hi, nullptr, nullptr, nullptr,
                     it.move, 1, 0, it.S};
        oc_prepare_body(a, Blk{_k.y, it.n_elem});
    }
}
__global__ void __launch_bounds__(256) b_oc_pass_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        oc_pass_body(batch_oc_args(it), Blk{_k.y, it.n_elem});
        __syncthreads();
    }
}
__global__ void __launch_bounds__(256) b_oc_final_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        oc_final_body(batch_oc_args(it), it.rho, it.dcf, it.move, it.rho_new, Blk{_k.y, it.n_elem});
        __syncthreads();
    }
}
__global__ void __launch_bounds__(256) b_copy_density_kernel(const BatchItem *items, WorkList W) {
    AMK_BATCH_LOOP(W) {
        const BatchItem &it = items[_k.x];
        if (it.S->frozen) continue;
        for (long long e = (long long)_k.y * blockDim.x + threadIdx.x; e < it.L.nel;
             e += (long long)it.n_elem * blockDim.x)
            it.rho[e] = it.rho_new[e];
    }
}
cudaError_t batch_update(const BatchItem *it, WorkList elem, WorkList prob, int grid, cudaStream_t st) {
    const int ge = std::max(1, std::min(grid, elem.n)), gp = std::max(1, std::min(grid, prob.n));
    b_sens_kernel<<<ge, 256, 0, st>>>(it, elem);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_fu_kernel<<<gp, 256, 0, st>>>(it, prob);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_filter_kernel<<<ge, 256, 0, st>>>(it, elem);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_oc_prepare_kernel<<<ge, 256, 0, st>>>(it, elem);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    for (int k = 0; k < 100; ++k) {
        b_oc_pass_kernel<<<ge, 256, 0, st>>>(it, elem);
        if (cudaError_t e = counted(cudaGetLastError())) return e;
    }
    b_oc_final_kernel<<<ge, 256, 0, st>>>(it, elem);
    if (cudaError_t e = counted(cudaGetLastError())) return e;
    b_copy_density_kernel<<<ge, 256, 0, st>>>(it, elem);
    return counted(cudaGetLastError());
}
#undef AMK_BATCH_LOOP

}  // namespace amk
