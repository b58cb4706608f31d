// ku3.cu -- host side of the TMA-staged FP32 PCG K*u (ku3.cuh): tensor maps,
// the padded copies they read, the launch plan and the launchers; and the same
// kernel over a batch of problems (one CTA per tile of one problem).
#include <cudaTypedefs.h>

#include <algorithm>
#include <new>

#include "batch.cuh"
#include "kernels.cuh"
#include "ku3.cuh"

namespace amk {

__host__ __device__ inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

void ku3_padded_sizes(const Layout &L, long long *scale_entries, long long *mask_bytes) {
    if (scale_entries) *scale_entries = round_up(L.nx, 4) * L.ny * L.nz;
    if (mask_bytes) *mask_bytes = round_up(L.nx + 1, 16) * (L.ny + 1) * (L.nz + 1);
}

// scale_pad[(ez ny + ey) sxe + ex] = s32[(ez ny + ey) nx + ex];
// mask_pad[(iz (ny+1) + iy) sxm + ix] = mask[iz sxy + iy sx + ix]
// (entries i0, i0 + stride, ... of both)
__device__ __forceinline__ void ku3_pad_body(const Layout &L, const float *__restrict__ s32,
                                             const uint8_t *__restrict__ mask, float *__restrict__ scale_pad,
                                             uint8_t *__restrict__ mask_pad, int sxe, int sxm, long long i0,
                                             long long stride) {
    for (long long e = i0; e < L.nel; e += stride) {
        const long long row = e / L.nx;
        const int ex = (int)(e - row * L.nx);
        scale_pad[row * sxe + ex] = s32[e];
    }
    const long long nrow = (long long)(L.ny + 1) * (L.nz + 1);
    const long long nn = nrow * (L.nx + 1);
    for (long long n = i0; n < nn; n += stride) {
        const long long row = n / (L.nx + 1);  // iz (ny+1) + iy
        const int ix = (int)(n - row * (L.nx + 1));
        const long long iz = row / (L.ny + 1), iy = row - iz * (L.ny + 1);
        mask_pad[row * sxm + ix] = mask[iz * L.sxy + iy * L.sx + ix];
    }
}
__global__ void ku3_pad_kernel(Layout L, const float *__restrict__ s32, const uint8_t *__restrict__ mask,
                               float *__restrict__ scale_pad, uint8_t *__restrict__ mask_pad, int sxe, int sxm) {
    ku3_pad_body(L, s32, mask, scale_pad, mask_pad, sxe, sxm, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}
// the same for every problem of a batch: block b of a problem's n handles
// entries b * 256 + t, stride n * 256
__global__ void __launch_bounds__(256) b_ku3_pad_kernel(const BatchItem *items, WorkList W) {
    for (int w = blockIdx.x; w < W.n; w += gridDim.x) {
        const int2 k = W.w[w];
        const BatchItem &it = items[k.x];
        if (it.S->frozen) continue;
        ku3_pad_body(it.L, it.s32, it.mask, it.s32pad, it.maskpad, (int)round_up(it.L.nx, 4),
                     (int)round_up(it.L.nx + 1, 16), (long long)k.y * blockDim.x + threadIdx.x,
                     (long long)it.n_vec * blockDim.x);
    }
}

cudaError_t ku3_pad(const Layout &L, const float *s32, const uint8_t *mask, float *scale_pad, uint8_t *mask_pad,
                    cudaStream_t st) {
    const long long n = std::max<long long>(L.nel, (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1));
    const int nb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8));
    ku3_pad_kernel<<<nb, 256, 0, st>>>(L, s32, mask, scale_pad, mask_pad, (int)round_up(L.nx, 4),
                                       (int)round_up(L.nx + 1, 16));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn(cudaError_t *err) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            *err = e != cudaSuccess ? e : cudaErrorSymbolNotFound;
            return nullptr;
        }
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// rank-3 (x, y, z) or rank-4 (x, y, z, component) tiled map without swizzle;
// strides in bytes of dims 1..rank-1; out-of-bound elements read as zero
bool encode(PFN_cuTensorMapEncodeTiled_v12000 fn, CUtensorMap *m, CUtensorMapDataType dt, int rank, const void *base,
            const cuuint64_t *dims, const cuuint64_t *strides, const cuuint32_t *box) {
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(m, dt, (cuuint32_t)rank, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

Ku3Maps *ku3_make_maps(const Layout &L, const float *r, const float *pa, const float *pb, const float *dinv,
                       const uint8_t *mask_pad, const float *scale_pad, float *q, int warps, cudaError_t *err) {
    *err = cudaSuccess;
    if (warps != 7 && warps != 8) {
        *err = cudaErrorInvalidValue;
        return nullptr;
    }
    // boxes of the tile shape (the node columns and the staged widths do not depend on warps)
    using Sh = Ku3Shape<8, 4>;
    const cuuint32_t BY = 2 * warps + 1, BYE = 2 * warps, TY = 2 * warps - 1;
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn(err);
    if (!fn) return nullptr;
    Ku3Maps *T = new (std::nothrow) Ku3Maps;
    if (!T) {
        *err = cudaErrorMemoryAllocation;
        return nullptr;
    }
    const cuuint64_t nx1 = L.nx + 1, ny1 = L.ny + 1, nz1 = L.nz + 1;
    const cuuint64_t vdims[4] = {nx1, ny1, nz1, 3};
    const cuuint64_t vstr[3] = {(cuuint64_t)L.sx * 4, (cuuint64_t)L.sxy * 4, (cuuint64_t)L.cs * 4};
    const cuuint32_t vload[4] = {Sh::BX, BY, 1, 3};
    const cuuint32_t vstore[4] = {Sh::TX, TY, 1, 1};
    const cuuint64_t ndims[3] = {nx1, ny1, nz1};
    const cuuint32_t dbox[3] = {Sh::BX, BY, 1};
    const long long sxm = round_up(L.nx + 1, 16), sxe = round_up(L.nx, 4);
    const cuuint64_t mstr[2] = {(cuuint64_t)sxm, (cuuint64_t)(sxm * (L.ny + 1))};
    const cuuint32_t mbox[3] = {Sh::BXM, BY, 1};
    const cuuint64_t edims[3] = {(cuuint64_t)L.nx, (cuuint64_t)L.ny, (cuuint64_t)L.nz};
    const cuuint64_t estr[2] = {(cuuint64_t)sxe * 4, (cuuint64_t)(sxe * L.ny * 4)};
    const cuuint32_t ebox[3] = {Sh::BX, BYE, 1};
    const CUtensorMapDataType F = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const bool ok = encode(fn, &T->r, F, 4, r, vdims, vstr, vload) && encode(fn, &T->pa, F, 4, pa, vdims, vstr, vload) &&
                    encode(fn, &T->pb, F, 4, pb, vdims, vstr, vload) &&
                    encode(fn, &T->d, F, 3, dinv, ndims, vstr, dbox) &&
                    encode(fn, &T->m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, mask_pad, ndims, mstr, mbox) &&
                    encode(fn, &T->s, F, 3, scale_pad, edims, estr, ebox) &&
                    encode(fn, &T->qst, F, 4, q, vdims, vstr, vstore) &&
                    encode(fn, &T->past, F, 4, pa, vdims, vstr, vstore) &&
                    encode(fn, &T->pbst, F, 4, pb, vdims, vstr, vstore);
    if (!ok) {
        delete T;
        *err = cudaErrorInvalidValue;
        return nullptr;
    }
    return T;
}

void ku3_free_maps(Ku3Maps *m) { delete m; }

// The launch plan for tiles of `warps` warps (2 warps - 1 node rows): one wave of
// tiles (every tile resident at once, the z chunks as long as that allows)
// whenever it keeps at least 3/4 of the CTA slots busy, else the plan that
// minimises waves x chunk height.  Measured on GB300 (8-warp tiles): on the
// 256x128x128 grid 3 chunks of 43 planes (270 tiles, one wave) take 68.8 us
// against 71.9 us for 10 chunks of 13 (900 tiles, three waves) -- each tile's
// pipeline fill and p.q hand-off cost more than the idle slots -- and on 192x96x96
// the one-wave plan is the minimiser's choice already (6 chunks of 17 planes,
// 35.5 us; 9 or 13 planes 40.7 / 41.6 us).
static KuLaunch ku3_plan_w(const Layout &L, int warps, int sms, long long *one_wave_tiles) {
    const int tx = Ku3Shape<8, 4>::TX, ty = 2 * warps - 1;
    const long long cols = (long long)((L.nx + tx) / tx) * ((L.ny + ty) / ty);
    const long long slots = 2LL * sms;
    const int planes = L.nz + 1;
    int tz = 0;
    *one_wave_tiles = 0;
    if (cols <= slots) {
        const int chunks = (int)std::min<long long>(slots / cols, std::max(1, planes / 4));
        const int t = (planes + chunks - 1) / chunks;
        const long long tiles = cols * ((planes + t - 1) / t);
        if (4 * tiles >= 3 * slots) {
            tz = t;
            *one_wave_tiles = tiles;
        }
    }
    return ku_plan_shape(L, tx, ty, warps, 2, tz, sms);
}
// warps 0: 7-warp tiles (13 node rows) when their one-wave plan keeps more CTA
// slots busy than the 8-warp tiles' (15 rows) does, else 8-warp tiles.  On
// 256x128x128 the 7-warp plan is 300 tiles against 270: 63.5 against 69.5 us; on
// 192x96x96 it is 280 against 294: 36.7 against 35.6 us (GB300, 30 launches each).
KuLaunch ku3_plan(const Layout &L, int warps, int sms) {
    long long t8 = 0, t7 = 0;
    const KuLaunch k8 = ku3_plan_w(L, 8, sms, &t8);
    if (warps == 8) return k8;
    const KuLaunch k7 = ku3_plan_w(L, 7, sms, &t7);
    if (warps == 7) return k7;
    return t7 > t8 ? k7 : k8;
}

cudaError_t ku3_init_attributes() {
    cudaError_t e = cudaFuncSetAttribute(ku3_kernel<8, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Ku3Shape<8, 3>::SMEM_ALLOC);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ku3_kernel<8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ku3Shape<8, 4>::SMEM_ALLOC);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ku3_kernel<7, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ku3Shape<7, 4>::SMEM_ALLOC);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ku3b_kernel<8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ku3bShape<8, 4>::SMEM_ALLOC);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ku3b_kernel<8, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ku3bShape<8, 5>::SMEM_ALLOC);
    return e;
}

cudaError_t ku3_pcg(const Ku3Maps *T, const KuLaunch &K, const Layout &L, const Modal<float> &M, double *partial,
                    Scalars *S, int stages, cudaStream_t st) {
    if (!T || (K.warps != 8 && K.warps != 7) || K.tx != Ku3Shape<8, 4>::TX || K.ty != 2 * K.warps - 1)
        return cudaErrorInvalidValue;
    Ku3Args a{};
    a.M = M;
    a.partial = partial;
    a.S = S;
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tz = K.tz;
    a.nz = L.nz;
    if (K.warps == 7 && stages == 4)
        ku3_kernel<7, 4><<<K.ntiles(), 224, Ku3Shape<7, 4>::SMEM_ALLOC, st>>>(*T, a);
    else if (K.warps == 8 && stages == 4)
        ku3_kernel<8, 4><<<K.ntiles(), 256, Ku3Shape<8, 4>::SMEM_ALLOC, st>>>(*T, a);
    else if (K.warps == 8 && stages == 3)
        ku3_kernel<8, 3><<<K.ntiles(), 256, Ku3Shape<8, 3>::SMEM_ALLOC, st>>>(*T, a);
    else
        return cudaErrorInvalidValue;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

cudaError_t ku3b_pcg(const Ku3Maps *T, const KuLaunch &K, const Layout &L, const Modal<float> &M, float *q, float *pa,
                     float *pb, double *partial, Scalars *S, int stages, cudaStream_t st) {
    if (!T || K.warps != 8 || K.tx != Ku3Shape<8, 4>::TX || K.ty != Ku3Shape<8, 4>::TY) return cudaErrorInvalidValue;
    // the kernel forms node offsets in 32-bit arithmetic
    if (3 * L.cs >= (1LL << 31) || L.sxy >= (1LL << 31)) return cudaErrorInvalidValue;
    Ku3bArgs a{};
    a.M = M;
    a.partial = partial;
    a.S = S;
    a.q = q;
    a.pa = pa;
    a.pb = pb;
    a.tiles_x = K.tiles_x;
    a.tiles_y = K.tiles_y;
    a.tz = K.tz;
    a.nx = L.nx;
    a.ny = L.ny;
    a.nz = L.nz;
    a.sx = L.sx;
    a.sxy = (int)L.sxy;
    a.cs = (int)L.cs;
    if (stages == 5)
        ku3b_kernel<8, 5><<<K.ntiles(), 256, Ku3bShape<8, 5>::SMEM_ALLOC, st>>>(*T, a);
    else if (stages == 4)
        ku3b_kernel<8, 4><<<K.ntiles(), 256, Ku3bShape<8, 4>::SMEM_ALLOC, st>>>(*T, a);
    else
        return cudaErrorInvalidValue;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

// ---- batches ----------------------------------------------------------------------

// One tile of one problem per CTA (work items (problem, tile), the longest tiles
// first); problems that are frozen or whose PCG is done leave at once.
// The element constants come from the launch's parameters (one material per
// batch), so the arithmetic can read them there as the single-problem kernel does.
__global__ void __launch_bounds__(256, 2) b_ku3_kernel(const Ku3BatchItem *items, WorkList W, const Modal<float> M) {
    const int2 k = W.w[blockIdx.x];
    const Ku3BatchItem &it = items[k.x];
    Ku3Args A = it.A;
    A.M = M;
    if (A.S->frozen || A.S->done) return;
    if (threadIdx.x == 0) {
        for (const CUtensorMap *m : {&it.T.r, &it.T.pa, &it.T.pb, &it.T.d, &it.T.m, &it.T.s, &it.T.qst, &it.T.past,
                                     &it.T.pbst})
            tensormap_acquire(m);
    }
    ku3_tile<8, 4>(it.T, A, k.y, it.ntiles);
}

cudaError_t batch_ku3_init_attributes() {
    return cudaFuncSetAttribute(b_ku3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, Ku3Shape<8, 4>::SMEM_ALLOC);
}

cudaError_t batch_ku3_pcg(const Ku3BatchItem *items, WorkList k3, const Modal<float> &M, cudaStream_t st) {
    if (k3.n < 1) return cudaSuccess;
    b_ku3_kernel<<<k3.n, 256, Ku3Shape<8, 4>::SMEM_ALLOC, st>>>(items, k3, M);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

cudaError_t batch_ku3_pad(const BatchItem *items, WorkList vec, int grid, cudaStream_t st) {
    if (vec.n < 1) return cudaSuccess;
    b_ku3_pad_kernel<<<std::max(1, std::min(grid, vec.n)), 256, 0, st>>>(items, vec);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    return e;
}

}  // namespace amk
