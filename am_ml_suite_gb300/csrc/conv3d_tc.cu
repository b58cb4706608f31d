// conv3d_tc.cu -- the 3x3x3 convolutions of the learned preconditioner on the
// 5th-generation tensor cores: tcgen05.mma with the accumulator in tensor memory,
// operands staged by tiled tensor copies (TMA) through a ring of shared-memory
// stages, one thread issuing the copies and one the MMAs.
//
// Forward / backward-data (implicit GEMM): a CTA owns M = 128 output voxels, an
// 8 (x) x 4 (y) x 4 (z) box of one batch entry, and all N = cout output
// channels.  K runs over the 27 taps x cin/16 channel chunks; for each (tap,
// chunk) one copy brings the tap-shifted 8x4x4 input box (8 channels at a time,
// so it lands in the K-major core-matrix layout of tc.cuh) -- outside the grid
// the copy engine fills zeros, which is the convolution's zero padding -- and
// one copy the N x 16 weights of that tap; one MMA of 128 x N x 16 consumes
// them.  The epilogue reads the 128 x N FP32 accumulator out of tensor memory
// (each warp its 32 lanes), applies ReLU, and writes BF16 and/or FP32 channels.
//
// Backward-weight: dW[tap][cout][cin] = sum_v dY[v][cout] X[v + tap][cin] as a
// GEMM with M = cout (padded to 128: rows past cout read zeros), N = cin, K =
// voxels; both operands are channel-contiguous (MN-major) boxes of 128 voxels.
// A CTA reduces a run of voxel boxes for one tap into tensor memory and adds its
// 128 x cin partial into the FP32 gradient with atomics.
//
// Every wait is bounded (200 ms; a healthy one lasts microseconds); a CTA whose wait runs out
// raises the error flag, lets the copies and MMAs it issued finish (bounded
// again), frees its tensor memory and returns; later CTAs see the flag and skip
// their work, and the host reports the launch as timed out.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "conv3d.cuh"
#include "tc.cuh"

namespace amk {

namespace {

// bound of every wait (a healthy wait lasts microseconds)
constexpr unsigned long long kWaitNs = 200000000ull;

__device__ __forceinline__ bool wait(uint64_t *bar, unsigned parity) { return bulk::bar_wait(bar, parity, kWaitNs); }
constexpr int kBoxX = 8, kBoxY = 4, kBoxZ = 4;  // 128 voxels per tile
constexpr int kAHalf = 128 * 16;                // bytes of one 8-channel half of an A tile


struct TcFwdArgs {
    __nv_bfloat16 *y;
    int ycs, yco;
    float *yf;
    int yfcs, yfco;
    int dz, dy, dx;
    int tiles_x, tiles_y, tiles_z;
    int cin, relu;
    int wrow0;  // first weight row (output channel) of this launch; the output pointer is offset to match
    int *err;
};

__device__ __forceinline__ void raise_err(int *err) {
    if (err) atomicExch(err, 1);
}

// Persistent forward kernel.  Warp 0 (one thread) issues the tensor copies of
// every (tile, K step) into a ring of stages; warp 1 (one thread) issues the MMAs
// of a tile into one of two TMEM accumulators (N columns each) and commits it;
// warps 2-5 read a finished accumulator (warp w: TMEM lanes 32 (w % 4) ...), write
// the outputs and hand the accumulator back -- so one tile's epilogue runs under
// the next tile's MMAs and copies.  A K step stages CW channels of one tap: a
// 128-voxel box of the input and the N x CW weights, in the K-major layout with
// CW*2-byte swizzled rows; it feeds CW / 16 MMAs of 128 x N x 16.
constexpr int kMaxStages = 32;
constexpr int kFwdThreads = 192;

__host__ __device__ constexpr int stage_bytes_fwd2(int n, int cw) {
    return (128 * cw * 2 + n * cw * 2 + 1023) / 1024 * 1024;
}

template <int N, int CW>
__global__ void __launch_bounds__(kFwdThreads, 1) conv_tc_fwd_kernel(const __grid_constant__ CUtensorMap mx,
                                                                     const __grid_constant__ CUtensorMap mw,
                                                                     TcFwdArgs A, int ntiles, int stages) {
    constexpr int STAGE = stage_bytes_fwd2(N, CW);
    constexpr int A_BYTES = 128 * CW * 2;
    constexpr uint32_t ROW = CW * 2;  // swizzle span / row bytes
    constexpr uint32_t TCOLS = 2 * N <= 32 ? 32 : 2 * N <= 64 ? 64 : 2 * N <= 128 ? 128 : 2 * N <= 256 ? 256 : 512;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, N);
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[kMaxStages], empty[kMaxStages], acc_full[2], acc_empty[2], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int aborted;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    volatile int &stop = aborted;  // written by whichever role gives up a wait
    if (A.err && *reinterpret_cast<volatile int *>(A.err)) return;

    if (warp == 0) tc::tmem_alloc(&tmem_slot, TCOLS);
    if (tid == 32) {
        for (int s = 0; s < stages; ++s) {
            bulk::bar_init(&full[s], 1);
            bulk::bar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            bulk::bar_init(&acc_full[b], 1);
            bulk::bar_init(&acc_empty[b], 4);
        }
        bulk::bar_init(&drain, 1);
        bulk::bar_init_fence();
        aborted = 0;
        tc::prefetch_map(&mx);
        tc::prefetch_map(&mw);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const int kch = A.cin / CW;
    const int ksteps = 27 * kch;
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == 0) {
        if (lane == 0) {
            long long g = 0, issued = 0;
            for (int i = 0; i < my_tiles && !stop; ++i) {
                int b = blockIdx.x + i * gridDim.x;
                const int tx = b % A.tiles_x;
                b /= A.tiles_x;
                const int ty = b % A.tiles_y;
                b /= A.tiles_y;
                const int tz = b % A.tiles_z;
                const int nb = b / A.tiles_z;
                const int x0 = tx * kBoxX, y0 = ty * kBoxY, z0 = tz * kBoxZ;
                for (int k = 0; k < ksteps; ++k, ++g) {
                    const int s = (int)(g % stages);
                    const long long use = g / stages;
                    if (use > 0 && !wait(&empty[s], (unsigned)((use - 1) & 1))) {
                        stop = 1;
                        break;
                    }
                    const int tap = k / kch, kc = k - tap * kch;
                    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
                    uint8_t *sa = smem + s * STAGE;
                    bulk::bar_expect(&full[s], A_BYTES + N * CW * 2);
                    tc::load_5d(sa, &mx, kc * CW, x0 + dx, y0 + dy, z0 + dz, nb, &full[s]);
                    tc::load_3d(sa + A_BYTES, &mw, kc * CW, A.wrow0, tap, &full[s]);
                    issued = g + 1;
                }
            }
            // every copy issued lands before the CTA can leave
            for (long long q = issued > stages ? issued - stages : 0; q < issued; ++q)
                wait(&full[q % stages], (unsigned)((q / stages) & 1));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            long long g = 0;
            for (int i = 0; i < my_tiles && !stop; ++i) {
                const int buf = i & 1;
                if (i >= 2 && !wait(&acc_empty[buf], (unsigned)(((i >> 1) - 1) & 1))) {
                    stop = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t d = tmem + (uint32_t)(buf * N);
                for (int k = 0; k < ksteps; ++k, ++g) {
                    const int s = (int)(g % stages);
                    if (!wait(&full[s], (unsigned)((g / stages) & 1))) {
                        stop = 1;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint8_t *sa = smem + s * STAGE;
                    const uint8_t *sb = sa + A_BYTES;
#pragma unroll
                    for (int kk = 0; kk < CW / 16; ++kk)
                        tc::mma_bf16(d, tc::smem_desc_sw(sa + kk * 32, ROW), tc::smem_desc_sw(sb + kk * 32, ROW),
                                     IDESC, (k > 0 || kk > 0) ? 1u : 0u);
                    tc::mma_commit(&empty[s]);
                }
                if (stop) break;
                tc::mma_commit(&acc_full[buf]);
            }
            tc::mma_commit(&drain);  // completes once every MMA issued has
        }
    } else {
        // epilogue warps 2-5: TMEM lane quadrant warp % 4
        const int q = warp & 3;
        const int m = q * 32 + lane;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            const bool ok = wait(&acc_full[buf], (unsigned)((i >> 1) & 1));
            if (!ok || stop) {
                if (lane == 0) stop = 1;
                break;
            }
            tc::fence_after_sync();
            int b = blockIdx.x + i * gridDim.x;
            const int tx = b % A.tiles_x;
            b /= A.tiles_x;
            const int ty = b % A.tiles_y;
            b /= A.tiles_y;
            const int tz = b % A.tiles_z;
            const int nb = b / A.tiles_z;
            const int x = tx * kBoxX + (m & 7), y = ty * kBoxY + ((m >> 3) & 3), z = tz * kBoxZ + (m >> 5);
            const bool in = x < A.dx && y < A.dy && z < A.dz;
            const long long vox = (((long long)nb * A.dz + z) * A.dy + y) * A.dx + x;
#pragma unroll
            for (int c0 = 0; c0 < N; c0 += 16) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * N + c0), v);
                if (!in) continue;
                if (A.y) {
                    uint4 pk[2];
                    uint32_t *w = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        float a = v[2 * t], bb = v[2 * t + 1];
                        if (A.relu) {
                            a = fmaxf(a, 0.f);
                            bb = fmaxf(bb, 0.f);
                        }
                        const __nv_bfloat162 h = __floats2bfloat162_rn(a, bb);
                        w[t] = *reinterpret_cast<const uint32_t *>(&h);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(A.y + vox * A.ycs + A.yco + c0);
                    dst[0] = pk[0];
                    dst[1] = pk[1];
                }
                if (A.yf) {
                    float4 *dst = reinterpret_cast<float4 *>(A.yf + vox * A.yfcs + A.yfco + c0);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        float4 o = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
                        if (A.relu) {
                            o.x = fmaxf(o.x, 0.f);
                            o.y = fmaxf(o.y, 0.f);
                            o.z = fmaxf(o.z, 0.f);
                            o.w = fmaxf(o.w, 0.f);
                        }
                        dst[t] = o;
                    }
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[buf]);
        }
    }
    __syncwarp();
    // the MMAs issued have completed before tensor memory is released
    wait(&drain, 0);
    tc::fence_before_sync();
    __syncthreads();
    if (stop && tid == 0) raise_err(A.err);
    if (warp == 0) tc::tmem_free(tmem, TCOLS);
}

// ---- plane-marching forward (small channel counts) --------------------------------
// A CTA owns an 8 (x) x 16 (y) column of output voxels and a run of z planes of
// one batch entry and marches up z.  Input planes z0-1 .. z1 (10 x 18 voxels: the
// column with its halo) pass through a ring of MR shared-memory slots, one tiled
// copy per 8 channels landing in the no-swizzle K-major layout (voxel rows of 16
// bytes, x fastest).  For output plane z the A operand of tap (dx, dy, dz) is
// then the slot of plane z+dz read from ((1+dx) + 10 (1+dy)) voxels on: 8
// consecutive x rows form a core matrix and the 16 y rows follow 10 voxels (160
// bytes) apart, the uniform group stride of the descriptor -- no data moves per
// tap.  The 27 x cin x N weights stay resident for the CTA's whole life.  Warp
// roles and the double-buffered accumulator are those of the persistent kernel.
constexpr int kMarchRing = 4;
constexpr int kPlaneHalf = 2944;  // bytes of one 8-channel half of a staged plane (180 x 16, padded to 128)

template <int N, int CIN>
__global__ void __launch_bounds__(kFwdThreads, 1) conv_tc_march_kernel(const __grid_constant__ CUtensorMap mx,
                                                                       const __grid_constant__ CUtensorMap mw,
                                                                       TcFwdArgs A, int tiles_y16, int zrun,
                                                                       int nitems) {
    constexpr int KCH = CIN / 16;
    constexpr int SLOT = KCH * 2 * kPlaneHalf;
    constexpr int WBYTES = 27 * KCH * 2 * N * 16;
    constexpr uint32_t TCOLS = 2 * N <= 32 ? 32 : 2 * N <= 64 ? 64 : 128;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, N);
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t pfull[kMarchRing], pempty[kMarchRing], wfull, acc_full[2], acc_empty[2], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int aborted;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *wsm = smem;                           // weights [27][KCH][2 halves][N][16 B]
    uint8_t *ring = smem + (WBYTES + 1023) / 1024 * 1024;  // [MR][KCH][2][kPlaneHalf]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    volatile int &stop = aborted;
    if (A.err && *reinterpret_cast<volatile int *>(A.err)) return;

    if (warp == 0) tc::tmem_alloc(&tmem_slot, TCOLS);
    if (tid == 32) {
        for (int r = 0; r < kMarchRing; ++r) {
            bulk::bar_init(&pfull[r], 1);
            bulk::bar_init(&pempty[r], 1);
        }
        bulk::bar_init(&wfull, 1);
        for (int b = 0; b < 2; ++b) {
            bulk::bar_init(&acc_full[b], 1);
            bulk::bar_init(&acc_empty[b], 4);
        }
        bulk::bar_init(&drain, 1);
        bulk::bar_init_fence();
        aborted = 0;
        tc::prefetch_map(&mx);
        tc::prefetch_map(&mw);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const int tz_runs = (A.dz + zrun - 1) / zrun;
    // work item -> (x tile, y tile, z run, batch entry)
    auto item = [&](int it, int &x0, int &y0, int &z0, int &z1, int &nb) {
        int b = it;
        const int tx = b % A.tiles_x;
        b /= A.tiles_x;
        const int ty = b % tiles_y16;
        b /= tiles_y16;
        const int tzr = b % tz_runs;
        nb = b / tz_runs;
        x0 = tx * 8;
        y0 = ty * 16;
        z0 = tzr * zrun;
        z1 = min(z0 + zrun, A.dz);
    };

    if (warp == 0) {
        if (lane == 0) {
            bulk::bar_expect(&wfull, WBYTES);
            for (int t = 0; t < 27; ++t)
                for (int kc = 0; kc < KCH; ++kc)
                    for (int h = 0; h < 2; ++h)
                        tc::load_3d(wsm + ((t * KCH + kc) * 2 + h) * N * 16, &mw, kc * 16 + h * 8, 0, t, &wfull);
            long long G = 0, issued = 0;
            for (int it = blockIdx.x; it < nitems && !stop; it += gridDim.x) {
                int x0, y0, z0, z1, nb;
                item(it, x0, y0, z0, z1, nb);
                for (int j = 0; j < z1 - z0 + 2; ++j, ++G) {
                    const int r = (int)(G % kMarchRing);
                    const long long use = G / kMarchRing;
                    if (use > 0 && !wait(&pempty[r], (unsigned)((use - 1) & 1))) {
                        stop = 1;
                        break;
                    }
                    uint8_t *slot = ring + r * SLOT;
                    bulk::bar_expect(&pfull[r], KCH * 2 * 2880);
                    for (int kc = 0; kc < KCH; ++kc)
                        for (int h = 0; h < 2; ++h)
                            tc::load_5d(slot + (kc * 2 + h) * kPlaneHalf, &mx, kc * 16 + h * 8, x0 - 1, y0 - 1,
                                        z0 - 1 + j, nb, &pfull[r]);
                    issued = G + 1;
                }
            }
            for (long long q = issued > kMarchRing ? issued - kMarchRing : 0; q < issued; ++q)
                wait(&pfull[q % kMarchRing], (unsigned)((q / kMarchRing) & 1));
            wait(&wfull, 0);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            if (!wait(&wfull, 0)) stop = 1;
            long long G0 = 0;  // global index of the item's first plane
            int i = 0;         // accumulator uses (output planes) so far
            for (int it = blockIdx.x; it < nitems && !stop; it += gridDim.x) {
                int x0, y0, z0, z1, nb;
                item(it, x0, y0, z0, z1, nb);
                const int S = z1 - z0;
                long long ready = G0;  // planes G0 .. ready-1 are known to be full
                for (int s = 0; s < S && !stop; ++s, ++i) {
                    for (; ready <= G0 + s + 2; ++ready)
                        if (!wait(&pfull[ready % kMarchRing], (unsigned)((ready / kMarchRing) & 1))) {
                            stop = 1;
                            break;
                        }
                    const int buf = i & 1;
                    if (!stop && i >= 2 && !wait(&acc_empty[buf], (unsigned)(((i >> 1) - 1) & 1))) stop = 1;
                    if (stop) break;
                    tc::fence_after_sync();
                    const uint32_t d = tmem + (uint32_t)(buf * N);
                    // descriptors of the three planes z-1, z, z+1 and of the weights; a tap
                    // adds a constant to the start-address field (addresses stay < 256 KB)
                    const int r0 = (int)((G0 + s) & (kMarchRing - 1));
                    uint64_t pd[3];
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        pd[q] = tc::smem_desc(ring + ((r0 + q) & (kMarchRing - 1)) * SLOT, kPlaneHalf, 160);
                    const uint64_t wd = tc::smem_desc(wsm, N * 16, 128);
#pragma unroll
                    for (int t = 0; t < 27; ++t) {
                        const int off = ((1 + t % 3 - 1) + 10 * (1 + (t / 3) % 3 - 1)) * 16;
#pragma unroll
                        for (int kc = 0; kc < KCH; ++kc)
                            tc::mma_bf16(d, pd[t / 9] + (uint64_t)((kc * 2 * kPlaneHalf + off) >> 4),
                                         wd + (uint64_t)(((t * KCH + kc) * 2 * N * 16) >> 4), IDESC,
                                         (t > 0 || kc > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&acc_full[buf]);
                    tc::mma_commit(&pempty[(G0 + s) % kMarchRing]);  // plane z-1 of this output plane is done
                }
                if (stop) break;
                // the item's last two planes
                tc::mma_commit(&pempty[(G0 + S) % kMarchRing]);
                tc::mma_commit(&pempty[(G0 + S + 1) % kMarchRing]);
                G0 += S + 2;
            }
            tc::mma_commit(&drain);
        }
    } else {
        const int q = warp & 3;
        const int m = q * 32 + lane;
        int i = 0;
        for (int it = blockIdx.x; it < nitems && !stop; it += gridDim.x) {
            int x0, y0, z0, z1, nb;
            item(it, x0, y0, z0, z1, nb);
            for (int z = z0; z < z1; ++z, ++i) {
                const int buf = i & 1;
                if (!wait(&acc_full[buf], (unsigned)((i >> 1) & 1)) || stop) {
                    if (lane == 0) stop = 1;
                    break;
                }
                tc::fence_after_sync();
                const int x = x0 + (m & 7), y = y0 + (m >> 3);
                const bool in = x < A.dx && y < A.dy;
                const long long vox = (((long long)nb * A.dz + z) * A.dy + y) * A.dx + x;
#pragma unroll
                for (int c0 = 0; c0 < N; c0 += 16) {
                    float v[16];
                    tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * N + c0), v);
                    if (!in) continue;
                    if (A.y) {
                        uint4 pk[2];
                        uint32_t *w = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
                        for (int t = 0; t < 8; ++t) {
                            float a = v[2 * t], bb = v[2 * t + 1];
                            if (A.relu) {
                                a = fmaxf(a, 0.f);
                                bb = fmaxf(bb, 0.f);
                            }
                            const __nv_bfloat162 h2 = __floats2bfloat162_rn(a, bb);
                            w[t] = *reinterpret_cast<const uint32_t *>(&h2);
                        }
                        uint4 *dst = reinterpret_cast<uint4 *>(A.y + vox * A.ycs + A.yco + c0);
                        dst[0] = pk[0];
                        dst[1] = pk[1];
                    }
                    if (A.yf) {
                        float4 *dst = reinterpret_cast<float4 *>(A.yf + vox * A.yfcs + A.yfco + c0);
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            float4 o = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
                            if (A.relu) {
                                o.x = fmaxf(o.x, 0.f);
                                o.y = fmaxf(o.y, 0.f);
                                o.z = fmaxf(o.z, 0.f);
                                o.w = fmaxf(o.w, 0.f);
                            }
                            dst[t] = o;
                        }
                    }
                }
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&acc_empty[buf]);
            }
        }
    }
    __syncwarp();
    wait(&drain, 0);
    tc::fence_before_sync();
    __syncthreads();
    if (stop && tid == 0) raise_err(A.err);
    if (warp == 0) tc::tmem_free(tmem, TCOLS);
}

// ---- backward-weight ------------------------------------------------------------
// A CTA: one tap, one 128-row block of output channels (M), all input channels
// (N = cin <= 256, in one MMA per 16 voxels), a run of `boxes_per_cta` voxel
// boxes.  Per box (128 voxels = 8 K steps of 16) the stage holds dY^T -- 16
// channel groups x 128 voxels x 8 channels (MN-major core matrices: 8 voxels x 8
// channels, 128 bytes) -- and X^T of the tap-shifted box, cin/8 groups likewise.
struct TcWgArgs {
    float *dw;  // [27][cout][cin_total]; this launch adds columns cin_off .. cin_off + CIN
    int dz, dy, dx;
    int tiles_x, tiles_y, tiles_z, ntiles;  // voxel boxes of the whole batch
    int cin, cout, boxes_per_cta;
    int cin_total, cin_off;
    int *err;
};

__host__ __device__ constexpr int stage_bytes_wg(int cin) { return ((16 + cin / 8) * kAHalf + 1023) / 1024 * 1024; }

template <int CIN>
__global__ void __launch_bounds__(128) conv_tc_wgrad_kernel(const __grid_constant__ CUtensorMap mdy,
                                                            const __grid_constant__ CUtensorMap mx, TcWgArgs A) {
    constexpr int STAGES = 2;
    constexpr int STAGE = stage_bytes_wg(CIN);
    constexpr uint32_t TCOLS = CIN <= 32 ? 32 : CIN <= 64 ? 64 : CIN <= 128 ? 128 : 256;
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                               ((uint32_t)(CIN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int aborted;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y, mblk = blockIdx.z;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int box0 = blockIdx.x * A.boxes_per_cta;
    const int nbox = min(A.boxes_per_cta, A.ntiles - box0);
    if (A.err && *reinterpret_cast<volatile int *>(A.err)) return;

    if (warp == 0) tc::tmem_alloc(&tmem_slot, TCOLS);
    if (tid == 32) {
        for (int s = 0; s < STAGES; ++s) {
            bulk::bar_init(&full[s], 1);
            bulk::bar_init(&empty[s], 1);
        }
        bulk::bar_init(&done, 1);
        bulk::bar_init_fence();
        aborted = 0;
        tc::prefetch_map(&mdy);
        tc::prefetch_map(&mx);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr int GX = CIN / 8;  // channel groups of X

    if (tid == 0) {
        int issued = 0;
        for (int i = 0; i < nbox; ++i) {
            const int s = i % STAGES, use = i / STAGES;
            if (use > 0 && !wait(&empty[s], (use - 1) & 1)) {
                aborted = 1;
                break;
            }
            int t = box0 + i;
            const int tx = t % A.tiles_x;
            t /= A.tiles_x;
            const int ty = t % A.tiles_y;
            t /= A.tiles_y;
            const int tz = t % A.tiles_z;
            const int nb = t / A.tiles_z;
            const int x0 = tx * kBoxX, y0 = ty * kBoxY, z0 = tz * kBoxZ;
            uint8_t *sa = smem + s * STAGE;
            uint8_t *sb = sa + 16 * kAHalf;
            bulk::bar_expect(&full[s], (16 + GX) * kAHalf);
            // dY: channel groups of this M block (beyond cout the copy reads zeros)
            for (int g = 0; g < 16; ++g)
                tc::load_5d(sa + g * kAHalf, &mdy, mblk * 128 + g * 8, x0, y0, z0, nb, &full[s]);
            for (int g = 0; g < GX; ++g)
                tc::load_5d(sb + g * kAHalf, &mx, g * 8, x0 + dx, y0 + dy, z0 + dz, nb, &full[s]);
            issued = i + 1;
        }
        for (int i = std::max(0, issued - STAGES); i < issued; ++i)
            wait(&full[i % STAGES], (i / STAGES) & 1);
    } else if (tid == 32) {
        int kstep = 0;
        for (int i = 0; i < nbox; ++i) {
            const int s = i % STAGES, use = i / STAGES;
            if (!wait(&full[s], use & 1)) {
                aborted = 1;
                break;
            }
            tc::fence_after_sync();
            const uint8_t *sa = smem + s * STAGE;
            const uint8_t *sb = sa + 16 * kAHalf;
            // 8 K steps of 16 voxels: MN-major core matrices are 8 voxels x 16 B,
            // two of them (256 B) per K step; channel groups kAHalf apart
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                tc::mma_bf16(tmem, tc::smem_desc(sa + kk * 256, 128, kAHalf), tc::smem_desc(sb + kk * 256, 128, kAHalf),
                             IDESC, kstep > 0 ? 1u : 0u);
                ++kstep;
            }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&done);
    }
    __syncwarp();
    const bool ok = wait(&done, 0);
    tc::fence_after_sync();
    if (!ok || aborted) {
        if (lane == 0) raise_err(A.err);
    } else if (nbox > 0) {
        const int co = mblk * 128 + warp * 32 + lane;
        float *dst = A.dw + ((size_t)tap * A.cout + co) * A.cin_total + A.cin_off;
#pragma unroll 1
        for (int c0 = 0; c0 < CIN; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (co < A.cout) {
#pragma unroll
                for (int i = 0; i < 16; ++i) atomicAdd(dst + c0 + i, v[i]);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, TCOLS);
}

// ---- host ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// BF16 activations [n][dz][dy][dx][cstride] read from channel `coff` on: a rank-5
// map (channel, x, y, z, batch) whose box is box_c channels x 8 x 4 x 4 voxels;
// zero fill outside the tensor
bool act_map(CUtensorMap *m, const Grid5 &g, TensorView t, int channels, int box_c = 8,
             CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_NONE) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t cs = (cuuint64_t)t.cstride * 2;
    const cuuint64_t dims[5] = {(cuuint64_t)channels, (cuuint64_t)g.dx, (cuuint64_t)g.dy, (cuuint64_t)g.dz,
                                (cuuint64_t)g.n};
    const cuuint64_t strides[4] = {cs, cs * g.dx, cs * g.dx * g.dy, cs * g.dx * g.dy * g.dz};
    const cuuint32_t box[5] = {(cuuint32_t)box_c, kBoxX, kBoxY, kBoxZ, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const void *base = static_cast<const __nv_bfloat16 *>(t.p) + t.coff;
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the same map with the staged-plane box of the plane-marching kernel: 8
// channels x 10 x 18 voxels x 1 plane
bool plane_map(CUtensorMap *m, const Grid5 &g, TensorView t, int channels) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t cs = (cuuint64_t)t.cstride * 2;
    const cuuint64_t dims[5] = {(cuuint64_t)channels, (cuuint64_t)g.dx, (cuuint64_t)g.dy, (cuuint64_t)g.dz,
                                (cuuint64_t)g.n};
    const cuuint64_t strides[4] = {cs, cs * g.dx, cs * g.dx * g.dy, cs * g.dx * g.dy * g.dz};
    const cuuint32_t box[5] = {8, 10, 18, 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const void *base = static_cast<const __nv_bfloat16 *>(t.p) + t.coff;
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// BF16 weights [27][rows][cols]: box of box_c columns x box_rows rows of one tap
bool weight_map_rows(CUtensorMap *m, const __nv_bfloat16 *w, int rows, int box_rows, int cols, int box_c,
                     CUtensorMapSwizzle sw) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, 27};
    const cuuint64_t strides[2] = {(cuuint64_t)cols * 2, (cuuint64_t)cols * rows * 2};
    const cuuint32_t box[3] = {(cuuint32_t)box_c, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(w), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// BF16 weights [27][rows][cols]: box of box_c columns x `rows` rows of one tap
bool weight_map(CUtensorMap *m, const __nv_bfloat16 *w, int rows, int cols, int box_c = 8,
                CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_NONE) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, 27};
    const cuuint64_t strides[2] = {(cuuint64_t)cols * 2, (cuuint64_t)cols * rows * 2};
    const cuuint32_t box[3] = {(cuuint32_t)box_c, (cuuint32_t)rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(w), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int *g_err = nullptr;  // device error flag of the bounded waits (per process, device 0 context)

int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

template <int N, int CW>
cudaError_t launch_fwd(const CUtensorMap &mx, const CUtensorMap &mw, const TcFwdArgs &a, int ntiles,
                       cudaStream_t st) {
    constexpr int STAGE = stage_bytes_fwd2(N, CW);
    // two CTAs per SM where their accumulators fit the 512 TMEM columns together
    constexpr int per_sm = 2 * N <= 256 ? 2 : 1;
    const int stages = std::max(2, std::min(kMaxStages, (per_sm == 2 ? 104 : 200) * 1024 / STAGE));
    const int smem = stages * STAGE + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(conv_tc_fwd_kernel<N, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int grid = std::min(ntiles, per_sm * sm_count());
    conv_tc_fwd_kernel<N, CW><<<grid, kFwdThreads, smem, st>>>(mx, mw, a, ntiles, stages);
    return cudaGetLastError();
}

template <int N, int CIN>
cudaError_t launch_march(const CUtensorMap &mx, const CUtensorMap &mw, const TcFwdArgs &a, const Grid5 &g,
                         cudaStream_t st) {
    constexpr int KCH = CIN / 16;
    constexpr int WBYTES = 27 * KCH * 2 * N * 16;
    const int smem = (WBYTES + 1023) / 1024 * 1024 + kMarchRing * KCH * 2 * kPlaneHalf + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(conv_tc_march_kernel<N, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int sms = sm_count();
    const int ty16 = (g.dy + 15) / 16;
    const long long columns = (long long)a.tiles_x * ty16 * g.n;
    // a CTA spends most of a plane step waiting on copies and MMAs: as many CTAs per
    // SM as registers and shared memory allow (at most 4; their accumulators take at
    // most 4 x 64 of the 512 tensor-memory columns), about four work items each, runs
    // of at least 4 planes
    static int per_sm = 0;
    if (!per_sm) {
        int nb = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, conv_tc_march_kernel<N, CIN>, kFwdThreads, smem) !=
            cudaSuccess)
            nb = 1;
        per_sm = std::max(1, std::min(4, nb));
    }
    const long long ctas = (long long)per_sm * sms;
    const long long runs = std::max<long long>(1, std::min<long long>((4LL * ctas + columns - 1) / columns,
                                                                      (g.dz + 3) / 4));
    const int zrun = (int)((g.dz + runs - 1) / runs);
    const long long nitems = columns * ((g.dz + zrun - 1) / zrun);
    if (nitems > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int grid = (int)std::min<long long>(nitems, ctas);
    conv_tc_march_kernel<N, CIN><<<grid, kFwdThreads, smem, st>>>(mx, mw, a, ty16, zrun, (int)nitems);
    return cudaGetLastError();
}

template <int CW>
cudaError_t launch_fwd_n(int cout, const CUtensorMap &mx, const CUtensorMap &mw, const TcFwdArgs &a, int ntiles,
                         cudaStream_t st) {
    switch (cout) {
        case 16: return launch_fwd<16, CW>(mx, mw, a, ntiles, st);
        case 32: return launch_fwd<32, CW>(mx, mw, a, ntiles, st);
        case 48: return launch_fwd<48, CW>(mx, mw, a, ntiles, st);
        case 64: return launch_fwd<64, CW>(mx, mw, a, ntiles, st);
        case 96: return launch_fwd<96, CW>(mx, mw, a, ntiles, st);
        case 128: return launch_fwd<128, CW>(mx, mw, a, ntiles, st);
        case 192: return launch_fwd<192, CW>(mx, mw, a, ntiles, st);
        default: return launch_fwd<256, CW>(mx, mw, a, ntiles, st);
    }
}

template <int CIN>
cudaError_t launch_wg(const CUtensorMap &mdy, const CUtensorMap &mx, const TcWgArgs &a, dim3 grid, cudaStream_t st) {
    const int smem = 2 * stage_bytes_wg(CIN) + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(conv_tc_wgrad_kernel<CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    conv_tc_wgrad_kernel<CIN><<<grid, 128, smem, st>>>(mdy, mx, a);
    return cudaGetLastError();
}

cudaError_t err_flag(int **out) {
    if (!g_err) {
        cudaError_t e = cudaMalloc(&g_err, sizeof(int));
        if (e != cudaSuccess) return e;
        e = cudaMemset(g_err, 0, sizeof(int));
        if (e != cudaSuccess) return e;
    }
    *out = g_err;
    return cudaSuccess;
}

bool tc_aligned(TensorView t) {
    return t.p && t.cstride % 8 == 0 && t.coff % 8 == 0 && (reinterpret_cast<uintptr_t>(t.p) & 15) == 0;
}

}  // namespace

namespace {

bool fwd_n_ok(int n) { return n == 16 || n == 32 || n == 48 || n == 64 || n == 96 || n == 128 || n == 192 || n == 256; }

// output channels row0 .. row0 + n of a convolution with cout_total weight rows
cudaError_t fwd_generic(const Grid5 &g, TensorView x, int cin, const __nv_bfloat16 *w, int cout_total, int row0,
                        int n, TensorView y, TensorView yf, int relu, cudaStream_t st) {
    // channels per K step: 64 (128-byte swizzled rows) where cin allows, else 32 or 16
    const int cw = cin % 64 == 0 ? 64 : cin % 32 == 0 ? 32 : 16;
    const CUtensorMapSwizzle sw = cw == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                  : cw == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                             : CU_TENSOR_MAP_SWIZZLE_32B;
    CUtensorMap mx, mw;
    if (!act_map(&mx, g, x, cin, cw, sw) || !weight_map_rows(&mw, w, cout_total, n, cin, cw, sw))
        return cudaErrorInvalidValue;
    TcFwdArgs a{};
    a.y = y.p ? static_cast<__nv_bfloat16 *>(y.p) : nullptr;
    a.ycs = y.cstride;
    a.yco = y.coff + row0;
    a.yf = static_cast<float *>(yf.p);
    a.yfcs = yf.cstride;
    a.yfco = yf.coff + row0;
    a.dz = g.dz;
    a.dy = g.dy;
    a.dx = g.dx;
    a.tiles_x = (g.dx + kBoxX - 1) / kBoxX;
    a.tiles_y = (g.dy + kBoxY - 1) / kBoxY;
    a.tiles_z = (g.dz + kBoxZ - 1) / kBoxZ;
    a.cin = cin;
    a.relu = relu;
    a.wrow0 = row0;
    cudaError_t e = err_flag(&a.err);
    if (e != cudaSuccess) return e;
    const long long ntiles = (long long)a.tiles_x * a.tiles_y * a.tiles_z * g.n;
    if (ntiles < 1 || ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (cw == 64) return launch_fwd_n<64>(n, mx, mw, a, (int)ntiles, st);
    if (cw == 32) return launch_fwd_n<32>(n, mx, mw, a, (int)ntiles, st);
    return launch_fwd_n<16>(n, mx, mw, a, (int)ntiles, st);
}

}  // namespace

cudaError_t conv3d_fwd_tc(const Grid5 &g, TensorView x, int cin, const __nv_bfloat16 *w, int cout, TensorView y,
                          TensorView yf, int relu, cudaStream_t st) {
    // more than 256 output channels: two launches of half the channels each (an MMA's N is at most 256)
    const bool split = cout > 256 && cout % 32 == 0 && fwd_n_ok(cout / 2);
    if (cin % 16 || cin > 512 || (!fwd_n_ok(cout) && !split) || !tc_aligned(x) ||
        (reinterpret_cast<uintptr_t>(w) & 15) || (y.p && !tc_aligned(y)) ||
        (yf.p && (yf.cstride % 4 || yf.coff % 4 || (reinterpret_cast<uintptr_t>(yf.p) & 15))) ||
        x.coff + cin > x.cstride)
        return cudaErrorInvalidValue;
    if (cin <= 48 && cout <= 32) {
        // small channel counts: the plane-marching kernel (weights resident, planes reused by all taps)
        CUtensorMap mx, mw;
        if (!plane_map(&mx, g, x, cin) || !weight_map(&mw, w, cout, cin)) return cudaErrorInvalidValue;
        TcFwdArgs a{};
        a.y = static_cast<__nv_bfloat16 *>(y.p);
        a.ycs = y.cstride;
        a.yco = y.coff;
        a.yf = static_cast<float *>(yf.p);
        a.yfcs = yf.cstride;
        a.yfco = yf.coff;
        a.dz = g.dz;
        a.dy = g.dy;
        a.dx = g.dx;
        a.tiles_x = (g.dx + 7) / 8;
        a.tiles_y = (g.dy + 15) / 16;
        a.tiles_z = g.dz;
        a.cin = cin;
        a.relu = relu;
        cudaError_t e = err_flag(&a.err);
        if (e != cudaSuccess) return e;
        const int key = cin * 1000 + cout;
        switch (key) {
            case 16016: return launch_march<16, 16>(mx, mw, a, g, st);
            case 16032: return launch_march<32, 16>(mx, mw, a, g, st);
            case 32016: return launch_march<16, 32>(mx, mw, a, g, st);
            case 32032: return launch_march<32, 32>(mx, mw, a, g, st);
            case 48016: return launch_march<16, 48>(mx, mw, a, g, st);
            case 48032: return launch_march<32, 48>(mx, mw, a, g, st);
            default: break;
        }
    }
    if (split) {
        const cudaError_t e = fwd_generic(g, x, cin, w, cout, 0, cout / 2, y, yf, relu, st);
        if (e != cudaSuccess) return e;
        return fwd_generic(g, x, cin, w, cout, cout / 2, cout / 2, y, yf, relu, st);
    }
    return fwd_generic(g, x, cin, w, cout, 0, cout, y, yf, relu, st);
}

namespace {

bool wg_cin_ok(int c) { return c == 16 || c == 32 || c == 48 || c == 64 || c == 96 || c == 128 || c == 192 || c == 256; }

// weight-gradient columns cin_off .. cin_off + cin of a convolution with cin_total inputs
cudaError_t wgrad_part(const Grid5 &g, TensorView x, int cin, int cin_total, int cin_off, TensorView dy, int cout,
                       float *dw, cudaStream_t st) {
    CUtensorMap mdy, mx;
    TensorView xs = x;
    xs.coff += cin_off;
    if (!act_map(&mdy, g, dy, cout) || !act_map(&mx, g, xs, cin)) return cudaErrorInvalidValue;
    TcWgArgs a{};
    a.dw = dw;
    a.dz = g.dz;
    a.dy = g.dy;
    a.dx = g.dx;
    a.tiles_x = (g.dx + kBoxX - 1) / kBoxX;
    a.tiles_y = (g.dy + kBoxY - 1) / kBoxY;
    a.tiles_z = (g.dz + kBoxZ - 1) / kBoxZ;
    a.ntiles = a.tiles_x * a.tiles_y * a.tiles_z * g.n;
    a.cin = cin;
    a.cout = cout;
    a.cin_total = cin_total;
    a.cin_off = cin_off;
    // enough CTAs for about four waves over 152 SMs, each reducing >= 4 boxes
    const long long per_tap = std::max<long long>(1, (152LL * 16) / (27LL * ((cout + 127) / 128)));
    a.boxes_per_cta = (int)std::max<long long>(4, (a.ntiles + per_tap - 1) / per_tap);
    cudaError_t e = err_flag(&a.err);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((a.ntiles + a.boxes_per_cta - 1) / a.boxes_per_cta), 27, (unsigned)((cout + 127) / 128));
    switch (cin) {
        case 16: return launch_wg<16>(mdy, mx, a, grid, st);
        case 32: return launch_wg<32>(mdy, mx, a, grid, st);
        case 48: return launch_wg<48>(mdy, mx, a, grid, st);
        case 64: return launch_wg<64>(mdy, mx, a, grid, st);
        case 96: return launch_wg<96>(mdy, mx, a, grid, st);
        case 128: return launch_wg<128>(mdy, mx, a, grid, st);
        case 192: return launch_wg<192>(mdy, mx, a, grid, st);
        default: return launch_wg<256>(mdy, mx, a, grid, st);
    }
}

}  // namespace

cudaError_t conv3d_wgrad_tc(const Grid5 &g, TensorView x, int cin, TensorView dy, int cout, float *dw,
                            cudaStream_t st) {
    // more than 256 input channels: two launches of half the columns each (an MMA's N is at most 256)
    const bool split = cin > 256 && wg_cin_ok(cin / 2) && cin % 32 == 0;
    if ((!wg_cin_ok(cin) && !split) || cout % 16 || cout > 256 || !tc_aligned(x) || !tc_aligned(dy) ||
        x.coff + cin > x.cstride || dy.coff + cout > dy.cstride)
        return cudaErrorInvalidValue;
    if (split) {
        const cudaError_t e = wgrad_part(g, x, cin / 2, cin, 0, dy, cout, dw, st);
        if (e != cudaSuccess) return e;
        return wgrad_part(g, x, cin / 2, cin, cin / 2, dy, cout, dw, st);
    }
    return wgrad_part(g, x, cin, cin, 0, dy, cout, dw, st);
}

cudaError_t conv3d_tc_error(int *flag, bool clear, cudaStream_t st) {
    *flag = 0;
    if (!g_err) return cudaSuccess;  // no tensor-core convolution has run
    cudaError_t e = cudaMemcpyAsync(flag, g_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && clear && *flag) e = cudaMemsetAsync(g_err, 0, sizeof(int), st);
    if (e == cudaSuccess && clear && *flag) e = cudaStreamSynchronize(st);
    return e;
}

}  // namespace amk
