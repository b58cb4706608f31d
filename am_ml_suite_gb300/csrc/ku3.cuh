// ku3.cuh -- FP32 PCG K*u with the node planes staged by TMA tensor copies.
//
// The operator and its arithmetic are those of ku2.cuh (k2::face_modes and
// k2::layer_math: Walsh-basis hex8 element transform, two elements per lane in
// packed FP32x2 instructions, face modes carried up z), and so is the warp
// layout: a warp owns two element rows of a tile and its lanes are element
// columns.  What changes is how data moves:
//   * each CTA keeps a ring of S shared-memory stages; a stage holds one node
//     plane of the tile with its halo -- r and p (3 components), the inverse
//     diagonal, the constraint bits -- and the element scales of the layer below
//     it, each brought in by one tiled cp.async.bulk.tensor copy issued by one
//     thread and completed on the stage's mbarrier, S-1 planes ahead of use;
//   * lanes read their values from shared memory at constant offsets, so the
//     per-layer global address arithmetic, the bounds predicates and the
//     exposed load latency of the register-direct form are gone; nodes and
//     elements outside the grid arrive as the copies' zero fill;
//   * the outputs q = mask(K p) and p = D^-1 r + beta p of the owned nodes are
//     written to a double-buffered shared tile and leave as two tensor stores
//     per layer (clipped to the grid by the copy engine).
// Tile: 28 owned node columns (x0 a multiple of 4: a tensor copy starts on a
// 16-byte boundary), 2W-1 owned node rows, a chunk of tz node planes.  Lane l
// holds node/element column x0-1+l (lanes 1..28 own their node).  For equal W
// the node values are bitwise those of ku2_kernel.
// All waits on the stages are bounded (one second); a CTA that runs out of time
// stops at the next layer, drains its copies, sets Scalars::kerr and still
// takes part in the p.q reduction, and the PCG update then ends the solve with
// ST_TIMEOUT.
#pragma once
#include <cuda.h>

#include "am_common.cuh"
#include "bulk.cuh"
#include "ku.cuh"
#include "ku2.cuh"

namespace amk {

// Tensor maps of one problem's FP32 PCG vectors (built on the host by
// ku3_make_maps, passed by value as a __grid_constant__ kernel parameter).
struct Ku3Maps {
    CUtensorMap r, pa, pb;     // loads: [3][nz+1][ny+1][nx+1] FP32, box 36 x (2W+1) x 1 x 3
    CUtensorMap d;             // load: inverse diagonal [nz+1][ny+1][nx+1], box 36 x (2W+1) x 1
    CUtensorMap m;             // load: constraint bits (padded copy, 16-byte rows), box 48 x (2W+1) x 1
    CUtensorMap s;             // load: element scales (padded copy) [nz][ny][nx], box 36 x 2W x 1
    CUtensorMap qst, past, pbst;  // stores: box 28 x (2W-1) x 1 x 1 (one per component)
};

struct Ku3Args {
    Modal<float> M;
    double *partial;  // per-tile p.q
    Scalars *S;
    int tiles_x, tiles_y, tz, nz;
};

template <int W, int S>
struct Ku3Shape {
    static constexpr int NT = 32 * W;
    static constexpr int TX = 28;         // owned node columns
    static constexpr int TY = 2 * W - 1;  // owned node rows
    static constexpr int BX = 36;         // staged node / element columns x0-4 .. x0+31
    static constexpr int BY = 2 * W + 1;  // staged node rows y0-1 .. y0+2W-1
    static constexpr int BYE = 2 * W;     // staged element rows y0-1 .. y0+2W-2
    static constexpr int BXM = 48;        // staged constraint-bit columns (x start a multiple of 16)
    static constexpr int r128(int b) { return (b + 127) / 128 * 128; }
    static constexpr int VEC_B = 3 * BY * BX * 4;
    static constexpr int DIN_B = BY * BX * 4;
    static constexpr int MSK_B = BY * BXM;
    static constexpr int SCL_B = BYE * BX * 4;
    static constexpr int OFF_R = 0;
    static constexpr int OFF_P = OFF_R + r128(VEC_B);
    static constexpr int OFF_D = OFF_P + r128(VEC_B);
    static constexpr int OFF_M = OFF_D + r128(DIN_B);
    static constexpr int OFF_S = OFF_M + r128(MSK_B);
    static constexpr int STAGE = OFF_S + r128(SCL_B);
    // one output tile [3][TY+1][TX]: row TY of each component is a scratch row
    // that lanes and rows owning no node write to, so the stores need no branch.
    // A tensor copy's shared-memory operand starts on a 128-byte boundary, so
    // the component stride is rounded up to 32 floats (448 already for 8 warps).
    static constexpr int OUT_CS = ((TY + 1) * TX + 31) / 32 * 32;  // component stride (floats)
    static constexpr int OUT_B = 3 * OUT_CS * 4;
    static constexpr int OFF_OUT = S * STAGE;  // q[2], p[2]
    static constexpr int OFF_XCH = OFF_OUT + 4 * r128(OUT_B);
    // row exchange between warps [2][W+1][3][32]: slot 0 stays zero, warp w
    // writes slot w+1 and reads slot w
    static constexpr int XCH_B = 2 * (W + 1) * 3 * 32 * 4;
    static constexpr int OFF_RED = OFF_XCH + XCH_B;
    static constexpr int OFF_BAR = OFF_RED + r128(2 * W * 8);
    static constexpr int OFF_FLAG = OFF_BAR + 8 * S;  // two ints: copy-wait failure, last-block flag
    static constexpr int SMEM = OFF_FLAG + 8;
    // dynamic shared memory requested: the kernel aligns its base to 1024 bytes
    static constexpr int SMEM_ALLOC = SMEM + 1024;
    // every tensor-copy destination and source in shared memory on a 128-byte boundary
    static_assert(OFF_P % 128 == 0 && OFF_D % 128 == 0 && OFF_M % 128 == 0 && OFF_S % 128 == 0 && STAGE % 128 == 0,
                  "stage buffers must start on 128-byte boundaries");
    static_assert(OFF_OUT % 128 == 0 && (OUT_CS * 4) % 128 == 0 && r128(OUT_B) % 128 == 0,
                  "output tiles and their components must start on 128-byte boundaries");
    static_assert(OFF_BAR % 8 == 0, "mbarriers are 8-byte aligned");
};

namespace tma {
__device__ __forceinline__ void load3(void *dst, const CUtensorMap *m, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(bulk::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(bulk::smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void load4(void *dst, const CUtensorMap *m, int x, int y, int z, int c, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(bulk::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(bulk::smem_addr(bar))
        : "memory");
}
// coordinates must be >= 0 (the copy engine clips the far side to the tensor)
__device__ __forceinline__ void store4(const CUtensorMap *m, int x, int y, int z, int c, const void *src) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
                     reinterpret_cast<uint64_t>(m)),
                 "r"(x), "r"(y), "r"(z), "r"(c), "r"(bulk::smem_addr(src))
                 : "memory");
}
__device__ __forceinline__ void commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the stores committed so far have finished reading shared memory
__device__ __forceinline__ void wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the stores committed so far are complete
__device__ __forceinline__ void wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void prefetch_map(const CUtensorMap *m) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}
}  // namespace tma

// p = D^-1 r + beta p_prev (p_prev / p the ping-pong pair chosen by the parity of
// S->it), q = mask(K p), partial p.q -> S->alpha (last block).  One tile per CTA.
// The body of one tile: tile `blk` of the problem's `nblk`, which take part in
// the p.q reduction together (ku3_kernel: one problem, a tile per CTA; the
// batched kernel: a tile of one problem of a batch per CTA).  T may live in the
// kernel's parameters or in global memory.
template <int W, int S>
__device__ __forceinline__ void ku3_tile(const Ku3Maps &T, const Ku3Args &A, const int blk, const int nblk) {
    using namespace k2;
    using Sh = Ku3Shape<W, S>;
    constexpr int TX = Sh::TX, BX = Sh::BX, BY = Sh::BY, BXM = Sh::BXM, TY = Sh::TY, OCS = Sh::OUT_CS;
    extern __shared__ __align__(1024) unsigned char ku3_smem[];
    // tensor-copy destinations want 128-byte alignment: align the base to 1024
    unsigned char *smem = ku3_smem + ((1024u - (bulk::smem_addr(ku3_smem) & 1023u)) & 1023u);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + Sh::OFF_BAR);
    float(*xch)[W + 1][3][32] = reinterpret_cast<float(*)[W + 1][3][32]>(smem + Sh::OFF_XCH);
    double *red = reinterpret_cast<double *>(smem + Sh::OFF_RED);
    int &s_fail = reinterpret_cast<int *>(smem + Sh::OFF_FLAG)[0];
    int &last_flag = reinterpret_cast<int *>(smem + Sh::OFF_FLAG)[1];

    if (A.S->done) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int b = blk;
    const int tx_ = b % A.tiles_x;
    b /= A.tiles_x;
    const int ty_ = b % A.tiles_y;
    const int tz_ = b / A.tiles_y;
    const int x0 = tx_ * TX, y0 = ty_ * TY, z0 = tz_ * A.tz;
    const int z1 = min(z0 + A.tz, A.nz + 1);
    const int np = z1 - z0 + 2;  // planes z0-1 .. z1 pass through the stages
    const bool odd = (A.S->it & 1) != 0;
    const float beta = (float)A.S->beta;
    const bool use_p = beta != 0.f;
    const CUtensorMap *map_pin = odd ? &T.pb : &T.pa;
    const CUtensorMap *map_pout = odd ? &T.past : &T.pbst;
    const int xm0 = (x0 - 1) & ~15;        // constraint-bit box origin (x0-1 rounded down to 16)
    const int col = lane + 3;              // this lane's column in a staged node / element row
    const int mcol = x0 - 1 - xm0 + lane;  // ... and in a staged constraint-bit row (< 47)
    const bool own_lane = lane >= 1 && lane <= TX;
    const unsigned tx_bytes = (unsigned)(Sh::VEC_B * (use_p ? 2 : 1) + Sh::DIN_B + Sh::MSK_B + Sh::SCL_B);
    // output offsets (floats, component 0) of this lane's q rows 0, 1 and p rows
    // 1, 2; the scratch row where the lane or the warp owns no node
    const int scratch = TY * TX + (lane & 15);
    const int oq0 = (own_lane && w >= 1) ? (2 * w - 1) * TX + lane - 1 : scratch;
    const int oq1 = own_lane ? (2 * w) * TX + lane - 1 : scratch;
    const int op2 = (own_lane && w < W - 1) ? (2 * w + 1) * TX + lane - 1 : scratch;
    const float f0 = (own_lane && w >= 1) ? 1.f : 0.f;  // p.q weights of rows 0 and 1
    const float f1 = own_lane ? 1.f : 0.f;

    // plane z0-1+j (and element layer z0-2+j) into stage j % S
    auto issue = [&](int j) {
        const int st = j % S, iz = z0 - 1 + j;
        unsigned char *sb = smem + st * Sh::STAGE;
        bulk::bar_expect(&bar[st], tx_bytes);
        tma::load4(sb + Sh::OFF_R, &T.r, x0 - 4, y0 - 1, iz, 0, &bar[st]);
        if (use_p) tma::load4(sb + Sh::OFF_P, map_pin, x0 - 4, y0 - 1, iz, 0, &bar[st]);
        tma::load3(sb + Sh::OFF_D, &T.d, x0 - 4, y0 - 1, iz, &bar[st]);
        tma::load3(sb + Sh::OFF_M, &T.m, xm0, y0 - 1, iz, &bar[st]);
        tma::load3(sb + Sh::OFF_S, &T.s, x0 - 4, y0 - 1, iz - 1, &bar[st]);
    };
    // output tile o (0/1) of q or p: [3][TY+1][TX]
    auto qout = [&](int o) { return reinterpret_cast<float *>(smem + Sh::OFF_OUT + o * Sh::r128(Sh::OUT_B)); };
    auto pout = [&](int o) { return reinterpret_cast<float *>(smem + Sh::OFF_OUT + (2 + o) * Sh::r128(Sh::OUT_B)); };
    // the tensor stores of the outputs written at iteration j (tile j & 1):
    // q of plane z0-2+j (an owned plane for j >= 2), p of plane z0-1+j (owned for j <= z1-z0)
    auto store_outputs = [&](int j) {
        bool any = false;
        if (j >= 2) {
#pragma unroll
            for (int c = 0; c < 3; ++c) tma::store4(&T.qst, x0, y0, z0 - 2 + j, c, qout(j & 1) + c * OCS);
            any = true;
        }
        if (j >= 1 && j <= z1 - z0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) tma::store4(map_pout, x0, y0, z0 - 1 + j, c, pout(j & 1) + c * OCS);
            any = true;
        }
        if (any) tma::commit();
    };
    // p on rows 2w .. 2w+2 of the plane in stage st, its constraint bits (rows 2w,
    // 2w+1) and the scales of the element layer below it
    auto read_plane = [&](int st, float (&v)[3][3], unsigned &mbits, float &sA, float &sB) {
        const unsigned char *sb = smem + st * Sh::STAGE;
        const float *Rs = reinterpret_cast<const float *>(sb + Sh::OFF_R);
        const float *Ps = reinterpret_cast<const float *>(sb + Sh::OFF_P);
        const float *Ds = reinterpret_cast<const float *>(sb + Sh::OFF_D);
        const float *Ss = reinterpret_cast<const float *>(sb + Sh::OFF_S);
        const uint8_t *Ms = sb + Sh::OFF_M;
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) {
            const int o = (2 * w + rr) * BX + col;
            const float d = Ds[o];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float rv = Rs[c * BY * BX + o];
                const float pv = use_p ? Ps[c * BY * BX + o] : 0.f;
                v[rr][c] = fmaf(beta, pv, d * rv);
            }
        }
        mbits = (unsigned)Ms[(2 * w) * BXM + mcol] | ((unsigned)Ms[(2 * w + 1) * BXM + mcol] << 8);
        sA = Ss[(2 * w) * BX + col];
        sB = Ss[(2 * w + 1) * BX + col];
    };
    auto faces = [&](const float (&v)[3][3], Face (&F)[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float n0 = __shfl_down_sync(0xffffffffu, v[0][c], 1);
            const float n1 = __shfl_down_sync(0xffffffffu, v[1][c], 1);
            const float n2 = __shfl_down_sync(0xffffffffu, v[2][c], 1);
            F[c] = face_modes(v[0][c], v[1][c], v[2][c], n0, n1, n2);
        }
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < S; ++k) bulk::bar_init(&bar[k], 1);
        bulk::bar_init_fence();
        s_fail = 0;
    }
    if (threadIdx.x < 2 * 3 * 32) xch[threadIdx.x / 96][0][(threadIdx.x / 32) % 3][threadIdx.x & 31] = 0.f;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int j = 0; j < S && j < np; ++j) issue(j);

    const float2 lam = splat(A.M.lam), mu = splat(A.M.mu), twomu = splat(2.f * A.M.mu), thrmu = splat(3.f * A.M.mu);
    Face FB[3], CT[3];
    float pcur[2][3];  // p of rows 0, 1 of the plane the current layer completes
    unsigned mcur;     // constraint bits of those rows (row 0: bits 0-2, row 1: bits 8-10)
    Acc<float> dot;
    {
        // plane z0-1: face modes only
        if (!bulk::bar_wait(&bar[0], 0u)) s_fail = 1;
        float v[3][3], sA, sB;
        read_plane(0, v, mcur, sA, sB);
        faces(v, FB);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            CT[c].ss = CT[c].sd = CT[c].ds = CT[c].dd = make_float2(0.f, 0.f);
            pcur[0][c] = v[0][c];
            pcur[1][c] = v[1][c];
        }
        __syncthreads();
        if (threadIdx.x == 0 && !s_fail && S < np) {
            bulk::proxy_fence();
            issue(S);
        }
    }
    int j = 1;
    if (!s_fail) {
        // two planes per trip: the carried face modes, p and constraint bits are
        // renamed instead of copied
#pragma unroll 2
        for (; j < np; ++j) {
            const int st = j % S;
            if (!bulk::bar_wait(&bar[st], (unsigned)(j / S) & 1u)) s_fail = 1;
            float v[3][3], sA, sB;
            unsigned mnew;
            read_plane(st, v, mnew, sA, sB);
            Face FT[3];
            faces(v, FT);
            float V[3][3];
            layer_math(FB, FT, CT, make_float2(sA, sB), A.M, lam, mu, twomu, thrmu, V);
            const int o = j & 1;
#pragma unroll
            for (int c = 0; c < 3; ++c) xch[o][w + 1][c][lane] = V[2][c];
            // the stores issued after the previous barrier have read their tile
            if (threadIdx.x == 0) tma::wait_read_all();
            __syncthreads();
            if (s_fail) break;
            if (threadIdx.x == 0) {
                if (j + S < np) {
                    bulk::proxy_fence();
                    issue(j + S);
                }
                store_outputs(j - 1);
            }
            // q of plane z0-2+j (rows 0, 1) and p of plane z0-1+j (rows 1, 2) into
            // tile o; rows or planes this tile does not own land in rows it never
            // stores
            float *Q = qout(o), *Pp = pout(o);
            float ds0 = 0.f, ds1 = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float v0 = V[0][c] + xch[o][w][c][lane];
                const float q0 = ((mcur >> c) & 1u) ? 0.f : v0;
                const float q1 = ((mcur >> (8 + c)) & 1u) ? 0.f : V[1][c];
                Q[c * OCS + oq0] = q0;
                Q[c * OCS + oq1] = q1;
                Pp[c * OCS + oq1] = v[1][c];
                Pp[c * OCS + op2] = v[2][c];
                ds0 = fmaf(pcur[0][c], q0, ds0);
                ds1 = fmaf(pcur[1][c], q1, ds1);
            }
            if (j >= 2) dot.add(fmaf(f0, ds0, f1 * ds1));
            bulk::proxy_fence();  // this thread's tile writes before the copy engine reads them
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                FB[c] = FT[c];
                pcur[0][c] = v[0][c];
                pcur[1][c] = v[1][c];
            }
            mcur = mnew;
        }
    }
    if (s_fail) {
        // a stage did not arrive in time: wait (bounded) for this CTA's copies
        // still in flight, then flag the launch
        if (threadIdx.x == 0) {
            for (int k = j; k < np && k < j + S; ++k) bulk::bar_wait(&bar[k % S], (unsigned)(k / S) & 1u);
            tma::wait_all();
            atomicExch(&A.S->kerr, 1);
        }
    } else {
        __syncthreads();
        if (threadIdx.x == 0) {
            store_outputs(np - 1);
            tma::wait_all();
        }
    }

    double dv[1] = {dot.value()};
    block_sum<1>(dv, red);
    if (threadIdx.x == 0) A.partial[2 * blk] = dv[0];
    if (!arrive_last_n(&A.S->cnt_ku, &last_flag, nblk)) return;
    double tot[1];
    reduce_partials<1>(A.partial, nblk, 2, tot, red);
    if (threadIdx.x == 0) {
        Scalars *Sc = A.S;
        const double pq = tot[0];
        Sc->pq = pq;
        if (!(pq > 0.0) || !isfinite(pq)) {
            Sc->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
            Sc->done = 1;
            Sc->alpha = 0.0;
        } else {
            Sc->alpha = Sc->rz / pq;
        }
        Sc->cnt_ku = 0;
    }
}

template <int W, int S>
__global__ void __launch_bounds__(32 * W, 2) ku3_kernel(const __grid_constant__ Ku3Maps T, const Ku3Args A) {
    ku3_tile<W, S>(T, A, blockIdx.x, gridDim.x);
}

// ---- batches: one tile of one problem per CTA ---------------------------------------
// A batch problem's tensor maps and arguments (a 64-byte aligned record per
// problem in global memory) and its tile count, the p.q reduction's participants.
struct Ku3BatchItem {
    Ku3Maps T;
    Ku3Args A;
    int ntiles;
};

// orders this thread's later tensor copies through map m after the map's bytes
// were written to global memory (by a copy from the host before the launch)
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *m) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(m))
                 : "memory");
}

// ---- the same product without a CTA-wide barrier per plane -----------------------
// ku3b_kernel computes exactly what ku3_kernel computes (same staging, same
// arithmetic, same order of every sum: p and q bitwise equal, p.q equal), but
// the warps of a CTA are no longer held in lockstep:
//   * stage reuse: each stage has a "full" barrier (the tensor copies' bytes) and
//     an "empty" one that every warp arrives on once it has read the plane;
//     thread 0 refills the stage of plane j-1 while its warp works on plane j,
//     so a warp may run one plane ahead of the slowest before it waits, and
//     S-1 planes are in flight;
//   * the one node row shared by warps w-1 and w goes through a two-slot
//     mailbox per warp pair with its own full/empty barriers, so a warp waits
//     only for its lower neighbour's row, never for the whole CTA;
//   * q and p of the owned nodes leave as coalesced per-lane global stores (rows
//     of 28 consecutive floats) instead of shared tiles and tensor stores, so no
//     warp waits for a tile to drain and no proxy fence is issued per plane.
// Every wait is bounded (one second) and warp-uniform (a wait counts as
// successful only if it succeeded in every lane); a warp whose wait runs out
// raises the CTA's failure flag and leaves the plane loop, the others leave at
// their next plane or when their own wait runs out, thread 0 waits (bounded)
// for its copies in flight, and the launch reports Scalars::kerr.
struct Ku3bArgs {
    Modal<float> M;
    double *partial;  // per-tile p.q
    Scalars *S;
    float *q, *pa, *pb;  // outputs: q = mask(K p); p into pa (odd iterations) or pb (even)
    int tiles_x, tiles_y, tz, nx, ny, nz;
    int sx, sxy, cs;  // node row, plane and component strides (the host checks 3 cs < 2^31)
};

template <int W, int S>
struct Ku3bShape {
    using B = Ku3Shape<W, S>;
    static constexpr int STAGE = B::STAGE;
    static constexpr int OFF_XCH = S * STAGE;
    // mailbox [W][2][3][32]: slot w (w >= 1) carries warp w-1's row 2 to warp w
    static constexpr int XCH_B = W * 2 * 3 * 32 * 4;
    static constexpr int OFF_RED = OFF_XCH + XCH_B;
    static constexpr int OFF_BAR = OFF_RED + B::r128(2 * W * 8);
    // full[S], empty[S], xfull[W][2], xempty[W][2]
    static constexpr int NBAR = 2 * S + 4 * W;
    static constexpr int OFF_FLAG = OFF_BAR + 8 * NBAR;
    static constexpr int SMEM = OFF_FLAG + 8;
    static constexpr int SMEM_ALLOC = SMEM + 1024;
};

// true if the wait succeeded in every lane of the (fully active) warp
__device__ __forceinline__ bool warp_wait(uint64_t *bar, unsigned parity) {
    return __all_sync(0xffffffffu, bulk::bar_wait(bar, parity)) != 0;
}

template <int W, int S>
__global__ void __launch_bounds__(32 * W, 2) ku3b_kernel(const __grid_constant__ Ku3Maps T, const Ku3bArgs A) {
    using namespace k2;
    using Sh0 = Ku3Shape<W, S>;
    using Sh = Ku3bShape<W, S>;
    constexpr int TX = Sh0::TX, BX = Sh0::BX, BY = Sh0::BY, BXM = Sh0::BXM;
    extern __shared__ __align__(1024) unsigned char ku3_smem[];
    unsigned char *smem = ku3_smem + ((1024u - (bulk::smem_addr(ku3_smem) & 1023u)) & 1023u);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + Sh::OFF_BAR);
    uint64_t *empty = full + S;
    uint64_t *xfull = empty + S;     // [W][2]
    uint64_t *xempty = xfull + 2 * W;  // [W][2]
    float(*xch)[2][3][32] = reinterpret_cast<float(*)[2][3][32]>(smem + Sh::OFF_XCH);
    double *red = reinterpret_cast<double *>(smem + Sh::OFF_RED);
    volatile int &s_fail = reinterpret_cast<int *>(smem + Sh::OFF_FLAG)[0];
    int &last_flag = reinterpret_cast<int *>(smem + Sh::OFF_FLAG)[1];

    if (A.S->done) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int b = blockIdx.x;
    const int tx_ = b % A.tiles_x;
    b /= A.tiles_x;
    const int ty_ = b % A.tiles_y;
    const int tz_ = b / A.tiles_y;
    const int x0 = tx_ * TX, y0 = ty_ * Sh0::TY, z0 = tz_ * A.tz;
    const int z1 = min(z0 + A.tz, A.nz + 1);
    const int np = z1 - z0 + 2;  // planes z0-1 .. z1 pass through the stages
    const bool odd = (A.S->it & 1) != 0;
    const float beta = (float)A.S->beta;
    const bool use_p = beta != 0.f;
    const CUtensorMap *map_pin = odd ? &T.pb : &T.pa;
    float *const pout = odd ? A.pa : A.pb;
    const int xm0 = (x0 - 1) & ~15;
    const int col = lane + 3;
    const int mcol = x0 - 1 - xm0 + lane;
    const bool own_lane = lane >= 1 && lane <= TX;
    const unsigned tx_bytes = (unsigned)(Sh0::VEC_B * (use_p ? 2 : 1) + Sh0::DIN_B + Sh0::MSK_B + Sh0::SCL_B);
    // stores: this lane's node column, rows y0+2w-1 (q), y0+2w (q, p), y0+2w+1 (p)
    const int gx = x0 - 1 + lane;
    const bool colok = own_lane && gx <= A.nx;
    const int ya = y0 + 2 * w - 1;
    const bool okq0 = colok && w >= 1 && ya <= A.ny;
    const bool okq1 = colok && ya + 1 <= A.ny;
    const bool okp2 = colok && w < W - 1 && ya + 2 <= A.ny;
    const int oq0 = ya * A.sx + gx, oq1 = oq0 + A.sx, op2 = oq1 + A.sx;
    const float f0 = (own_lane && w >= 1) ? 1.f : 0.f;
    const float f1 = own_lane ? 1.f : 0.f;

    auto issue = [&](int j, int st) {
        const int iz = z0 - 1 + j;
        unsigned char *sb = smem + st * Sh::STAGE;
        bulk::bar_expect(&full[st], tx_bytes);
        tma::load4(sb + Sh0::OFF_R, &T.r, x0 - 4, y0 - 1, iz, 0, &full[st]);
        if (use_p) tma::load4(sb + Sh0::OFF_P, map_pin, x0 - 4, y0 - 1, iz, 0, &full[st]);
        tma::load3(sb + Sh0::OFF_D, &T.d, x0 - 4, y0 - 1, iz, &full[st]);
        tma::load3(sb + Sh0::OFF_M, &T.m, xm0, y0 - 1, iz, &full[st]);
        tma::load3(sb + Sh0::OFF_S, &T.s, x0 - 4, y0 - 1, iz - 1, &full[st]);
    };
    auto read_plane = [&](int st, float (&v)[3][3], unsigned &mbits, float &sA, float &sB) {
        const unsigned char *sb = smem + st * Sh::STAGE;
        const float *Rs = reinterpret_cast<const float *>(sb + Sh0::OFF_R);
        const float *Ps = reinterpret_cast<const float *>(sb + Sh0::OFF_P);
        const float *Ds = reinterpret_cast<const float *>(sb + Sh0::OFF_D);
        const float *Ss = reinterpret_cast<const float *>(sb + Sh0::OFF_S);
        const uint8_t *Ms = sb + Sh0::OFF_M;
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) {
            const int o = (2 * w + rr) * BX + col;
            const float d = Ds[o];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float rv = Rs[c * BY * BX + o];
                const float pv = use_p ? Ps[c * BY * BX + o] : 0.f;
                v[rr][c] = fmaf(beta, pv, d * rv);
            }
        }
        mbits = (unsigned)Ms[(2 * w) * BXM + mcol] | ((unsigned)Ms[(2 * w + 1) * BXM + mcol] << 8);
        sA = Ss[(2 * w) * BX + col];
        sB = Ss[(2 * w + 1) * BX + col];
    };
    auto faces = [&](const float (&v)[3][3], Face (&F)[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float n0 = __shfl_down_sync(0xffffffffu, v[0][c], 1);
            const float n1 = __shfl_down_sync(0xffffffffu, v[1][c], 1);
            const float n2 = __shfl_down_sync(0xffffffffu, v[2][c], 1);
            F[c] = face_modes(v[0][c], v[1][c], v[2][c], n0, n1, n2);
        }
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < S; ++k) {
            bulk::bar_init(&full[k], 1);
            bulk::bar_init(&empty[k], W);
        }
        for (int k = 0; k < 2 * W; ++k) {
            bulk::bar_init(&xfull[k], 1);
            bulk::bar_init(&xempty[k], 1);
        }
        bulk::bar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    int issued = 0;  // planes whose copies thread 0 has issued
    if (threadIdx.x == 0)
        for (; issued < S && issued < np; ++issued) issue(issued, issued);

    const float2 lam = splat(A.M.lam), mu = splat(A.M.mu), twomu = splat(2.f * A.M.mu), thrmu = splat(3.f * A.M.mu);
    Face FB[3], CT[3];
    float pcur[2][3];
    unsigned mcur;
    Acc<float> dot;
    int j = 0;  // the plane being consumed (planes < j are read)
    bool ok = warp_wait(&full[0], 0u);
    if (ok) {
        j = 1;
        float v[3][3], sA, sB;
        read_plane(0, v, mcur, sA, sB);
        __syncwarp();
        if (lane == 0) bulk::bar_arrive(&empty[0]);
        faces(v, FB);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            CT[c].ss = CT[c].sd = CT[c].ds = CT[c].dd = make_float2(0.f, 0.f);
            pcur[0][c] = v[0][c];
            pcur[1][c] = v[1][c];
        }
    }
    // stage and phase of plane j
    int st = 1 % S, ph = S == 1 ? 1 : 0;
    if (ok) {
#pragma unroll 2
        for (; j < np; ++j) {
            if (s_fail || !warp_wait(&full[st], (unsigned)ph)) {
                ok = false;
                break;
            }
            float v[3][3], sA, sB;
            unsigned mnew;
            read_plane(st, v, mnew, sA, sB);
            __syncwarp();
            if (lane == 0) bulk::bar_arrive(&empty[st]);
            // refill the stage of plane j-1 (= issued - S) once every warp has read it
            if (threadIdx.x == 0 && issued < np) {
                const int k = issued - S;
                if (bulk::bar_wait(&empty[k % S], (unsigned)(k / S) & 1u)) {
                    bulk::proxy_fence();
                    issue(issued, k % S);
                    ++issued;
                } else {
                    s_fail = 1;
                }
            }
            Face FT[3];
            faces(v, FT);
            float V[3][3];
            layer_math(FB, FT, CT, make_float2(sA, sB), A.M, lam, mu, twomu, thrmu, V);
            // mailbox slot o, used for the u-th time: hand row 2 up, take the row below
            const int o = j & 1;
            const unsigned u = (unsigned)(j - 1) >> 1;
            if (w < W - 1) {
                if (u >= 1 && !warp_wait(&xempty[2 * (w + 1) + o], (u - 1) & 1u)) {
                    ok = false;
                    break;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) xch[w + 1][o][c][lane] = V[2][c];
                __syncwarp();
                if (lane == 0) bulk::bar_arrive(&xfull[2 * (w + 1) + o]);
            }
            float below[3] = {0.f, 0.f, 0.f};
            if (w > 0) {
                if (!warp_wait(&xfull[2 * w + o], u & 1u)) {
                    ok = false;
                    break;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) below[c] = xch[w][o][c][lane];
                __syncwarp();
                if (lane == 0) bulk::bar_arrive(&xempty[2 * w + o]);
            }
            // q of plane z0-2+j (rows ya, ya+1), p of plane z0-1+j (rows ya+1, ya+2)
            const bool qplane = j >= 2, pplane = j <= z1 - z0;
            const int zq = (z0 - 2 + j) * A.sxy, zp = zq + A.sxy;
            float ds0 = 0.f, ds1 = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float v0 = V[0][c] + below[c];
                const float q0 = ((mcur >> c) & 1u) ? 0.f : v0;
                const float q1 = ((mcur >> (8 + c)) & 1u) ? 0.f : V[1][c];
                float *qc = A.q + c * A.cs;
                float *pc = pout + c * A.cs;
                if (qplane && okq0) qc[zq + oq0] = q0;
                if (qplane && okq1) qc[zq + oq1] = q1;
                if (pplane && okq1) pc[zp + oq1] = v[1][c];
                if (pplane && okp2) pc[zp + op2] = v[2][c];
                ds0 = fmaf(pcur[0][c], q0, ds0);
                ds1 = fmaf(pcur[1][c], q1, ds1);
            }
            if (qplane) dot.add(fmaf(f0, ds0, f1 * ds1));
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                FB[c] = FT[c];
                pcur[0][c] = v[0][c];
                pcur[1][c] = v[1][c];
            }
            mcur = mnew;
            if (++st == S) {
                st = 0;
                ph ^= 1;
            }
        }
    }
    if (!ok) s_fail = 1;
    __syncthreads();
    if (s_fail) {
        // a wait ran out: wait (bounded) for this CTA's copies still in flight
        // (every plane issued and not yet consumed), then flag the launch
        if (threadIdx.x == 0) {
            for (int k = j; k < issued; ++k) bulk::bar_wait(&full[k % S], (unsigned)(k / S) & 1u);
            atomicExch(&A.S->kerr, 1);
        }
    }

    double dv[1] = {dot.value()};
    block_sum<1>(dv, red);
    if (threadIdx.x == 0) A.partial[2 * blockIdx.x] = dv[0];
    if (!arrive_last_n(&A.S->cnt_ku, &last_flag, gridDim.x)) return;
    double tot[1];
    reduce_partials<1>(A.partial, gridDim.x, 2, tot, red);
    if (threadIdx.x == 0) {
        Scalars *Sc = A.S;
        const double pq = tot[0];
        Sc->pq = pq;
        if (!(pq > 0.0) || !isfinite(pq)) {
            Sc->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
            Sc->done = 1;
            Sc->alpha = 0.0;
        } else {
            Sc->alpha = Sc->rz / pq;
        }
        Sc->cnt_ku = 0;
    }
}

}  // namespace amk
