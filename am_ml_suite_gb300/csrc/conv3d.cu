// conv3d.cu -- BF16 3x3x3 convolution kernels on the tensor cores
// (mma.sync m16n8k16, FP32 accumulate) and the tensor kernels of the learned
// preconditioner (conv3d.cuh).
//
// Forward / backward-data: implicit GEMM, M = voxels (128 per CTA), N = output
// channels (16, 32 or 64 per CTA), K = 27 taps x input channels.  A pipeline
// stage holds 4 (tap, 16-channel) units -- a 128 x 64 slab of tap-shifted voxel
// rows (zero-filled outside the grid) and the matching N x 64 weights -- staged
// with cp.async (double buffered) and read with ldmatrix, so each barrier pair
// covers 4 K steps of 16.  Backward-weight: GEMM over voxels, M = output channels, N = input
// channels (tiles of 16/32), K = voxels in chunks of 64, split over the warps of a
// CTA and over CTAs, finished with FP32 atomics.
#include <algorithm>

#include "conv3d.cuh"

namespace amk {

namespace {

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// 16-byte async copy; when !valid nothing is read and the destination is zeroed
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(smem)), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldsm_x4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// 16-byte chunk index inside a shared-memory row of `c` BF16 channels, XOR
// swizzled so that the 8 rows an ldmatrix reads fall on distinct banks
__device__ __forceinline__ int swz(int row, int chunk, int c) {
    return c == 16 ? (chunk ^ ((row >> 2) & 1)) : (chunk ^ ((row >> 1) & 3));
}

struct FwdArgs {
    const __nv_bfloat16 *x;
    int xcs, xco;
    const __nv_bfloat16 *w;
    __nv_bfloat16 *y;
    int ycs, yco;
    float *yf;
    int yfcs, yfco;
    int n, dz, dy, dx, cin, cout, relu;
    long long V;
};

constexpr int FM = 128;  // voxels per forward CTA
constexpr int KU = 4;    // (tap, 16-channel) units per pipeline stage: K = 64 per barrier pair

// 16-byte chunk index inside a 128-byte (KU x 16 BF16) shared-memory row, XOR
// swizzled by the row so the 8 rows an ldmatrix reads fall on distinct banks
__device__ __forceinline__ int swz8(int row, int chunk) { return chunk ^ (row & 7); }

template <int NT>
__global__ void __launch_bounds__(256) conv_fwd_kernel(FwdArgs A) {
    constexpr int WN = NT >= 32 ? 2 : 1;  // warps along N
    constexpr int WM = 8 / WN;            // warps along M
    constexpr int TM = FM / WM, TN = NT / WN;
    constexpr int MI = TM / 16, NI = TN / 8;
    __shared__ __align__(128) __nv_bfloat16 sA[2][FM * KU * 16];
    __shared__ __align__(128) __nv_bfloat16 sB[2][NT * KU * 16];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp % WM, wn = warp / WM;
    const long long v0 = (long long)blockIdx.x * FM;
    const int n0 = blockIdx.y * NT;
    const int Dx = A.dx, Dy = A.dy, Dz = A.dz;
    // the input row this thread stages: row tid/2, units (tid%2)*2 and +1
    const int arow = tid >> 1, apart = tid & 1;
    const long long av = v0 + arow;
    const bool arow_ok = av < A.V;
    int ax = 0, ay = 0, az = 0;
    {
        long long t = arow_ok ? av : 0;
        ax = (int)(t % Dx);
        t /= Dx;
        ay = (int)(t % Dy);
        t /= Dy;
        az = (int)(t % Dz);
    }
    const int ksteps = A.cin / 16;
    const int units = 27 * ksteps;  // (tap, 16-channel chunk) pairs, tap-major
    const int nstages = (units + KU - 1) / KU;
    auto load_stage = [&](int s, int buf) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int j = apart * 2 + q;  // unit of the stage
            const int u = s * KU + j;
            const int tap = u / ksteps, kc = u - tap * ksteps;
            const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
            const int sx = ax + dx, sy = ay + dy, sz = az + dz;
            const bool ok = u < units && arow_ok && sx >= 0 && sx < Dx && sy >= 0 && sy < Dy && sz >= 0 && sz < Dz;
            const long long sv = av + ((long long)dz * Dy + dy) * Dx + dx;
            const __nv_bfloat16 *src = ok ? A.x + sv * A.xcs + A.xco + kc * 16 : A.x;
            cp_async16(&sA[buf][arow * KU * 16 + swz8(arow, 2 * j) * 8], src, ok);
            cp_async16(&sA[buf][arow * KU * 16 + swz8(arow, 2 * j + 1) * 8], ok ? src + 8 : A.x, ok);
        }
        for (int t = tid; t < NT * KU * 2; t += 256) {
            const int brow = t / (KU * 2), c = t % (KU * 2);
            const int u = s * KU + c / 2;
            const bool ok = u < units;
            const int tap = ok ? u / ksteps : 0, kc = ok ? u - tap * ksteps : 0;
            const __nv_bfloat16 *wsrc =
                ok ? A.w + ((long long)tap * A.cout + n0 + brow) * A.cin + kc * 16 + (c & 1) * 8 : A.w;
            cp_async16(&sB[buf][brow * KU * 16 + swz8(brow, c) * 8], wsrc, ok);
        }
        cp_async_commit();
    };
    float acc[MI][NI][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
    load_stage(0, 0);
    const int mtx = lane >> 3, mrow = lane & 7;
    for (int s = 0; s < nstages; ++s) {
        const int buf = s & 1;
        if (s + 1 < nstages) {
            load_stage(s + 1, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < KU; ++j) {
            unsigned a[MI][4];
#pragma unroll
            for (int mi = 0; mi < MI; ++mi) {
                const int r = wm * TM + mi * 16 + mrow + ((mtx & 1) ? 8 : 0);
                const int c = 2 * j + (mtx >> 1);
                ldsm_x4(a[mi][0], a[mi][1], a[mi][2], a[mi][3], &sA[buf][r * KU * 16 + swz8(r, c) * 8]);
            }
            unsigned b[NI][2];
#pragma unroll
            for (int nj = 0; nj < NI; nj += 2) {
                const int r = wn * TN + nj * 8 + mrow + ((mtx >> 1) ? 8 : 0);
                const int c = 2 * j + (mtx & 1);
                ldsm_x4(b[nj][0], b[nj][1], b[nj + 1][0], b[nj + 1][1], &sB[buf][r * KU * 16 + swz8(r, c) * 8]);
            }
#pragma unroll
            for (int mi = 0; mi < MI; ++mi)
#pragma unroll
                for (int ni = 0; ni < NI; ++ni) mma_bf16(acc[mi][ni], a[mi], b[ni][0], b[ni][1]);
        }
        __syncthreads();
    }
    // epilogue: rows g and g+8 of each m16 tile, columns 2*tig, 2*tig+1 of each n8 tile
    const int g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int mi = 0; mi < MI; ++mi)
#pragma unroll
        for (int hr = 0; hr < 2; ++hr) {
            const long long v = v0 + wm * TM + mi * 16 + g + hr * 8;
            if (v >= A.V) continue;
#pragma unroll
            for (int ni = 0; ni < NI; ++ni) {
                const int c = n0 + wn * TN + ni * 8 + tig * 2;
                float f0 = acc[mi][ni][2 * hr], f1 = acc[mi][ni][2 * hr + 1];
                if (A.relu) {
                    f0 = fmaxf(f0, 0.f);
                    f1 = fmaxf(f1, 0.f);
                }
                if (A.y)
                    *reinterpret_cast<__nv_bfloat162 *>(A.y + v * A.ycs + A.yco + c) = __floats2bfloat162_rn(f0, f1);
                if (A.yf) *reinterpret_cast<float2 *>(A.yf + v * A.yfcs + A.yfco + c) = make_float2(f0, f1);
            }
        }
}

struct WgArgs {
    const __nv_bfloat16 *x;
    int xcs, xco;
    const __nv_bfloat16 *dy;
    int dycs, dyco;
    float *dw;
    int n, dz, dy_, dx, cin, cout;
    long long V;
    long long chunk;  // voxels per CTA (multiple of 64)
};

// dw[tap][co][ci] for one tap (blockIdx.y), one (MT x NT) tile (blockIdx.x) and
// one voxel range (blockIdx.z); 4 warps, each owning one 16-voxel K step of a
// 64-voxel stage.
template <int MT, int NT>
__global__ void __launch_bounds__(128) conv_wgrad_kernel(WgArgs A) {
    constexpr int MI = MT / 16, NI = NT / 8;
    __shared__ __align__(128) __nv_bfloat16 sD[2][64 * MT];
    __shared__ __align__(128) __nv_bfloat16 sX[2][64 * NT];
    __shared__ float red[4][MT * NT];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tiles_n = A.cin / NT;
    const int co0 = (blockIdx.x / tiles_n) * MT, ci0 = (blockIdx.x % tiles_n) * NT;
    const int tap = blockIdx.y;
    const int tdz = tap / 9 - 1, tdy = (tap / 3) % 3 - 1, tdx = tap % 3 - 1;
    const long long kb = (long long)blockIdx.z * A.chunk;
    const long long ke = min(A.V, kb + A.chunk);
    const int Dx = A.dx, Dy = A.dy_, Dz = A.dz;
    auto load_stage = [&](long long vb, int buf) {
        // dY rows: 64 voxels x MT/8 chunks; X rows: 64 voxels x NT/8 chunks
        constexpr int CD = MT / 8, CX = NT / 8;
        for (int t = tid; t < 64 * (CD + CX); t += 128) {
            if (t < 64 * CD) {
                const int r = t / CD, c = t % CD;
                const long long v = vb + r;
                const bool ok = v < ke;
                const __nv_bfloat16 *src = ok ? A.dy + v * A.dycs + A.dyco + co0 + c * 8 : A.dy;
                cp_async16(&sD[buf][r * MT + swz(r, c, MT) * 8], src, ok);
            } else {
                const int u = t - 64 * CD;
                const int r = u / CX, c = u % CX;
                const long long v = vb + r;
                bool ok = v < ke;
                long long sv = 0;
                if (ok) {
                    long long q = v;
                    const int x = (int)(q % Dx);
                    q /= Dx;
                    const int y = (int)(q % Dy);
                    q /= Dy;
                    const int z = (int)(q % Dz);
                    const int sx = x + tdx, sy = y + tdy, sz = z + tdz;
                    ok = sx >= 0 && sx < Dx && sy >= 0 && sy < Dy && sz >= 0 && sz < Dz;
                    sv = v + ((long long)tdz * Dy + tdy) * Dx + tdx;
                }
                const __nv_bfloat16 *src = ok ? A.x + sv * A.xcs + A.xco + ci0 + c * 8 : A.x;
                cp_async16(&sX[buf][r * NT + swz(r, c, NT) * 8], src, ok);
            }
        }
        cp_async_commit();
    };
    float acc[MI][NI][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
    const int mtx = lane >> 3, mrow = lane & 7;
    const int nst = (int)((ke - kb + 63) / 64);
    if (nst > 0) load_stage(kb, 0);
    for (int s = 0; s < nst; ++s) {
        const int buf = s & 1;
        if (s + 1 < nst) {
            load_stage(kb + (long long)(s + 1) * 64, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int k0 = warp * 16;  // this warp's 16 voxels of the stage
        unsigned a[MI][4];
#pragma unroll
        for (int mi = 0; mi < MI; ++mi) {
            // A[m = co][k = v] from sD[v][co] (transposed load)
            const int r = k0 + ((mtx >> 1) ? 8 : 0) + mrow;
            const int c = (mi * 16 + ((mtx & 1) ? 8 : 0)) / 8;
            ldsm_x4_t(a[mi][0], a[mi][1], a[mi][2], a[mi][3], &sD[buf][r * MT + swz(r, c, MT) * 8]);
        }
        unsigned b[NI][2];
#pragma unroll
        for (int nj = 0; nj < NI; nj += 2) {
            // B[k = v][n = ci] from sX[v][ci] (transposed load)
            const int r = k0 + ((mtx & 1) ? 8 : 0) + mrow;
            const int c = (nj * 8 + ((mtx >> 1) ? 8 : 0)) / 8;
            ldsm_x4_t(b[nj][0], b[nj][1], b[nj + 1][0], b[nj + 1][1], &sX[buf][r * NT + swz(r, c, NT) * 8]);
        }
#pragma unroll
        for (int mi = 0; mi < MI; ++mi)
#pragma unroll
            for (int ni = 0; ni < NI; ++ni) mma_bf16(acc[mi][ni], a[mi], b[ni][0], b[ni][1]);
        __syncthreads();
    }
    // sum the four warps' tiles, then one atomic per weight
    const int g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int mi = 0; mi < MI; ++mi)
#pragma unroll
        for (int ni = 0; ni < NI; ++ni)
#pragma unroll
            for (int hr = 0; hr < 2; ++hr) {
                const int m = mi * 16 + g + hr * 8, nn = ni * 8 + tig * 2;
                red[warp][m * NT + nn] = acc[mi][ni][2 * hr];
                red[warp][m * NT + nn + 1] = acc[mi][ni][2 * hr + 1];
            }
    __syncthreads();
    for (int i = tid; i < MT * NT; i += 128) {
        const float sum = red[0][i] + red[1][i] + red[2][i] + red[3][i];
        const int m = i / NT, nn = i % NT;
        if (sum != 0.f) atomicAdd(A.dw + ((long long)tap * A.cout + co0 + m) * A.cin + ci0 + nn, sum);
    }
}

__device__ __forceinline__ void unflatten(long long v, int Dx, int Dy, int Dz, int &n, int &z, int &y, int &x) {
    x = (int)(v % Dx);
    v /= Dx;
    y = (int)(v % Dy);
    v /= Dy;
    z = (int)(v % Dz);
    n = (int)(v / Dz);
}

__global__ void flip_transpose_kernel(const __nv_bfloat16 *w, int cout, int cin, __nv_bfloat16 *wt) {
    const long long total = 27LL * cout * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int tap = (int)(i / ((long long)cout * cin));
        const long long r = i - (long long)tap * cout * cin;
        const int co = (int)(r / cin), ci = (int)(r % cin);
        wt[((long long)(26 - tap) * cin + ci) * cout + co] = w[i];
    }
}

__global__ void relu_bwd_kernel(long long V, __nv_bfloat16 *g, int gcs, int gco, const __nv_bfloat16 *y, int ycs,
                                int yco, int c) {
    const long long total = V * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / c;
        const int ch = (int)(i % c);
        if (!(__bfloat162float(y[v * ycs + yco + ch]) > 0.f)) g[v * gcs + gco + ch] = __float2bfloat16(0.f);
    }
}

__global__ void avgpool_fwd_kernel(int N, int dz, int dy, int dx, const __nv_bfloat16 *in, int ics, int ico,
                                   __nv_bfloat16 *out, int ocs, int oco, int c) {
    const long long V = (long long)N * dz * dy * dx;
    const long long total = V * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / c;
        const int ch = (int)(i % c);
        int n, z, y, x;
        unflatten(v, dx, dy, dz, n, z, y, x);
        const int fx = 2 * dx, fy = 2 * dy, fz = 2 * dz;
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long fv = (((long long)n * fz + 2 * z + (k >> 2)) * fy + 2 * y + ((k >> 1) & 1)) * fx + 2 * x +
                                 (k & 1);
            s += __bfloat162float(in[fv * ics + ico + ch]);
        }
        out[v * ocs + oco + ch] = __float2bfloat16(0.125f * s);
    }
}

__global__ void avgpool_bwd_kernel(int N, int dz, int dy, int dx, const __nv_bfloat16 *dout, int ocs, int oco,
                                   __nv_bfloat16 *din, int ics, int ico, int c, int accumulate) {
    const long long V = (long long)N * dz * dy * dx;
    const long long total = V * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / c;
        const int ch = (int)(i % c);
        int n, z, y, x;
        unflatten(v, dx, dy, dz, n, z, y, x);
        const float gv = 0.125f * __bfloat162float(dout[v * ocs + oco + ch]);
        const int fx = 2 * dx, fy = 2 * dy, fz = 2 * dz;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long fv = (((long long)n * fz + 2 * z + (k >> 2)) * fy + 2 * y + ((k >> 1) & 1)) * fx + 2 * x +
                                 (k & 1);
            __nv_bfloat16 *d = din + fv * ics + ico + ch;
            *d = __float2bfloat16(accumulate ? __bfloat162float(*d) + gv : gv);
        }
    }
}

// one thread per (fine voxel, 8 channels): 16-byte copies (channel strides and
// offsets are multiples of 8)
__global__ void upsample_fwd_kernel(int N, int dz, int dy, int dx, const __nv_bfloat16 *in, int ics, int ico,
                                    __nv_bfloat16 *out, int ocs, int oco, int c) {
    const long long V = (long long)N * dz * dy * dx;
    const int g = c / 8;
    const long long total = V * g;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / g;
        const int ch = (int)(i - v * g) * 8;
        int n, z, y, x;
        unflatten(v, dx, dy, dz, n, z, y, x);
        const long long cv = (((long long)n * (dz / 2) + z / 2) * (dy / 2) + y / 2) * (dx / 2) + x / 2;
        *reinterpret_cast<uint4 *>(out + v * ocs + oco + ch) =
            *reinterpret_cast<const uint4 *>(in + cv * ics + ico + ch);
    }
}

__global__ void upsample_bwd_kernel(int N, int dz, int dy, int dx, const __nv_bfloat16 *dout, int ocs, int oco,
                                    __nv_bfloat16 *din, int ics, int ico, int c) {
    // dz, dy, dx: the fine grid; one thread per coarse value
    const int cz = dz / 2, cy = dy / 2, cx = dx / 2;
    const long long V = (long long)N * cz * cy * cx;
    const long long total = V * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / c;
        const int ch = (int)(i % c);
        int n, z, y, x;
        unflatten(v, cx, cy, cz, n, z, y, x);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long fv = (((long long)n * dz + 2 * z + (k >> 2)) * dy + 2 * y + ((k >> 1) & 1)) * dx + 2 * x +
                                 (k & 1);
            s += __bfloat162float(dout[fv * ocs + oco + ch]);
        }
        din[v * ics + ico + ch] = __float2bfloat16(s);
    }
}

__global__ void adam_kernel(float *w, float *m, float *v, const float *grad, __nv_bfloat16 *wb, long long n, float lr,
                            float b1, float b2, float eps, float c1, float c2, float gs) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gr = grad[i] * gs;
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        wb[i] = __float2bfloat16(wi);
    }
}

__global__ void f32_to_bf16_kernel(const float *a, __nv_bfloat16 *b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16(a[i]);
}
__global__ void zero_bf16_kernel(__nv_bfloat16 *a, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        a[i] = __float2bfloat16(0.f);
}

int ew_blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

bool aligned8(const TensorView &t) { return t.cstride % 8 == 0 && t.coff % 8 == 0; }

}  // namespace

static int g_conv_impl = 1;
void conv3d_set_impl(int impl) { g_conv_impl = impl ? 1 : 0; }
int conv3d_impl() { return g_conv_impl; }

cudaError_t conv3d_fwd(const Grid5 &g, TensorView x, int cin, const __nv_bfloat16 *w, int cout, TensorView y,
                       TensorView yf, int relu, cudaStream_t st) {
    if (g_conv_impl == 1) return conv3d_fwd_tc(g, x, cin, w, cout, y, yf, relu, st);
    if (cin % 16 || cout % 16 || !aligned8(x) || (y.p && (y.cstride % 2 || y.coff % 2)) ||
        (yf.p && (yf.cstride % 2 || yf.coff % 2)))
        return cudaErrorInvalidValue;
    FwdArgs a{};
    a.x = static_cast<const __nv_bfloat16 *>(x.p);
    a.xcs = x.cstride;
    a.xco = x.coff;
    a.w = w;
    a.y = static_cast<__nv_bfloat16 *>(y.p);
    a.ycs = y.cstride;
    a.yco = y.coff;
    a.yf = static_cast<float *>(yf.p);
    a.yfcs = yf.cstride;
    a.yfco = yf.coff;
    a.n = g.n;
    a.dz = g.dz;
    a.dy = g.dy;
    a.dx = g.dx;
    a.cin = cin;
    a.cout = cout;
    a.relu = relu;
    a.V = g.voxels();
    const unsigned gx = (unsigned)((a.V + FM - 1) / FM);
    if (cout % 64 == 0) {
        conv_fwd_kernel<64><<<dim3(gx, cout / 64), 256, 0, st>>>(a);
    } else if (cout % 32 == 0) {
        conv_fwd_kernel<32><<<dim3(gx, cout / 32), 256, 0, st>>>(a);
    } else {
        conv_fwd_kernel<16><<<dim3(gx, cout / 16), 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t conv3d_wgrad(const Grid5 &g, TensorView x, int cin, TensorView dy, int cout, float *dw, cudaStream_t st) {
    if (g_conv_impl == 1) return conv3d_wgrad_tc(g, x, cin, dy, cout, dw, st);
    if (cin % 16 || cout % 16 || !aligned8(x) || !aligned8(dy)) return cudaErrorInvalidValue;
    WgArgs a{};
    a.x = static_cast<const __nv_bfloat16 *>(x.p);
    a.xcs = x.cstride;
    a.xco = x.coff;
    a.dy = static_cast<const __nv_bfloat16 *>(dy.p);
    a.dycs = dy.cstride;
    a.dyco = dy.coff;
    a.dw = dw;
    a.n = g.n;
    a.dz = g.dz;
    a.dy_ = g.dy;
    a.dx = g.dx;
    a.cin = cin;
    a.cout = cout;
    a.V = g.voxels();
    const int MT = cout % 32 == 0 ? 32 : 16, NT = cin % 32 == 0 ? 32 : 16;
    const int tiles = (cout / MT) * (cin / NT);
    // enough CTAs for ~4 waves of 152 SMs, at least 64 voxels each
    long long split = std::max<long long>(1, (152LL * 8) / (27LL * tiles));
    long long chunk = (a.V + split - 1) / split;
    chunk = std::max<long long>(64, (chunk + 63) / 64 * 64);
    split = (a.V + chunk - 1) / chunk;
    a.chunk = chunk;
    const dim3 grid((unsigned)tiles, 27, (unsigned)split);
    if (MT == 32 && NT == 32) conv_wgrad_kernel<32, 32><<<grid, 128, 0, st>>>(a);
    else if (MT == 32) conv_wgrad_kernel<32, 16><<<grid, 128, 0, st>>>(a);
    else if (NT == 32) conv_wgrad_kernel<16, 32><<<grid, 128, 0, st>>>(a);
    else conv_wgrad_kernel<16, 16><<<grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t conv3d_flip_transpose(const __nv_bfloat16 *w, int cout, int cin, __nv_bfloat16 *wt, cudaStream_t st) {
    flip_transpose_kernel<<<ew_blocks(27LL * cout * cin), 256, 0, st>>>(w, cout, cin, wt);
    return cudaGetLastError();
}

cudaError_t relu_bwd(const Grid5 &g, TensorView grad, TensorView y, int c, cudaStream_t st) {
    relu_bwd_kernel<<<ew_blocks(g.voxels() * c), 256, 0, st>>>(g.voxels(), static_cast<__nv_bfloat16 *>(grad.p),
                                                                grad.cstride, grad.coff,
                                                                static_cast<const __nv_bfloat16 *>(y.p), y.cstride,
                                                                y.coff, c);
    return cudaGetLastError();
}

cudaError_t avgpool2_fwd(const Grid5 &g, TensorView in, TensorView out, int c, cudaStream_t st) {
    avgpool_fwd_kernel<<<ew_blocks(g.voxels() * c), 256, 0, st>>>(
        g.n, g.dz, g.dy, g.dx, static_cast<const __nv_bfloat16 *>(in.p), in.cstride, in.coff,
        static_cast<__nv_bfloat16 *>(out.p), out.cstride, out.coff, c);
    return cudaGetLastError();
}

cudaError_t avgpool2_bwd(const Grid5 &g, TensorView dout, TensorView din, int c, int accumulate, cudaStream_t st) {
    avgpool_bwd_kernel<<<ew_blocks(g.voxels() * c), 256, 0, st>>>(
        g.n, g.dz, g.dy, g.dx, static_cast<const __nv_bfloat16 *>(dout.p), dout.cstride, dout.coff,
        static_cast<__nv_bfloat16 *>(din.p), din.cstride, din.coff, c, accumulate);
    return cudaGetLastError();
}

cudaError_t upsample2_fwd(const Grid5 &g, TensorView in, TensorView out, int c, cudaStream_t st) {
    if (c % 8 || in.cstride % 8 || in.coff % 8 || out.cstride % 8 || out.coff % 8) return cudaErrorInvalidValue;
    upsample_fwd_kernel<<<ew_blocks(g.voxels() * (c / 8)), 256, 0, st>>>(
        g.n, g.dz, g.dy, g.dx, static_cast<const __nv_bfloat16 *>(in.p), in.cstride, in.coff,
        static_cast<__nv_bfloat16 *>(out.p), out.cstride, out.coff, c);
    return cudaGetLastError();
}

cudaError_t upsample2_bwd(const Grid5 &g, TensorView dout, TensorView din, int c, cudaStream_t st) {
    upsample_bwd_kernel<<<ew_blocks(g.voxels() / 8 * c), 256, 0, st>>>(
        g.n, g.dz, g.dy, g.dx, static_cast<const __nv_bfloat16 *>(dout.p), dout.cstride, dout.coff,
        static_cast<__nv_bfloat16 *>(din.p), din.cstride, din.coff, c);
    return cudaGetLastError();
}

cudaError_t adam_step(float *w, float *m, float *v, const float *grad, __nv_bfloat16 *wb, long long n, float lr,
                      float beta1, float beta2, float eps, int t, float grad_scale, cudaStream_t st) {
    const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
    adam_kernel<<<ew_blocks(n), 256, 0, st>>>(w, m, v, grad, wb, n, lr, beta1, beta2, eps, c1, c2, grad_scale);
    return cudaGetLastError();
}

cudaError_t f32_to_bf16(const float *a, __nv_bfloat16 *b, long long n, cudaStream_t st) {
    f32_to_bf16_kernel<<<ew_blocks(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

cudaError_t fill_zero_bf16(__nv_bfloat16 *a, long long n, cudaStream_t st) {
    zero_bf16_kernel<<<ew_blocks(n), 256, 0, st>>>(a, n);
    return cudaGetLastError();
}

}  // namespace amk
