// mg.cu -- geometric multigrid V-cycle preconditioner (see mg.h).
#include <cmath>
#include <vector>

#include "host_util.h"
#include "kernels.cuh"
#include "mg.h"

namespace amk {

namespace {

constexpr float MG_OMEGA = 0.6f;  // damped-Jacobi weight
constexpr int MG_NU = 2;          // sweeps before and after the coarse correction

inline int blocks_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8)); }

// coarse element scale = mean of the 8 children (FP64 and its FP32 copy)
__global__ void mg_coarse_scales_kernel(Layout Lf, Layout Lc, const double *__restrict__ sf, double *__restrict__ sc,
                                        float *__restrict__ sc32) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Lc.nel;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e / Lc.nx;
        const int ex = (int)(e - row * Lc.nx);
        const int ez = (int)(row / Lc.ny), ey = (int)(row - (long long)ez * Lc.ny);
        double acc = 0.0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) acc += sf[elem_index(Lf, 2 * ex + dx, 2 * ey + dy, 2 * ez + dz)];
        sc[e] = 0.125 * acc;
        sc32[e] = (float)(0.125 * acc);
    }
}

// coarse fixed bits: those of the coincident fine node
__global__ void mg_coarse_fixed_kernel(Layout Lf, Layout Lc, const uint8_t *__restrict__ ff, uint8_t *__restrict__ fc) {
    const long long nn = Lc.sxy * (Lc.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / Lc.sxy);
        const long long rem = n - (long long)iz * Lc.sxy;
        const int iy = (int)(rem / Lc.sx), ix = (int)(rem - (long long)iy * Lc.sx);
        fc[n] = (ix <= Lc.nx && ff) ? ff[node_index(Lf, 2 * ix, 2 * iy, 2 * iz)] : 0;
    }
}

// x = omega D^-1 b on the free DOFs (the first sweep from zero)
__global__ void mg_jacobi0_kernel(Layout L, const float *__restrict__ b, const float *__restrict__ dinv,
                                  const uint8_t *__restrict__ mask, float *__restrict__ x, float omega) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const unsigned m = mask[n];
        const float d = omega * dinv[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[n + c * L.cs] = ((m >> c) & 1u) ? 0.f : d * b[n + c * L.cs];
    }
}
// x += omega D^-1 (b - t) on the free DOFs (t = K x)
__global__ void mg_jacobi_kernel(Layout L, const float *__restrict__ b, const float *__restrict__ t,
                                 const float *__restrict__ dinv, const uint8_t *__restrict__ mask,
                                 float *__restrict__ x, float omega) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.cs;
         n += (long long)gridDim.x * blockDim.x) {
        const unsigned m = mask[n];
        const float d = omega * dinv[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long i = n + c * L.cs;
            if (!((m >> c) & 1u)) x[i] = fmaf(d, b[i] - t[i], x[i]);
        }
    }
}

// bc = R (bf - tf): full weighting of the fine residual (free DOFs) onto the
// coarse nodes, weights 1, 1/2, 1/4, 1/8 by the fine node's offset
__global__ void mg_restrict_kernel(Layout Lf, Layout Lc, const float *__restrict__ bf, const float *__restrict__ tf,
                                   const uint8_t *__restrict__ maskf, const uint8_t *__restrict__ maskc,
                                   float *__restrict__ bc) {
    const long long nn = Lc.sxy * (Lc.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / Lc.sxy);
        const long long rem = n - (long long)iz * Lc.sxy;
        const int iy = (int)(rem / Lc.sx), ix = (int)(rem - (long long)iy * Lc.sx);
        if (ix > Lc.nx) continue;
        float acc[3] = {0.f, 0.f, 0.f};
        for (int dz = -1; dz <= 1; ++dz) {
            const int fz = 2 * iz + dz;
            if (fz < 0 || fz > Lf.nz) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int fy = 2 * iy + dy;
                if (fy < 0 || fy > Lf.ny) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    const int fx = 2 * ix + dx;
                    if (fx < 0 || fx > Lf.nx) continue;
                    const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
                    const long long f = node_index(Lf, fx, fy, fz);
                    const unsigned m = maskf[f];
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        if (!((m >> c) & 1u)) acc[c] = fmaf(w, bf[f + c * Lf.cs] - tf[f + c * Lf.cs], acc[c]);
                }
            }
        }
        const unsigned m = maskc[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) bc[n + c * Lc.cs] = ((m >> c) & 1u) ? 0.f : acc[c];
    }
}

// xf += P xc on the free fine DOFs (trilinear interpolation)
__global__ void mg_prolong_kernel(Layout Lc, Layout Lf, const float *__restrict__ xc, const uint8_t *__restrict__ maskf,
                                  float *__restrict__ xf) {
    const long long nn = Lf.sxy * (Lf.nz + 1);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
         n += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(n / Lf.sxy);
        const long long rem = n - (long long)iz * Lf.sxy;
        const int iy = (int)(rem / Lf.sx), ix = (int)(rem - (long long)iy * Lf.sx);
        if (ix > Lf.nx) continue;
        const unsigned m = maskf[n];
        if (m == 7u) continue;
        // parents along each axis: an even fine index has one (weight 1), an odd one two (1/2 each)
        const int x0 = ix >> 1, x1 = (ix + 1) >> 1, y0 = iy >> 1, y1 = (iy + 1) >> 1, z0 = iz >> 1, z1 = (iz + 1) >> 1;
        const float wx = (ix & 1) ? 0.5f : 1.f, wy = (iy & 1) ? 0.5f : 1.f, wz = (iz & 1) ? 0.5f : 1.f;
        float acc[3] = {0.f, 0.f, 0.f};
        for (int kz = 0; kz <= (iz & 1); ++kz)
            for (int ky = 0; ky <= (iy & 1); ++ky)
                for (int kx = 0; kx <= (ix & 1); ++kx) {
                    const long long cidx = node_index(Lc, kx ? x1 : x0, ky ? y1 : y0, kz ? z1 : z0);
                    const float w = wx * wy * wz;
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[c] = fmaf(w, xc[cidx + c * Lc.cs], acc[c]);
                }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (!((m >> c) & 1u)) xf[n + c * Lf.cs] += acc[c];
    }
}

// x = A^-1 b on the coarsest grid; A^-1 symmetric, n x n, dense DOF order
// 3 * ((iz (ny+1) + iy)(nx+1) + ix) + c.  One warp per row of A^-1 (coalesced
// reads of the row, a shuffle reduction), every block holding b in shared memory.
__global__ void mg_dense_kernel(Layout L, int n, const float *__restrict__ ainv, const float *__restrict__ b,
                                float *__restrict__ x) {
    extern __shared__ float bd[];
    const int nx1 = L.nx + 1, ny1 = L.ny + 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = i % 3, nd = i / 3;
        const int ix = nd % nx1, iy = (nd / nx1) % ny1, iz = nd / (nx1 * ny1);
        bd[i] = b[node_index(L, ix, iy, iz) + c * L.cs];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = blockIdx.x * nw + (threadIdx.x >> 5); i < n; i += gridDim.x * nw) {
        const float *row = ainv + (long long)i * n;
        float acc = 0.f;
        for (int j = lane; j < n; j += 32) acc = fmaf(row[j], bd[j], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const int c = i % 3, nd = i / 3;
            const int ix = nd % nx1, iy = (nd / nx1) % ny1, iz = nd / (nx1 * ny1);
            x[node_index(L, ix, iy, iz) + c * L.cs] = acc;
        }
    }
}

__global__ void mg_to_float_kernel(const double *__restrict__ a, float *__restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void mg_to_double_kernel(const float *__restrict__ a, double *__restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T));
    return e;
}

// In-place Cholesky of the SPD matrix a (n x n, row-major, lower triangle used)
// and the inverse from it; false if a pivot is not positive.
bool spd_inverse(std::vector<double> &a, int n) {
    for (int j = 0; j < n; ++j) {
        double d = a[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= a[(size_t)j * n + k] * a[(size_t)j * n + k];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        a[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = a[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) s -= a[(size_t)i * n + k] * a[(size_t)j * n + k];
            a[(size_t)i * n + j] = s / d;
        }
    }
    // inverse of L (lower), then A^-1 = L^-T L^-1
    std::vector<double> li((size_t)n * n, 0.0);
    for (int j = 0; j < n; ++j) {
        li[(size_t)j * n + j] = 1.0 / a[(size_t)j * n + j];
        for (int i = j + 1; i < n; ++i) {
            double s = 0.0;
            for (int k = j; k < i; ++k) s -= a[(size_t)i * n + k] * li[(size_t)k * n + j];
            li[(size_t)i * n + j] = s / a[(size_t)i * n + i];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = 0.0;
            for (int k = i; k < n; ++k) s += li[(size_t)k * n + i] * li[(size_t)k * n + j];
            a[(size_t)i * n + j] = s;
            a[(size_t)j * n + i] = s;
        }
    return true;
}

}  // namespace

struct MgLevel {
    Layout L;
    KuLaunch plan;
    Modal<double> M64;
    Modal<float> M32;
    double ke00 = 0.0;
    // operator (level 0 borrows the problem's arrays)
    const float *s32 = nullptr, *dinv = nullptr;
    const uint8_t *mask = nullptr;
    const double *s64 = nullptr;
    double *s64_own = nullptr;
    float *s32_own = nullptr, *dinv_own = nullptr;
    uint8_t *mask_own = nullptr, *fixed_own = nullptr;
    // vectors [3][cs]: right-hand side, iterate, K iterate
    float *b = nullptr, *x = nullptr, *t = nullptr;
};

struct Mg {
    std::vector<MgLevel> lv;
    int n_dense = 0;
    float *ainv = nullptr;
};

int mg_num_levels(const Mg *m) { return m ? (int)m->lv.size() : 0; }

void mg_destroy(Mg *m) {
    if (!m) return;
    for (auto &l : m->lv) {
        cudaFree(l.s64_own);
        cudaFree(l.s32_own);
        cudaFree(l.dinv_own);
        cudaFree(l.mask_own);
        cudaFree(l.fixed_own);
        cudaFree(l.b);
        cudaFree(l.x);
        cudaFree(l.t);
    }
    cudaFree(m->ainv);
    delete m;
}

Mg *mg_create(const Layout &L0, double E0, double nu, double h, cudaError_t *err) {
    *err = cudaSuccess;
    std::vector<Layout> Ls{L0};
    auto dofs = [](const Layout &L) { return 3LL * (L.nx + 1) * (L.ny + 1) * (L.nz + 1); };
    while (dofs(Ls.back()) > MG_COARSE_DOFS && Ls.back().nx % 2 == 0 && Ls.back().ny % 2 == 0 &&
           Ls.back().nz % 2 == 0)
        Ls.push_back(make_layout(Ls.back().nx / 2, Ls.back().ny / 2, Ls.back().nz / 2));
    if (Ls.size() < 2 || dofs(Ls.back()) > MG_DENSE_MAX) return nullptr;
    Mg *m = new Mg;
    m->lv.resize(Ls.size());
    double hl = h;
    cudaError_t e = cudaSuccess;
    for (size_t l = 0; l < Ls.size() && e == cudaSuccess; ++l, hl *= 2.0) {
        MgLevel &v = m->lv[l];
        v.L = Ls[l];
        v.plan = ku_plan(v.L, false, 0);
        v.M64 = modal_constants(E0, nu, hl);
        v.M32 = modal_float(v.M64);
        v.ke00 = element_stiffness_entry(v.M64, 0, 0);
        const size_t nv = 3 * (size_t)v.L.cs;
        if (e == cudaSuccess) e = dalloc(&v.b, nv);
        if (e == cudaSuccess) e = dalloc(&v.x, nv);
        if (e == cudaSuccess) e = dalloc(&v.t, nv);
        if (l > 0) {
            if (e == cudaSuccess) e = dalloc(&v.s64_own, (size_t)v.L.nel);
            if (e == cudaSuccess) e = dalloc(&v.s32_own, (size_t)v.L.nel);
            if (e == cudaSuccess) e = dalloc(&v.dinv_own, (size_t)v.L.cs);
            if (e == cudaSuccess) e = dalloc(&v.mask_own, (size_t)v.L.cs);
            if (e == cudaSuccess) e = dalloc(&v.fixed_own, (size_t)v.L.cs);
            v.s64 = v.s64_own;
            v.s32 = v.s32_own;
            v.dinv = v.dinv_own;
            v.mask = v.mask_own;
        }
    }
    m->n_dense = (int)dofs(Ls.back());
    if (e == cudaSuccess) e = dalloc(&m->ainv, (size_t)m->n_dense * m->n_dense);
    if (e != cudaSuccess) {
        *err = e;
        mg_destroy(m);
        return nullptr;
    }
    return m;
}

cudaError_t mg_setup(Mg *m, const double *s64, const float *s32, const float *dinv32, const uint8_t *mask,
                     const uint8_t *fixed_bits, cudaStream_t st) {
    MgLevel &f = m->lv[0];
    f.s64 = s64;
    f.s32 = s32;
    f.dinv = dinv32;
    f.mask = mask;
    cudaError_t e = cudaSuccess;
    const uint8_t *fixed_prev = fixed_bits;
    for (size_t l = 1; l < m->lv.size() && e == cudaSuccess; ++l) {
        MgLevel &p = m->lv[l - 1], &c = m->lv[l];
        mg_coarse_scales_kernel<<<blocks_for(c.L.nel), 256, 0, st>>>(p.L, c.L, p.s64, c.s64_own, c.s32_own);
        mg_coarse_fixed_kernel<<<blocks_for(c.L.cs), 256, 0, st>>>(p.L, c.L, fixed_prev, c.fixed_own);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = diag_mask(c.L, c.s64_own, c.ke00, c.fixed_own, nullptr, c.dinv_own, c.mask_own, st);
        count_launches(2);
        fixed_prev = c.fixed_own;
    }
    if (e != cudaSuccess) return e;
    // coarsest level: dense K on the free DOFs (identity rows on the others), inverted on the host
    const MgLevel &c = m->lv.back();
    const Layout L = c.L;
    std::vector<double> sc((size_t)L.nel);
    std::vector<uint8_t> mk((size_t)L.cs);
    e = cudaMemcpyAsync(sc.data(), c.s64, sizeof(double) * L.nel, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mk.data(), c.mask, L.cs, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    const int n = m->n_dense, nx1 = L.nx + 1, ny1 = L.ny + 1;
    double ke[24][24];
    for (int r = 0; r < 24; ++r)
        for (int q = 0; q < 24; ++q) ke[r][q] = element_stiffness_entry(c.M64, r, q);
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    std::vector<double> a((size_t)n * n, 0.0);
    auto dof = [&](int ix, int iy, int iz, int cc) { return 3 * ((iz * ny1 + iy) * nx1 + ix) + cc; };
    for (int ez = 0; ez < L.nz; ++ez)
        for (int ey = 0; ey < L.ny; ++ey)
            for (int ex = 0; ex < L.nx; ++ex) {
                const double s = sc[(size_t)elem_index(L, ex, ey, ez)];
                if (s == 0.0) continue;
                for (int na = 0; na < 8; ++na)
                    for (int ca = 0; ca < 3; ++ca) {
                        const int i = dof(ex + off[na][0], ey + off[na][1], ez + off[na][2], ca);
                        for (int nb = 0; nb < 8; ++nb)
                            for (int cb = 0; cb < 3; ++cb) {
                                const int j = dof(ex + off[nb][0], ey + off[nb][1], ez + off[nb][2], cb);
                                a[(size_t)i * n + j] += s * ke[3 * na + ca][3 * nb + cb];
                            }
                    }
            }
    for (int iz = 0; iz <= L.nz; ++iz)
        for (int iy = 0; iy <= L.ny; ++iy)
            for (int ix = 0; ix <= L.nx; ++ix) {
                const unsigned bits = mk[(size_t)node_index(L, ix, iy, iz)];
                for (int cc = 0; cc < 3; ++cc) {
                    if (!((bits >> cc) & 1u)) continue;
                    const int i = dof(ix, iy, iz, cc);
                    for (int j = 0; j < n; ++j) a[(size_t)i * n + j] = a[(size_t)j * n + i] = 0.0;
                    a[(size_t)i * n + i] = 1.0;
                }
            }
    if (!spd_inverse(a, n)) return cudaErrorInvalidValue;
    std::vector<float> af((size_t)n * n);
    for (size_t i = 0; i < af.size(); ++i) af[i] = (float)a[i];
    e = cudaMemcpyAsync(m->ainv, af.data(), sizeof(float) * af.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

namespace {
cudaError_t vcycle(Mg *m, size_t l, cudaStream_t st) {
    MgLevel &v = m->lv[l];
    cudaError_t e;
    if (l + 1 == m->lv.size()) {
        const int n = m->n_dense;
        mg_dense_kernel<<<(n + 7) / 8, 256, sizeof(float) * n, st>>>(v.L, n, m->ainv, v.b, v.x);
        count_launches(1);
        return cudaGetLastError();
    }
    const int nb = blocks_for(v.L.cs);
    // pre-smoothing: the first sweep from zero, then MG_NU - 1 more
    mg_jacobi0_kernel<<<nb, 256, 0, st>>>(v.L, v.b, v.dinv, v.mask, v.x, MG_OMEGA);
    count_launches(1);
    for (int s = 1; s < MG_NU; ++s) {
        if ((e = ku_plain<float>(v.plan, v.L, v.M32, v.s32, v.x, v.t, st)) != cudaSuccess) return e;
        mg_jacobi_kernel<<<nb, 256, 0, st>>>(v.L, v.b, v.t, v.dinv, v.mask, v.x, MG_OMEGA);
        count_launches(1);
    }
    // coarse correction
    MgLevel &c = m->lv[l + 1];
    if ((e = ku_plain<float>(v.plan, v.L, v.M32, v.s32, v.x, v.t, st)) != cudaSuccess) return e;
    mg_restrict_kernel<<<blocks_for(c.L.cs), 256, 0, st>>>(v.L, c.L, v.b, v.t, v.mask, c.mask, c.b);
    count_launches(1);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = vcycle(m, l + 1, st)) != cudaSuccess) return e;
    mg_prolong_kernel<<<blocks_for(v.L.cs), 256, 0, st>>>(c.L, v.L, c.x, v.mask, v.x);
    count_launches(1);
    // post-smoothing
    for (int s = 0; s < MG_NU; ++s) {
        if ((e = ku_plain<float>(v.plan, v.L, v.M32, v.s32, v.x, v.t, st)) != cudaSuccess) return e;
        mg_jacobi_kernel<<<nb, 256, 0, st>>>(v.L, v.b, v.t, v.dinv, v.mask, v.x, MG_OMEGA);
        count_launches(1);
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t mg_apply(Mg *m, const double *r, double *z, cudaStream_t st) {
    MgLevel &f = m->lv[0];
    const long long n = 3 * f.L.cs;
    mg_to_float_kernel<<<blocks_for(n), 256, 0, st>>>(r, f.b, n);
    count_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = vcycle(m, 0, st);
    if (e != cudaSuccess) return e;
    mg_to_double_kernel<<<blocks_for(n), 256, 0, st>>>(f.x, z, n);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace amk
