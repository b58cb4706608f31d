// defl.cu -- rigid-body deflation of stiff passive inclusions (see defl.h).
//
// Deflation with rigid-body modes: Jonsthovel, van Gijzen, Vuik, Scarpas, "On the
// use of rigid body modes in the deflated preconditioned conjugate gradient
// method", SIAM J. Sci. Comput. 35 (2013).  Balancing form of the two-level
// preconditioner: Tang, Nabben, Vuik, Erlangga, "Comparison of two-level
// preconditioners derived from deflation, domain decomposition and multigrid
// methods", J. Sci. Comput. 39 (2009).
#include <algorithm>
#include <cmath>
#include <vector>

#include "defl.h"
#include "defl_space.h"

namespace amk {

namespace {

constexpr int DEFL_THREADS = 256;
constexpr int DEFL_CHUNK = 256;  // support entries per block of the dot products

inline int blocks_for(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + DEFL_THREADS - 1) / DEFL_THREADS, 152 * 8));
}

// z[t][k][u] = z0[t][k][u] on free DOFs, 0 on constrained / orphan ones
__global__ void defl_mask_kernel(long long nU, const long long *__restrict__ unode, const uint8_t *__restrict__ mask,
                                 const double *__restrict__ z0, double *__restrict__ z) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const unsigned m = mask[unode[u]];
#pragma unroll
        for (int t = 0; t < 6; ++t)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const long long i = (t * 3 + k) * nU + u;
                z[i] = ((m >> k) & 1u) ? 0.0 : z0[i];
            }
    }
}

// v[k cs + node(u)] = z[t][k][u]: mode t of every component, one full-grid vector
__global__ void defl_spread_kernel(long long nU, long long cs, const long long *__restrict__ unode,
                                   const double *__restrict__ z, int t, double *__restrict__ v) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const long long n = unode[u];
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k * cs + n] = z[(t * 3 + k) * nU + u];
    }
}

// kz[t][k][u] = (K v)[k cs + node(u)] on free DOFs, 0 on constrained ones
__global__ void defl_gather_kernel(long long nU, long long cs, const long long *__restrict__ unode,
                                   const uint8_t *__restrict__ mask, const double *__restrict__ w, int t,
                                   double *__restrict__ kz) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const long long n = unode[u];
        const unsigned m = mask[n];
#pragma unroll
        for (int k = 0; k < 3; ++k) kz[(t * 3 + k) * nU + u] = ((m >> k) & 1u) ? 0.0 : w[k * cs + n];
    }
}

// part[c][chunk][t] = sum over entries [chunk DEFL_CHUNK, +DEFL_CHUNK) of component
// c's support of V[t] . x; block (chunk, c), one warp per mode t (warps 6, 7 idle)
__global__ void __launch_bounds__(DEFL_THREADS)
    defl_dots_kernel(long long nU, long long cs, const long long *__restrict__ off,
                     const long long *__restrict__ unode, const double *__restrict__ V, const double *__restrict__ x,
                     int nchunk, double *__restrict__ part) {
    const int c = blockIdx.y, t = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (t >= 6) return;
    const long long b = off[c] + (long long)blockIdx.x * DEFL_CHUNK;
    const long long e = min(off[c + 1], b + DEFL_CHUNK);
    double acc = 0.0;
#pragma unroll 4
    for (long long u = b + lane; u < e; u += 32) {
        const long long n = unode[u];
#pragma unroll
        for (int k = 0; k < 3; ++k) acc = fma(V[(t * 3 + k) * nU + u], x[k * cs + n], acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) part[((long long)c * nchunk + blockIdx.x) * 6 + t] = acc;
}

// s = the chunk sums in chunk order; out = E^-1 s (block c: E_c^-1 s[6c .. 6c+5]),
// or base - E^-1 s when base is given
__global__ void defl_solve_kernel(int ncomp, int nchunk, const double *__restrict__ einv,
                                  const double *__restrict__ part, const double *__restrict__ base,
                                  double *__restrict__ out) {
    __shared__ double s[6 * DEFL_MAX_COMPONENTS];
    for (int i = threadIdx.x; i < 6 * ncomp; i += blockDim.x) {
        const int c = i / 6, t = i - 6 * c;
        double v = 0.0;
        for (int q = 0; q < nchunk; ++q) v += part[((long long)c * nchunk + q) * 6 + t];
        s[i] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 6 * ncomp; i += blockDim.x) {
        const int c = i / 6, t = i - 6 * c;
        double v = 0.0;
#pragma unroll
        for (int j = 0; j < 6; ++j) v = fma(einv[(c * 6 + t) * 6 + j], s[c * 6 + j], v);
        out[i] = base ? base[i] - v : v;
    }
}

// keep[k][u] = x[k cs + node(u)], then x[k cs + node(u)] -= sum_t KZ[t][k][u] a[...]
__global__ void defl_project_kernel(long long nU, long long cs, const long long *__restrict__ unode,
                                    const int *__restrict__ ucomp, const double *__restrict__ kz,
                                    const double *__restrict__ a, double *__restrict__ keep, double *__restrict__ x) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const long long n = unode[u];
        const double *cf = a + 6 * ucomp[u];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double v = 0.0;
#pragma unroll
            for (int t = 0; t < 6; ++t) v = fma(kz[(t * 3 + k) * nU + u], cf[t], v);
            const double xv = x[k * cs + n];
            keep[k * nU + u] = xv;
            x[k * cs + n] = xv - v;
        }
    }
}

// x[k cs + node(u)] = keep[k][u]: the entries defl_project_kernel changed, restored
__global__ void defl_restore_kernel(long long nU, long long cs, const long long *__restrict__ unode,
                                    const double *__restrict__ keep, double *__restrict__ x) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const long long n = unode[u];
#pragma unroll
        for (int k = 0; k < 3; ++k) x[k * cs + n] = keep[k * nU + u];
    }
}

// x[k cs + node(u)] += sign * sum_t V[t][k][u] coef[6 comp(u) + t]
__global__ void defl_scatter_kernel(long long nU, long long cs, const long long *__restrict__ unode,
                                    const int *__restrict__ ucomp, const double *__restrict__ V,
                                    const double *__restrict__ coef, double sign, double *__restrict__ x) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nU;
         u += (long long)gridDim.x * blockDim.x) {
        const long long n = unode[u];
        const double *cf = coef + 6 * ucomp[u];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double v = 0.0;
#pragma unroll
            for (int t = 0; t < 6; ++t) v = fma(V[(t * 3 + k) * nU + u], cf[t], v);
            x[k * cs + n] = fma(sign, v, x[k * cs + n]);
        }
    }
}

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T));
    return e;
}

// Cholesky inverse of the 6 x 6 SPD matrix a (row-major) in place; false if a
// pivot is not positive
bool inverse6(double *a) {
    double l[36] = {}, li[36] = {};
    for (int j = 0; j < 6; ++j) {
        double d = a[j * 6 + j];
        for (int k = 0; k < j; ++k) d -= l[j * 6 + k] * l[j * 6 + k];
        if (!(d > 0.0) || !std::isfinite(d)) return false;
        d = std::sqrt(d);
        l[j * 6 + j] = d;
        for (int i = j + 1; i < 6; ++i) {
            double s = a[i * 6 + j];
            for (int k = 0; k < j; ++k) s -= l[i * 6 + k] * l[j * 6 + k];
            l[i * 6 + j] = s / d;
        }
    }
    for (int j = 0; j < 6; ++j) {
        li[j * 6 + j] = 1.0 / l[j * 6 + j];
        for (int i = j + 1; i < 6; ++i) {
            double s = 0.0;
            for (int k = j; k < i; ++k) s -= l[i * 6 + k] * li[k * 6 + j];
            li[i * 6 + j] = s / l[i * 6 + i];
        }
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int k = std::max(i, j); k < 6; ++k) s += li[k * 6 + i] * li[k * 6 + j];
            a[i * 6 + j] = s;
        }
    return true;
}

}  // namespace

struct Defl {
    Layout L;
    int ncomp = 0;
    long long nU = 0;                 // support nodes of all components
    std::vector<long long> off_h;     // component c owns entries [off[c], off[c+1])
    long long *off = nullptr;
    long long *unode = nullptr;       // device node index of each entry
    int *ucomp = nullptr;             // component of each entry
    double *z0 = nullptr, *z = nullptr, *kz = nullptr;  // [6][3][nU]
    double *einv = nullptr;           // [ncomp][6][6]
    int nchunk = 1;                   // dot-product blocks per component (the largest support)
    double *part = nullptr;           // [ncomp][nchunk][6] chunk sums
    double *a = nullptr, *d = nullptr;  // [6 ncomp]
    double *keep = nullptr;           // [3][nU]: entries of r changed during an application
};

Defl *defl_create(const Layout &L, const uint8_t *solid, cudaError_t *err) {
    *err = cudaSuccess;
    DeflSpace sp;
    if (!defl_space(L.nx, L.ny, L.nz, L.sx, L.sxy, solid, sp)) return nullptr;
    const int ncomp = sp.ncomp;
    Defl *d = new Defl;
    d->L = L;
    d->ncomp = ncomp;
    d->off_h = sp.off;
    const long long nU = d->off_h.back();
    d->nU = nU;
    const std::vector<long long> &un = sp.unode;
    const std::vector<int> &uc = sp.ucomp;
    const std::vector<double> &z0 = sp.z0;
    const int nm = 6 * ncomp;
    long long longest = 1;
    for (int c = 0; c < ncomp; ++c) longest = std::max(longest, d->off_h[(size_t)c + 1] - d->off_h[(size_t)c]);
    d->nchunk = (int)((longest + DEFL_CHUNK - 1) / DEFL_CHUNK);
    cudaError_t e = dalloc(&d->off, (size_t)ncomp + 1);
    if (e == cudaSuccess) e = dalloc(&d->unode, (size_t)nU);
    if (e == cudaSuccess) e = dalloc(&d->ucomp, (size_t)nU);
    if (e == cudaSuccess) e = dalloc(&d->z0, (size_t)18 * nU);
    if (e == cudaSuccess) e = dalloc(&d->z, (size_t)18 * nU);
    if (e == cudaSuccess) e = dalloc(&d->kz, (size_t)18 * nU);
    if (e == cudaSuccess) e = dalloc(&d->einv, (size_t)36 * ncomp);
    if (e == cudaSuccess) e = dalloc(&d->part, (size_t)6 * ncomp * d->nchunk);
    if (e == cudaSuccess) e = dalloc(&d->a, (size_t)nm);
    if (e == cudaSuccess) e = dalloc(&d->d, (size_t)nm);
    if (e == cudaSuccess) e = dalloc(&d->keep, (size_t)3 * nU);
    if (e == cudaSuccess)
        e = cudaMemcpy(d->off, d->off_h.data(), sizeof(long long) * d->off_h.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d->unode, un.data(), sizeof(long long) * un.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d->ucomp, uc.data(), sizeof(int) * uc.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d->z0, z0.data(), sizeof(double) * z0.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        *err = e;
        defl_destroy(d);
        return nullptr;
    }
    return d;
}

void defl_destroy(Defl *d) {
    if (!d) return;
    for (void *p : {(void *)d->off, (void *)d->unode, (void *)d->ucomp, (void *)d->z0, (void *)d->z, (void *)d->kz,
                    (void *)d->einv, (void *)d->part, (void *)d->a, (void *)d->d, (void *)d->keep})
        if (p) cudaFree(p);
    delete d;
}

int defl_components(const Defl *d) { return d ? d->ncomp : 0; }

cudaError_t defl_setup(Defl *d, const KuLaunch &plan64, const Modal<double> &M64, const double *s64,
                       const uint8_t *mask, double *v, double *w, cudaStream_t st) {
    const Layout &L = d->L;
    const long long nU = d->nU;
    defl_mask_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, d->unode, mask, d->z0, d->z);
    count_launches(1);
    cudaError_t e = cudaGetLastError();
    for (int t = 0; t < 6 && e == cudaSuccess; ++t) {
        e = cudaMemsetAsync(v, 0, sizeof(double) * 3 * L.cs, st);
        if (e != cudaSuccess) break;
        defl_spread_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, L.cs, d->unode, d->z, t, v);
        count_launches(1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = ku_plain<double>(plan64, L, M64, s64, v, w, st);
        if (e != cudaSuccess) break;
        defl_gather_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, L.cs, d->unode, mask, w, t, d->kz);
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    std::vector<double> z((size_t)18 * nU), kz((size_t)18 * nU);
    e = cudaMemcpyAsync(z.data(), d->z, sizeof(double) * z.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(kz.data(), d->kz, sizeof(double) * kz.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    // E_c = Z_c^T K Z_c (symmetrised), inverted block by block; a block that is not
    // positive definite (a component with no free DOF) is left out (zero inverse)
    std::vector<double> einv((size_t)36 * d->ncomp, 0.0);
    for (int c = 0; c < d->ncomp; ++c) {
        double E[36] = {};
        for (long long u = d->off_h[(size_t)c]; u < d->off_h[(size_t)c + 1]; ++u)
            for (int t = 0; t < 6; ++t)
                for (int q = 0; q < 6; ++q)
                    for (int k = 0; k < 3; ++k)
                        E[t * 6 + q] += z[(size_t)(t * 3 + k) * nU + u] * kz[(size_t)(q * 3 + k) * nU + u];
        double S[36];
        for (int t = 0; t < 6; ++t)
            for (int q = 0; q < 6; ++q) S[t * 6 + q] = 0.5 * (E[t * 6 + q] + E[q * 6 + t]);
        if (inverse6(S)) std::copy(S, S + 36, einv.begin() + (size_t)36 * c);
    }
    e = cudaMemcpyAsync(d->einv, einv.data(), sizeof(double) * einv.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

cudaError_t defl_apply(Defl *d, Mg *mg, double *r, double *z, cudaStream_t st) {
    const Layout &L = d->L;
    const long long nU = d->nU;
    const dim3 gdot(d->nchunk, d->ncomp);
    // a = E^-1 Z^T r ; r <- P r = r - (K Z) a on the supports (old entries kept)
    defl_dots_kernel<<<gdot, DEFL_THREADS, 0, st>>>(nU, L.cs, d->off, d->unode, d->z, r, d->nchunk, d->part);
    defl_solve_kernel<<<1, 128, 0, st>>>(d->ncomp, d->nchunk, d->einv, d->part, nullptr, d->a);
    defl_project_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, L.cs, d->unode, d->ucomp, d->kz, d->a, d->keep,
                                                                  r);
    count_launches(3);
    cudaError_t e = cudaGetLastError();
    // y = M P r, then r restored exactly
    if (e == cudaSuccess) e = mg_apply(mg, r, z, st);
    defl_restore_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, L.cs, d->unode, d->keep, r);
    count_launches(1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // z = P^T y + Q r = y + Z (a - E^-1 (K Z)^T y)
    defl_dots_kernel<<<gdot, DEFL_THREADS, 0, st>>>(nU, L.cs, d->off, d->unode, d->kz, z, d->nchunk, d->part);
    defl_solve_kernel<<<1, 128, 0, st>>>(d->ncomp, d->nchunk, d->einv, d->part, d->a, d->d);
    defl_scatter_kernel<<<blocks_for(nU), DEFL_THREADS, 0, st>>>(nU, L.cs, d->unode, d->ucomp, d->z, d->d, 1.0, z);
    count_launches(3);
    return cudaGetLastError();
}

}  // namespace amk
