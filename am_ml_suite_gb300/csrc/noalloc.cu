// noalloc.cu -- FP64 residual r = f - K(s) u on caller-owned device buffers,
// without any device allocation.
//
// Callers that must not allocate device memory after start-up -- code running
// inside another framework's fixed memory pool, real-time or certified control
// loops that forbid allocation in their cycle, or plugins whose host owns every
// buffer -- cannot use the handle-based API (am_problem_create allocates its
// workspace).  This entry point takes every input and output from the caller
// and keeps its only scratch -- the per-tile partial sums of |r|^2 and the
// solver-scalar block the last tile writes -- in file-scope __device__ arrays of
// fixed size, present on every device that loads the library until exit.
#include <cuda_runtime.h>

#include <climits>
#include <mutex>
#include <string>

#include "../../include/am_gpu.h"
#include "kernels.cuh"
#include "ku.cuh"

using namespace amk;

namespace {

// Largest number of K*u tiles one call may use: a tile covers 32 x 4 node columns
// of the full z extent, so (nx+1)/32 * (ny+1)/4 (rounded up) must not exceed it.
constexpr int kNoAllocMaxTiles = 32768;
// The FP64 residual tile (32 x 4 node columns) must run without the opt-in to
// more than 48 KB of dynamic shared memory: that opt-in is made when a problem
// is created, and this entry point may be the first call into the library.
static_assert(KuShape<32, 4>::smem_bytes<double>() <= 48 * 1024,
              "the allocation-free residual relies on the default dynamic shared-memory limit");
static __device__ __align__(256) double g_noalloc_partial[2 * kNoAllocMaxTiles];  // 512 KB
static __device__ __align__(256) Scalars g_noalloc_scalars;

struct DeviceScratch {
    bool ready = false;
    double *partial = nullptr;
    Scalars *scalars = nullptr;
};
constexpr int kMaxDevices = 64;
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

am_status noalloc_fail(am_status s, const std::string &m) {
    set_last_error(m.c_str());  // read back with am_last_error()
    return s;
}

// Device addresses of the scratch arrays for the current device.  In host code
// the array names are host-side stand-ins, not device addresses, so the
// addresses are looked up once per device with that device current.
am_status scratch_for_current_device(DeviceScratch **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(AM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(AM_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    DeviceScratch &d = g_scratch[dev];
    if (!d.ready) {
        void *p = nullptr, *s = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partial);
        if (e != cudaSuccess)
            return noalloc_fail(AM_ERR_CUDA, std::string("cudaGetSymbolAddress(partial): ") + cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&s, g_noalloc_scalars);
        if (e != cudaSuccess)
            return noalloc_fail(AM_ERR_CUDA, std::string("cudaGetSymbolAddress(scalars): ") + cudaGetErrorString(e));
        d.partial = static_cast<double *>(p);
        d.scalars = static_cast<Scalars *>(s);
        d.ready = true;
    }
    *out = &d;
    return AM_OK;
}

}  // namespace

extern "C" am_status am_residual_noalloc(int nx, int ny, int nz, double h, double E0, double nu,
                                         const double *scale, const double *u, const double *f,
                                         const uint8_t *mask, double *r, double *rr, void *stream) {
    if (nx < 1 || ny < 1 || nz < 1) return noalloc_fail(AM_ERR_INVALID_ARG, "grid dimensions must be >= 1");
    if (nx >= INT_MAX || ny >= INT_MAX || nz >= INT_MAX)
        return noalloc_fail(AM_ERR_INVALID_ARG, "grid dimensions must be < INT_MAX");
    // tile count in 64-bit arithmetic, before any int-sized layout field is formed
    const long long tiles = ((long long)nx + 1 + 31) / 32 * (((long long)ny + 1 + 3) / 4);
    if (tiles > kNoAllocMaxTiles)
        return noalloc_fail(AM_ERR_SIZE_MISMATCH,
                            "grid too large for the fixed scratch: ceil((nx+1)/32)*ceil((ny+1)/4) = " +
                                std::to_string(tiles) + " > " + std::to_string(kNoAllocMaxTiles));
    if (!(h > 0.0) || !(E0 > 0.0) || !(nu > -1.0 && nu < 0.5))
        return noalloc_fail(AM_ERR_INVALID_ARG, "need h > 0, E0 > 0, -1 < nu < 0.5");
    if (!scale || !u || !f || !mask || !r || !rr) return noalloc_fail(AM_ERR_INVALID_ARG, "null device pointer");
    Layout L;
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.sx = nx + 1;  // compact layout: no row or plane padding
    L.sxy = (long long)(nx + 1) * (ny + 1);
    L.cs = L.sxy * (nz + 1);
    L.nel = (long long)nx * ny * nz;
    // FP64 tiles over the full z extent
    const KuLaunch K = ku_plan(L, true, nz + 1);
    if (K.ntiles() > kNoAllocMaxTiles)
        return noalloc_fail(AM_ERR_SIZE_MISMATCH,
                            "grid too large for the fixed scratch: ceil((nx+1)/32)*ceil((ny+1)/4) = " +
                                std::to_string(K.ntiles()) + " > " + std::to_string(kNoAllocMaxTiles));
    DeviceScratch *d = nullptr;
    am_status s = scratch_for_current_device(&d);
    if (s != AM_OK) return s;
    const double lam = E0 * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double mu = E0 / (2.0 * (1.0 + nu));
    const double a = h / 2.0;
    const Modal<double> M{lam, mu, a / 8.0, a / 24.0, a / 72.0, a / 72.0 * (lam + 4.0 * mu)};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the scalar block keeps the previous call's contents: its last-tile counter
    // must start at zero
    cudaError_t e = cudaMemsetAsync(d->scalars, 0, sizeof(Scalars), st);
    if (e != cudaSuccess) return noalloc_fail(AM_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    // no Jacobi weight: the kernel's r.(D^-1 r) sum is not formed
    e = ku_resid(K, L, M, scale, u, f, nullptr, mask, r, nullptr, d->partial, d->scalars, st);
    if (e != cudaSuccess) return noalloc_fail(AM_ERR_CUDA, std::string("residual kernel: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(rr, &d->scalars->res_rr, sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return noalloc_fail(AM_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return AM_OK;
}
