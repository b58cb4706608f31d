// selftest.cu -- checks of the engine's device-side safety paths that need no
// fault: a bounded wait on a copy barrier that nothing completes returns with an
// error flag instead of spinning.
#include <cuda_runtime.h>

#include <chrono>

#include "../../include/am_gpu.h"
#include "bulk.cuh"
#include "kernels.cuh"

using namespace amk;

namespace {

// One thread initialises a copy barrier expecting one arrival that never comes
// (no copy is issued), then waits on it with the bounded wait every copy stage
// of the solver uses, shortened to limit_ns; out[0] = 1 if the wait gave up,
// out[1] = the nanoseconds it waited.
__global__ void copy_wait_probe_kernel(unsigned long long limit_ns, unsigned long long *out) {
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    bulk::bar_init(&bar, 1);
    bulk::bar_init_fence();
    const unsigned long long t0 = bulk::now_ns();
    const bool ok = bulk::bar_wait(&bar, 0u, limit_ns);
    out[0] = ok ? 0ull : 1ull;
    out[1] = bulk::now_ns() - t0;
}

}  // namespace

extern "C" am_status am_selftest_copy_wait(double limit_ms, int *timed_out, double *waited_ms) {
    if (!timed_out || !waited_ms) return AM_ERR_INVALID_ARG;
    if (!(limit_ms > 0.0) || limit_ms > 100.0) return AM_ERR_INVALID_ARG;
    if (!am_is_available()) return AM_ERR_NO_DEVICE;
    unsigned long long *d = nullptr, h[2] = {0, 0};
    cudaError_t e = cudaMalloc(&d, sizeof(h));
    if (e == cudaSuccess) {
        copy_wait_probe_kernel<<<1, 32>>>((unsigned long long)(limit_ms * 1e6), d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return AM_ERR_CUDA;
    }
    count_launches(1);
    *timed_out = (int)h[0];
    *waited_ms = (double)h[1] * 1e-6;
    return AM_OK;
}
