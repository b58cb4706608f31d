// setup.cu -- problem set-up of the reference's BRK-A-01 bracket on the device:
// the voxel grid of create_bracket_domain (src/am/core/geometry.py:79-196; the
// C++ driver's BracketDomain, cpp_engine/src/am_topopt.cpp:98-239, is the same
// construction stored x-fastest), the eyelet load ring and the base constraints
// of create_brk_a_01_static_case_1/2 (src/am/core/loads.py:163-306; C++
// createForceVector / createFixedDofs, am_topopt.cpp:248-334).
//
// The reference marks the grid by successive loops that overwrite each other
// (base slab fixed; base holes void; eyelet ring fixed where not void; eyelet
// hole void; pillar fixed where not void).  Here one thread per voxel applies
// the same rules in the same order to its own voxel, so the grid is identical
// cell for cell.  The in-circle tests compare exact integer sums of squares
// against the rounded square of the radius with explicitly rounded products
// (no fused multiply-add), as the reference's double arithmetic does; the ring
// test takes the correctly rounded square root like numpy / std::sqrt.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "kernels.cuh"

using namespace amk;

namespace {

am_status sfail(am_status s, const std::string &m) {
    set_last_error(m.c_str());
    return s;
}

#define SCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            return sfail(e_ == cudaErrorMemoryAllocation ? AM_ERR_OOM : AM_ERR_CUDA,                        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                               \
    } while (0)

// Derived integer geometry, with the reference's truncating conversions.
struct Bracket {
    int nx, ny, nz;
    int base_z;
    double hole_r;
    int hx[4], hy[4];
    int ex, ey;                   // eyelet axis (nx / 2, ny / 2)
    int z_start, z_end;           // eyelet extent
    double outer_r, inner_r;      // eyelet ring / hole radii (elements)
    int eyelet_z;                 // node plane of the load ring
    double ring_in, ring_out;     // load ring radii (elements)
    int search;
};

Bracket derive(const am_bracket_params &p) {
    Bracket b{};
    b.nx = p.nx;
    b.ny = p.ny;
    b.nz = p.nz;
    const double res = p.resolution_mm;
    b.base_z = std::max(1, (int)(p.base_thickness_mm / res));
    b.hole_r = p.hole_diameter_mm / 2.0 / res;
    const int ox = (int)(p.hole_offset_mm / res), oy = (int)(p.hole_offset_mm / res);
    const int hx[4] = {ox, b.nx - ox, ox, b.nx - ox}, hy[4] = {oy, oy, b.ny - oy, b.ny - oy};
    for (int i = 0; i < 4; ++i) {
        b.hx[i] = hx[i];
        b.hy[i] = hy[i];
    }
    const int zoff = (int)(p.eyelet_z_offset_mm / res);
    const int height = std::max(1, (int)(p.eyelet_height_mm / res));
    const int zc = b.nz - zoff;
    b.ex = b.nx / 2;
    b.ey = b.ny / 2;
    b.z_start = std::max(0, zc - height / 2);
    b.z_end = std::min(b.nz, b.z_start + height);
    b.outer_r = (p.eyelet_diameter_mm / 2.0 + p.eyelet_offset_mm) / res;
    b.inner_r = p.eyelet_diameter_mm / 2.0 / res;
    // load ring (loads.py:213-259): mid-height node plane, a safety margin of 1.25
    // voxels inside the hole's edge
    b.eyelet_z = std::max(1, std::min(b.nz - 1, (b.z_start + b.z_end) / 2));
    double in_mm = p.eyelet_diameter_mm / 2.0 + res * 1.25;
    const double out_mm = p.eyelet_diameter_mm / 2.0 + p.eyelet_offset_mm;
    if (in_mm >= out_mm) in_mm = p.eyelet_diameter_mm / 2.0 + p.eyelet_offset_mm * 0.5;
    b.ring_out = out_mm / res;
    b.ring_in = in_mm / res;
    b.search = (int)b.ring_out + 2;
    return b;
}

__device__ __forceinline__ bool in_circle(int i, int j, double cx, double cy, double r) {
    const double di = (double)i - cx, dj = (double)j - cy;
    return __dadd_rn(__dmul_rn(di, di), __dmul_rn(dj, dj)) <= __dmul_rn(r, r);
}

// grid value of element (i, j, k), the reference's marking order
__global__ void bracket_grid_kernel(Bracket b, int layout, int8_t *__restrict__ grid) {
    const long long n = (long long)b.nx * b.ny * b.nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        // t enumerates the output layout
        int i, j, k;
        if (layout == AM_LAYOUT_ZFASTEST) {
            k = (int)(t % b.nz);
            j = (int)((t / b.nz) % b.ny);
            i = (int)(t / ((long long)b.nz * b.ny));
        } else {
            i = (int)(t % b.nx);
            j = (int)((t / b.nx) % b.ny);
            k = (int)(t / ((long long)b.nx * b.ny));
        }
        int8_t g = 0;
        if (k < b.base_z) g = 1;  // base flange
        if (k < b.base_z)         // holes through the flange
            for (int h = 0; h < 4; ++h)
                if (in_circle(i, j, b.hx[h], b.hy[h], b.hole_r)) g = -1;
        if (b.z_end > b.z_start && k >= b.z_start && k < b.z_end) {
            if (in_circle(i, j, b.ex, b.ey, b.outer_r) && g != -1) g = 1;  // eyelet ring
            if (in_circle(i, j, b.ex, b.ey, b.inner_r)) g = -1;             // eyelet hole
        }
        // pillar from the flange to the eyelet, same radius as the ring
        if (b.z_start > b.base_z && k >= b.base_z && k < b.z_start && in_circle(i, j, b.ex, b.ey, b.outer_r) &&
            g != -1)
            g = 1;
        grid[t] = g;
    }
}

// flag[(i - i0) * wj + (j - j0)] = node (i, j) of plane eyelet_z is on the load ring
__global__ void ring_kernel(Bracket b, int i0, int j0, int wi, int wj, uint8_t *__restrict__ flag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= wi * wj) return;
    const int i = i0 + t / wj, j = j0 + t % wj;
    const double di = (double)(i - b.ex), dj = (double)(j - b.ey);
    const double d = sqrt(__dadd_rn(__dmul_rn(di, di), __dmul_rn(dj, dj)));
    flag[t] = (uint8_t)(d > b.ring_in && d <= b.ring_out);
}

// base constraints: every node of plane k = 0, all three components, ascending
__global__ void base_dofs_kernel(Bracket b, long long *__restrict__ out) {
    const long long n = 3LL * (b.nx + 1) * (b.ny + 1);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long ij = t / 3;
        const int d = (int)(t % 3);
        const long long i = ij / (b.ny + 1), j = ij % (b.ny + 1);
        out[t] = 3 * (i * (b.ny + 1) * (b.nz + 1) + j * (b.nz + 1)) + d;
    }
}

// F: per load node the total force divided by the node count (loads.py:107-149)
__global__ void ring_force_kernel(const long long *__restrict__ nodes, long long count, double fx, double fy,
                                  double fz, double *__restrict__ F) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const long long n = nodes[t];
    F[3 * n + 0] = fx / (double)count;
    F[3 * n + 1] = fy / (double)count;
    F[3 * n + 2] = fz / (double)count;
}

int blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 8)); }

}  // namespace

extern "C" {

void am_bracket_params_default(am_bracket_params *p, double resolution_mm) {
    if (!p) return;
    p->size_mm[0] = 120.0;
    p->size_mm[1] = 60.0;
    p->size_mm[2] = 80.0;
    p->resolution_mm = resolution_mm;
    p->base_thickness_mm = 5.0;
    p->hole_diameter_mm = 8.0;
    p->hole_offset_mm = 15.0;
    p->eyelet_diameter_mm = 12.0;
    p->eyelet_offset_mm = 4.0;
    p->eyelet_z_offset_mm = 15.0;
    p->eyelet_height_mm = 20.0;
    p->nx = resolution_mm > 0.0 ? (int)(p->size_mm[0] / resolution_mm) : 0;
    p->ny = resolution_mm > 0.0 ? (int)(p->size_mm[1] / resolution_mm) : 0;
    p->nz = resolution_mm > 0.0 ? (int)(p->size_mm[2] / resolution_mm) : 0;
}

am_status am_bracket_build(const am_bracket_params *p, const double total_force[3], int layout, int8_t *grid,
                           double *F, int64_t *fixed, int64_t *n_fixed, int64_t *load_nodes, int64_t *n_load_nodes,
                           int64_t load_nodes_capacity) {
    if (!p) return sfail(AM_ERR_INVALID_ARG, "null parameters");
    if (p->nx < 1 || p->ny < 1 || p->nz < 1 || !(p->resolution_mm > 0.0))
        return sfail(AM_ERR_INVALID_ARG, "need nx, ny, nz >= 1 and resolution_mm > 0");
    if (layout != AM_LAYOUT_ZFASTEST && layout != AM_LAYOUT_XFASTEST)
        return sfail(AM_ERR_INVALID_ARG, "unknown layout");
    if (F && !total_force) return sfail(AM_ERR_INVALID_ARG, "F needs total_force");
    if (!am_is_available()) return sfail(AM_ERR_NO_DEVICE, "no CUDA device");
    const Bracket b = derive(*p);
    const long long nel = (long long)b.nx * b.ny * b.nz;
    const long long nnode = (long long)(b.nx + 1) * (b.ny + 1) * (b.nz + 1);
    cudaStream_t st = nullptr;
    SCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Guard {
        std::vector<void *> ptrs;
        cudaStream_t st;
        ~Guard() {
            if (st) cudaStreamSynchronize(st);
            for (void *q : ptrs) cudaFree(q);
            if (st) cudaStreamDestroy(st);
        }
    } guard{{}, st};
    auto dalloc = [&](size_t bytes, void **out) -> cudaError_t {
        cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 1));
        if (e == cudaSuccess) guard.ptrs.push_back(*out);
        return e;
    };
    if (grid) {
        int8_t *g = nullptr;
        SCK(dalloc((size_t)nel, reinterpret_cast<void **>(&g)));
        bracket_grid_kernel<<<blocks(nel), 256, 0, st>>>(b, layout, g);
        SCK(cudaGetLastError());
        SCK(cudaMemcpyAsync(grid, g, (size_t)nel, cudaMemcpyDeviceToHost, st));
        count_launches(1);
    }
    if (fixed || n_fixed) {
        const long long nf = 3LL * (b.nx + 1) * (b.ny + 1);
        if (n_fixed) *n_fixed = nf;
        if (fixed) {
            long long *d = nullptr;
            SCK(dalloc(sizeof(long long) * (size_t)nf, reinterpret_cast<void **>(&d)));
            base_dofs_kernel<<<blocks(nf), 256, 0, st>>>(b, d);
            SCK(cudaGetLastError());
            SCK(cudaMemcpyAsync(fixed, d, sizeof(long long) * (size_t)nf, cudaMemcpyDeviceToHost, st));
            count_launches(1);
        }
    }
    if (F || load_nodes || n_load_nodes) {
        // the load ring in the reference's loop order (i outer, j inner)
        const int i0 = std::max(0, b.ex - b.search), i1 = std::min(b.nx, b.ex + b.search);
        const int j0 = std::max(0, b.ey - b.search), j1 = std::min(b.ny, b.ey + b.search);
        const int wi = std::max(0, i1 - i0 + 1), wj = std::max(0, j1 - j0 + 1);
        std::vector<uint8_t> flag((size_t)wi * wj);
        if (!flag.empty()) {
            uint8_t *df = nullptr;
            SCK(dalloc(flag.size(), reinterpret_cast<void **>(&df)));
            ring_kernel<<<(int)((flag.size() + 255) / 256), 256, 0, st>>>(b, i0, j0, wi, wj, df);
            SCK(cudaGetLastError());
            SCK(cudaMemcpyAsync(flag.data(), df, flag.size(), cudaMemcpyDeviceToHost, st));
            SCK(cudaStreamSynchronize(st));
            count_launches(1);
        }
        std::vector<long long> nodes;
        for (int a = 0; a < wi; ++a)
            for (int c = 0; c < wj; ++c)
                if (flag[(size_t)a * wj + c])
                    nodes.push_back(((long long)(i0 + a) * (b.ny + 1) + (j0 + c)) * (b.nz + 1) + b.eyelet_z);
        if (nodes.empty())  // no ring node: the centre node (loads.py:262-264)
            nodes.push_back(((long long)b.ex * (b.ny + 1) + b.ey) * (b.nz + 1) + b.eyelet_z);
        if (n_load_nodes) *n_load_nodes = (int64_t)nodes.size();
        if (load_nodes) {
            if ((long long)nodes.size() > load_nodes_capacity)
                return sfail(AM_ERR_SIZE_MISMATCH, "load_nodes holds " + std::to_string(load_nodes_capacity) +
                                                       " entries, the ring has " + std::to_string(nodes.size()));
            std::copy(nodes.begin(), nodes.end(), load_nodes);
        }
        if (F) {
            double *dF = nullptr;
            long long *dn = nullptr;
            SCK(dalloc(sizeof(double) * 3 * (size_t)nnode, reinterpret_cast<void **>(&dF)));
            SCK(dalloc(sizeof(long long) * nodes.size(), reinterpret_cast<void **>(&dn)));
            SCK(cudaMemsetAsync(dF, 0, sizeof(double) * 3 * (size_t)nnode, st));
            SCK(cudaMemcpyAsync(dn, nodes.data(), sizeof(long long) * nodes.size(), cudaMemcpyHostToDevice, st));
            ring_force_kernel<<<(int)((nodes.size() + 255) / 256), 256, 0, st>>>(
                dn, (long long)nodes.size(), total_force[0], total_force[1], total_force[2], dF);
            SCK(cudaGetLastError());
            SCK(cudaMemcpyAsync(F, dF, sizeof(double) * 3 * (size_t)nnode, cudaMemcpyDeviceToHost, st));
            count_launches(1);
        }
    }
    SCK(cudaStreamSynchronize(st));
    return AM_OK;
}

}  // extern "C"
