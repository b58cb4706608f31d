// host_util.h -- host-side helpers shared by the single-problem engine
// (am_gpu.cu) and the batched engine (batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "am_common.cuh"
#include "ku.cuh"

namespace amk {

// Device layout of an nx*ny*nz grid (am_common.cuh): rows padded to 4 nodes,
// component planes padded to 64 entries.
inline Layout make_layout(int nx, int ny, int nz) {
    Layout L;
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.sx = ((nx + 1) + 3) / 4 * 4;
    L.sxy = (long long)L.sx * (ny + 1);
    L.cs = (L.sxy * (nz + 1) + 63) / 64 * 64;
    L.nel = (long long)nx * ny * nz;
    return L;
}

// Walsh-basis constants of the hex8 cube of edge h, material (E, nu) (ku.cuh).
inline Modal<double> modal_constants(double E, double nu, double h) {
    const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double mu = E / (2.0 * (1.0 + nu));
    const double a = h / 2.0;
    return Modal<double>{lam, mu, a / 8.0, a / 24.0, a / 72.0, a / 72.0 * (lam + 4.0 * mu)};
}
inline Modal<float> modal_float(const Modal<double> &M) {
    return Modal<float>{(float)M.lam, (float)M.mu, (float)M.c1, (float)M.c2, (float)M.c3, (float)M.c7};
}

// Entry (row, col) of KE, evaluated with the same operator the kernels apply.
inline double element_stiffness_entry(const Modal<double> &M, int row, int col) {
    double u[3][8] = {}, y[3][8];
    u[col % 3][col / 3] = 1.0;
    hex8_apply<double>(u, y, M, 1.0, nullptr);
    return y[row % 3][row / 3];
}

// Sensitivity-filter taps of radius r.  variant 0 (CPP): neighbour search order
// dz, dy, dx (topology_optimizer.cpp:76-101), weight max(0, r - dist) for
// dist <= r.  variant 1 (PY): the (2R+1)^3 box of r - dist for dist <= r,
// normalised by its sum taken in C order (topopt.py:135-151).
inline void filter_taps(double r, int variant, std::vector<int4> &d, std::vector<double> &w) {
    d.clear();
    w.clear();
    const int R = (int)std::ceil(r);
    for (int dz = -R; dz <= R; ++dz)
        for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
                const double dist = std::sqrt((double)(dx * dx + dy * dy + dz * dz));
                if (dist <= r) {
                    const double wt = variant == 0 ? std::max(0.0, r - dist) : r - dist;
                    if (variant == 1 && wt == 0.0) continue;
                    d.push_back(make_int4(dx, dy, dz, 0));
                    w.push_back(wt);
                }
            }
    if (variant == 1) {
        double t2 = 0.0;
        for (int a = 0; a < 2 * R + 1; ++a)
            for (int b = 0; b < 2 * R + 1; ++b)
                for (int c = 0; c < 2 * R + 1; ++c) {
                    const double dist =
                        std::sqrt((double)((a - R) * (a - R) + (b - R) * (b - R) + (c - R) * (c - R)));
                    if (dist <= r) t2 += r - dist;
                }
        for (auto &x : w) x /= t2;
    }
}

}  // namespace amk
