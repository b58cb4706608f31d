// batch_axes.h -- the axis order a batched problem is stored in, and the index
// maps between the caller's order and it (plain C++, host only; checked on the
// CPU by tests/batch_axes_check.cpp).
//
// The cube's element stiffness is the same when the three axes and the
// displacement components are permuted together, and the cone filter and the OC
// step do not see axes.  So each problem of a batch may keep its grid in whichever
// axis order makes the batched K*u's tiles overhang it least.  The caller's order
// is restored at the boundary: loads, constraints and densities.
#pragma once
#include <array>

namespace amk {

// The order for a grid of d[0] x d[1] x d[2] elements: out[a] is the caller's axis
// stored as internal axis a.  Chosen to minimise the element slots of tiles of tx
// node columns x ty node rows over all node planes plus a halo plane (32 lanes x
// (ty + 1) element rows per tile and plane); ties keep the caller's order.
inline std::array<int, 3> best_axes(const int d[3], int tx = 28, int ty = 15) {
    static const int P[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    auto div_up = [](long long a, long long b) { return (a + b - 1) / b; };
    long long best = -1;
    std::array<int, 3> out{0, 1, 2};
    for (const auto &q : P) {
        const long long slots =
            div_up(d[q[0]] + 1, tx) * 32 * div_up(d[q[1]] + 1, ty) * (ty + 1) * (long long)(d[q[2]] + 2);
        if (best < 0 || slots < best) {
            best = slots;
            out = {q[0], q[1], q[2]};
        }
    }
    return out;
}

// internal coordinates q of the caller's coordinates c3 (node or element)
inline void to_internal(const std::array<int, 3> &ax, const long long c3[3], long long q[3]) {
    for (int a = 0; a < 3; ++a) q[a] = c3[ax[a]];
}

// the internal displacement component of the caller's component c
inline int internal_component(const std::array<int, 3> &ax, int c) {
    for (int a = 0; a < 3; ++a)
        if (ax[a] == c) return a;
    return c;
}

// The caller's index of internal element (ex, ey, ez) on a grid whose caller-order
// dimensions are dm: C order over (nx, ny, nz) (z fastest) when zfastest, else x
// fastest.
inline long long host_element(const std::array<int, 3> &ax, const std::array<int, 3> &dm, bool zfastest,
                              long long ex, long long ey, long long ez) {
    long long c3[3];
    c3[ax[0]] = ex;
    c3[ax[1]] = ey;
    c3[ax[2]] = ez;
    return zfastest ? (c3[0] * dm[1] + c3[1]) * dm[2] + c3[2] : (c3[2] * dm[1] + c3[1]) * dm[0] + c3[0];
}

}  // namespace amk
