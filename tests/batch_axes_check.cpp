// CPU checks of the batch's axis order and its index maps (batch_axes.h): the
// order chosen for the shapes the GPU tests use, and for every order that the
// node, component and element maps are bijections that invert one another.
// Exits non-zero, naming the failed check, on the first failure.
#include <cstdio>
#include <vector>

#include "batch_axes.h"

using amk::best_axes;

static int fails = 0;
#define CHECK(cond, what)                   \
    do {                                    \
        if (!(cond)) {                      \
            std::printf("FAIL %s\n", what); \
            ++fails;                        \
        }                                   \
    } while (0)

int main() {
    // orders chosen for 28 x 15-node tiles (the staged kernel's)
    {
        const int a[3] = {6, 40, 9}, b[3] = {9, 5, 7}, c[3] = {20, 4, 3}, d[3] = {96, 48, 48};
        CHECK((best_axes(a) == std::array<int, 3>{1, 2, 0}), "(6, 40, 9): 40 in x, 9 in y, 6 marching");
        CHECK((best_axes(b) == std::array<int, 3>{0, 2, 1}), "(9, 5, 7): y and z swapped");
        CHECK((best_axes(c) == std::array<int, 3>{0, 1, 2}), "(20, 4, 3): caller's order");
        // 48 across the 28-column tiles (2 tile columns), 96 across the 15-row tiles (7):
        // 358,400 element slots against 409,600 in the caller's order; (2, 0, 1) ties
        // and the first of the two is kept
        CHECK((best_axes(d) == std::array<int, 3>{1, 0, 2}), "(96, 48, 48): 48 in x, 96 in y");
    }
    // the chosen order never computes more element slots than the caller's
    for (int x = 1; x <= 40; x += 3)
        for (int y = 1; y <= 40; y += 4)
            for (int z = 1; z <= 40; z += 5) {
                const int dd[3] = {x, y, z};
                const auto ax = best_axes(dd);
                auto slots = [&](int p, int q, int r) {
                    return (long long)((p + 28) / 28) * 32 * ((q + 15) / 15) * 16 * (r + 2);
                };
                CHECK(slots(dd[ax[0]], dd[ax[1]], dd[ax[2]]) <= slots(x, y, z), "no worse than the caller's order");
            }
    // every order: elements, nodes and components map one to one
    static const int P[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const std::array<int, 3> dm{5, 3, 4};
    for (const auto &q : P) {
        const std::array<int, 3> ax{q[0], q[1], q[2]};
        const int nxi = dm[ax[0]], nyi = dm[ax[1]], nzi = dm[ax[2]];
        for (int zf = 0; zf < 2; ++zf) {
            std::vector<int> seen(dm[0] * dm[1] * dm[2], 0);
            for (long long ez = 0; ez < nzi; ++ez)
                for (long long ey = 0; ey < nyi; ++ey)
                    for (long long ex = 0; ex < nxi; ++ex) {
                        const long long h = amk::host_element(ax, dm, zf != 0, ex, ey, ez);
                        CHECK(h >= 0 && h < (long long)seen.size(), "element index in range");
                        if (h >= 0 && h < (long long)seen.size()) ++seen[h];
                    }
            bool once = true;
            for (int v : seen) once = once && v == 1;
            CHECK(once, "every caller element exactly once");
        }
        // a caller node (i, j, k) lands on internal coordinates whose dimensions are
        // the permuted ones, and host_element inverts to_internal on elements
        for (long long i = 0; i < dm[0]; ++i)
            for (long long j = 0; j < dm[1]; ++j)
                for (long long k = 0; k < dm[2]; ++k) {
                    const long long c3[3] = {i, j, k};
                    long long qi[3];
                    amk::to_internal(ax, c3, qi);
                    CHECK(qi[0] < nxi && qi[1] < nyi && qi[2] < nzi, "internal coordinates in range");
                    CHECK(amk::host_element(ax, dm, true, qi[0], qi[1], qi[2]) == (i * dm[1] + j) * dm[2] + k,
                          "host_element inverts to_internal (z fastest)");
                    CHECK(amk::host_element(ax, dm, false, qi[0], qi[1], qi[2]) == (k * dm[1] + j) * dm[0] + i,
                          "host_element inverts to_internal (x fastest)");
                }
        // a displacement component follows its axis
        for (int c = 0; c < 3; ++c) CHECK(ax[amk::internal_component(ax, c)] == c, "component follows its axis");
    }
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
