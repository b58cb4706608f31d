// CPU checks of the rigid-body deflation space construction (defl_space.h):
// components, the merge radius, disjoint supports, mode values and the limits.
// Exits non-zero, naming the failed check, on the first failure.
#include <cmath>
#include <cstdio>
#include <set>
#include <vector>

#include "defl_space.h"

using amk::DeflSpace;

static int fails = 0;
#define CHECK(cond, what)                              \
    do {                                               \
        if (!(cond)) {                                 \
            std::printf("FAIL %s\n", what);            \
            ++fails;                                   \
        }                                              \
    } while (0)

struct Grid {
    int nx, ny, nz;
    std::vector<uint8_t> solid;
    Grid(int x, int y, int z) : nx(x), ny(y), nz(z), solid((size_t)x * y * z, 0) {}
    void column(int x0, int y0, int w) {  // w x w elements, full height
        for (int z = 0; z < nz; ++z)
            for (int y = y0; y < y0 + w; ++y)
                for (int x = x0; x < x0 + w; ++x) solid[((size_t)z * ny + y) * nx + x] = 1;
    }
};

static bool build(const Grid &g, DeflSpace &s, long long sx = -1) {
    if (sx < 0) sx = g.nx + 1;
    return amk::defl_space(g.nx, g.ny, g.nz, sx, sx * (g.ny + 1), g.solid.data(), s);
}

int main() {
    {  // two 2 x 2 columns far apart: two components, supports of 5 x 5 x 7 nodes
        Grid g(24, 12, 6);
        g.column(4, 4, 2);
        g.column(16, 4, 2);
        DeflSpace s;
        CHECK(build(g, s), "two columns: built");
        CHECK(s.ncomp == 2, "two columns: 2 components");
        const long long nU = s.off.back();
        CHECK(s.off[1] == 175 && nU == 350, "two columns: supports of 175 nodes");
        std::set<long long> seen(s.unode.begin(), s.unode.end());
        CHECK((long long)seen.size() == nU, "two columns: disjoint supports");
        for (int c = 0; c < 2; ++c) {
            double tx = 0, rsum[3] = {0, 0, 0}, rmax = 0;
            int core = 0;
            for (long long u = s.off[c]; u < s.off[c + 1]; ++u) {
                CHECK(s.ucomp[u] == c, "two columns: entry component");
                const double t = s.z0[(size_t)(0 * 3 + 0) * nU + u];
                CHECK(t == 0.0 || t == 1.0, "two columns: translation 0 or 1");
                tx += t;
                core += t == 1.0;
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) {
                        const double v = s.z0[(size_t)((3 + r) * 3 + k) * nU + u];
                        rsum[k] += r == 0 ? v : 0.0;
                        rmax = std::fmax(rmax, std::fabs(v));
                    }
            }
            CHECK(core == 63 && tx == 63.0, "two columns: 3 x 3 x 7 core nodes");
            CHECK(std::fabs(rsum[1]) < 1e-9 && std::fabs(rsum[2]) < 1e-9, "two columns: rotation about the centroid");
            CHECK(rmax > 0.99 && rmax <= 1.0 + 1e-12, "two columns: rotations of unit size at the edge");
        }
    }
    {  // columns 3 elements apart merge; 4 apart stay two components with disjoint supports
        Grid a(24, 12, 6);
        a.column(4, 4, 2);
        a.column(8, 4, 2);
        DeflSpace s;
        CHECK(build(a, s) && s.ncomp == 1, "merge radius 3: one component");
        Grid b(24, 12, 6);
        b.column(4, 4, 2);
        b.column(9, 4, 2);
        CHECK(build(b, s) && s.ncomp == 2, "4 apart: two components");
        std::set<long long> seen(s.unode.begin(), s.unode.end());
        CHECK((long long)seen.size() == s.off.back(), "4 apart: disjoint supports");
    }
    {  // padded strides: device indices follow sx, sxy
        Grid g(6, 4, 2);
        g.solid[0] = 1;  // element (0, 0, 0)
        DeflSpace s;
        CHECK(build(g, s, 8), "padded: built");
        bool has_far = false;
        for (long long u : s.unode) has_far |= u == 1 * 8 * 5 + 1 * 8 + 1;  // node (1, 1, 1)
        CHECK(has_far, "padded: node (1,1,1) at 1 sxy + 1 sx + 1");
    }
    {  // limits: more than a quarter solid; more than 64 components
        Grid g(8, 8, 8);
        for (size_t e = 0; e < g.solid.size() / 3; ++e) g.solid[e] = 1;
        DeflSpace s;
        CHECK(!build(g, s), "a third solid: no deflation");
        Grid h(40, 40, 1);
        for (int y = 0; y < 40; y += 4)
            for (int x = 0; x < 40; x += 4) h.solid[(size_t)y * 40 + x] = 1;
        CHECK(!build(h, s), "100 components: no deflation");
        Grid none(4, 4, 4);
        CHECK(!build(none, s), "no solid: no deflation");
    }
    if (fails == 0) std::printf("ok\n");
    return fails == 0 ? 0 : 1;
}
