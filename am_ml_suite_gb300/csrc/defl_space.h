// defl_space.h -- host construction of the rigid-body deflation space (defl.h):
// the components of the passive solid elements, their node supports and the six
// rigid-body modes of each.  Plain C++ (no CUDA), shared by defl.cu and the CPU
// test of this construction.
//
// Grid: nx * ny * nz elements, element e = (ez ny + ey) nx + ex; nodes (nx+1) *
// (ny+1) * (nz+1), device index of node (ix, iy, iz) = iz sxy + iy sx + ix.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <numeric>
#include <vector>

namespace amk {

constexpr int DEFL_MAX_COMPONENTS = 64;
constexpr int DEFL_MERGE = 3;  // components closer than this many elements are merged

struct DeflSpace {
    int ncomp = 0;
    std::vector<long long> off;    // component c owns entries [off[c], off[c+1])
    std::vector<long long> unode;  // device node index of each entry (its support: nodes + one ring)
    std::vector<int> ucomp;        // component of each entry
    std::vector<double> z0;        // [6][3][nU]: translations x, y, z, then rotations about x, y, z
};

// Builds the space for the elements flagged in solid (nx ny nz entries); false
// (no deflation) when there is none, when they are more than a quarter of the
// elements, or when they form more than DEFL_MAX_COMPONENTS components.  Elements
// within DEFL_MERGE of each other (Chebyshev distance of element indices) join one
// component, so the supports of different components are disjoint.
inline bool defl_space(int nx, int ny, int nz, long long sx, long long sxy, const uint8_t *solid, DeflSpace &out) {
    out = DeflSpace{};
    const long long nel = (long long)nx * ny * nz;
    std::vector<long long> elems;
    for (long long e = 0; e < nel; ++e)
        if (solid[e]) elems.push_back(e);
    // none, or so many that the coarse grids represent them (and the mode arrays
    // would span most of the grid): no deflation
    if (elems.empty() || (long long)elems.size() > nel / 4) return false;
    auto eidx = [&](int x, int y, int z) { return ((long long)z * ny + y) * nx + x; };
    // union-find over the solid elements, merging those within DEFL_MERGE elements
    std::vector<int> pos((size_t)nel, -1);
    for (size_t i = 0; i < elems.size(); ++i) pos[(size_t)elems[i]] = (int)i;
    std::vector<int> parent(elems.size());
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int i) {
        while (parent[i] != i) i = parent[i] = parent[parent[i]];
        return i;
    };
    for (size_t i = 0; i < elems.size(); ++i) {
        const long long e = elems[i];
        const int ex = (int)(e % nx), ey = (int)((e / nx) % ny), ez = (int)(e / ((long long)nx * ny));
        for (int dz = -DEFL_MERGE; dz <= DEFL_MERGE; ++dz)
            for (int dy = -DEFL_MERGE; dy <= DEFL_MERGE; ++dy)
                for (int dx = -DEFL_MERGE; dx <= DEFL_MERGE; ++dx) {
                    const int x = ex + dx, y = ey + dy, z = ez + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
                    const int j = pos[(size_t)eidx(x, y, z)];
                    if (j > (int)i) {
                        const int a = find((int)i), b = find(j);
                        if (a != b) parent[std::max(a, b)] = std::min(a, b);
                    }
                }
    }
    std::vector<int> label(elems.size()), root_id(elems.size(), -1);
    int ncomp = 0;
    for (size_t i = 0; i < elems.size(); ++i) {
        const int r = find((int)i);
        if (root_id[r] < 0) root_id[r] = ncomp++;
        label[i] = root_id[r];
    }
    if (ncomp > DEFL_MAX_COMPONENTS) return false;
    // core nodes (nodes of the component's elements) and support (core + one ring)
    const long long nnx = nx + 1, nny = ny + 1, nnz = nz + 1, nn = nnx * nny * nnz;
    auto nid = [&](long long x, long long y, long long z) { return (z * nny + y) * nnx + x; };
    std::vector<int> core((size_t)nn, -1), supp((size_t)nn, -1);
    for (size_t i = 0; i < elems.size(); ++i) {
        const long long e = elems[i];
        const int ex = (int)(e % nx), ey = (int)((e / nx) % ny), ez = (int)(e / ((long long)nx * ny));
        for (int c = 0; c < 8; ++c) core[(size_t)nid(ex + (c & 1), ey + ((c >> 1) & 1), ez + (c >> 2))] = label[i];
    }
    std::vector<double> cen((size_t)ncomp * 3, 0.0), cnt((size_t)ncomp, 0.0);
    std::vector<double> lo((size_t)ncomp * 3, 1e300), hi((size_t)ncomp * 3, -1e300);
    for (long long n = 0; n < nn; ++n) {
        const int c = core[(size_t)n];
        if (c < 0) continue;
        const long long x = n % nnx, y = (n / nnx) % nny, z = n / (nnx * nny);
        const double p[3] = {(double)x, (double)y, (double)z};
        for (int k = 0; k < 3; ++k) {
            cen[(size_t)c * 3 + k] += p[k];
            lo[(size_t)c * 3 + k] = std::min(lo[(size_t)c * 3 + k], p[k]);
            hi[(size_t)c * 3 + k] = std::max(hi[(size_t)c * 3 + k], p[k]);
        }
        cnt[(size_t)c] += 1.0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const long long X = x + dx, Y = y + dy, Z = z + dz;
                    if (X < 0 || Y < 0 || Z < 0 || X >= nnx || Y >= nny || Z >= nnz) continue;
                    supp[(size_t)nid(X, Y, Z)] = c;  // supports of merged-apart components are disjoint
                }
    }
    std::vector<double> scale((size_t)ncomp);
    for (int c = 0; c < ncomp; ++c) {
        double ext = 1.0;
        for (int k = 0; k < 3; ++k) {
            cen[(size_t)c * 3 + k] /= cnt[(size_t)c];
            ext = std::max(ext, 0.5 * (hi[(size_t)c * 3 + k] - lo[(size_t)c * 3 + k]));
        }
        scale[(size_t)c] = 1.0 / ext;  // rotations of unit size at the component's edge
    }
    // entries grouped by component, nodes ascending
    std::vector<std::vector<long long>> members((size_t)ncomp);
    for (long long n = 0; n < nn; ++n)
        if (supp[(size_t)n] >= 0) members[(size_t)supp[(size_t)n]].push_back(n);
    out.ncomp = ncomp;
    out.off.assign((size_t)ncomp + 1, 0);
    for (int c = 0; c < ncomp; ++c) out.off[(size_t)c + 1] = out.off[(size_t)c] + (long long)members[(size_t)c].size();
    const long long nU = out.off.back();
    out.unode.resize((size_t)nU);
    out.ucomp.resize((size_t)nU);
    out.z0.assign((size_t)18 * nU, 0.0);
    for (int c = 0; c < ncomp; ++c)
        for (size_t q = 0; q < members[(size_t)c].size(); ++q) {
            const long long u = out.off[(size_t)c] + (long long)q, n = members[(size_t)c][q];
            const long long x = n % nnx, y = (n / nnx) % nny, z = n / (nnx * nny);
            out.unode[(size_t)u] = z * sxy + y * sx + x;
            out.ucomp[(size_t)u] = c;
            if (core[(size_t)n] != c) continue;  // ring nodes: Z = 0, K Z may not be
            // coordinates in node steps, scaled so the rotations are of unit size at the edge
            const double s = scale[(size_t)c];
            const double dx = s * (x - cen[(size_t)c * 3]), dy = s * (y - cen[(size_t)c * 3 + 1]),
                         dz = s * (z - cen[(size_t)c * 3 + 2]);
            // translations, then rotations e_k x d
            const double modes[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, -dz, dy}, {dz, 0, -dx}, {-dy, dx, 0}};
            for (int t = 0; t < 6; ++t)
                for (int k = 0; k < 3; ++k) out.z0[(size_t)(t * 3 + k) * nU + u] = modes[t][k];
        }
    return true;
}

}  // namespace amk
