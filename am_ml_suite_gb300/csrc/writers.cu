// writers.cu -- the on-disk result formats of the reference's C++ driver
// (cpp_engine/src/am_topopt.cpp): the density field as a NumPy .npy file
// (saveNpy, :344-396), the run's metadata.json (saveMetadata, :401-447) and the
// convergence history.csv (:622-629).  Host code only; numbers are printed the way
// a default-configured C++ stream prints them (6 significant digits, %g).
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/am_gpu.h"
#include "kernels.cuh"

namespace {

am_status wfail(am_status s, const std::string &msg) {
    amk::set_last_error(msg.c_str());
    return s;
}

std::string g6(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%g", v);
    return b;
}

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) { f = std::fopen(path, mode); }
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

am_status am_write_density_npy(const char *path, const double *rho, int nx, int ny, int nz, int layout) {
    if (!path || !rho) return wfail(AM_ERR_INVALID_ARG, "null path or density");
    if (nx < 1 || ny < 1 || nz < 1) return wfail(AM_ERR_INVALID_ARG, "grid dimensions must be >= 1");
    if (layout != AM_LAYOUT_ZFASTEST && layout != AM_LAYOUT_XFASTEST)
        return wfail(AM_ERR_INVALID_ARG, "unknown layout");
    // header: magic, version 1.0, little-endian u16 length, the dict padded with
    // spaces so that the prefix is a multiple of 64 bytes, then a newline
    std::string dict = "{'descr': '<f8', 'fortran_order': False, 'shape': (" + std::to_string(nx) + ", " +
                       std::to_string(ny) + ", " + std::to_string(nz) + "), }";
    size_t hlen = dict.size() + 1;
    const size_t pad = (64 - (10 + hlen) % 64) % 64;
    hlen += pad;
    if (hlen > 65535) return wfail(AM_ERR_INVALID_ARG, "npy header too long");
    std::string head = "\x93NUMPY";
    head.push_back('\x01');
    head.push_back('\x00');
    head.push_back((char)(hlen & 0xff));
    head.push_back((char)(hlen >> 8));
    head += dict;
    head.append(pad, ' ');
    head.push_back('\n');
    // data in C order (i slowest, k fastest)
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> c(n);
    for (long long i = 0; i < nx; ++i)
        for (long long j = 0; j < ny; ++j)
            for (long long k = 0; k < nz; ++k) {
                const long long src = layout == AM_LAYOUT_ZFASTEST ? (i * ny + j) * nz + k : (k * ny + j) * nx + i;
                c[(size_t)((i * ny + j) * nz + k)] = rho[src];
            }
    File f(path, "wb");
    if (!f.f) return wfail(AM_ERR_INVALID_ARG, std::string("cannot open ") + path);
    if (std::fwrite(head.data(), 1, head.size(), f.f) != head.size() ||
        std::fwrite(c.data(), sizeof(double), n, f.f) != n)
        return wfail(AM_ERR_INVALID_ARG, std::string("write failed: ") + path);
    return AM_OK;
}

am_status am_write_history_csv(const char *path, const double *compliance, const double *volume, int n) {
    if (!path || n < 0 || (n > 0 && (!compliance || !volume)))
        return wfail(AM_ERR_INVALID_ARG, "need a path and n >= 0 history entries");
    std::string s = "iteration,compliance,volume\n";
    for (int i = 0; i < n; ++i) s += std::to_string(i) + "," + g6(compliance[i]) + "," + g6(volume[i]) + "\n";
    File f(path, "wb");
    if (!f.f) return wfail(AM_ERR_INVALID_ARG, std::string("cannot open ") + path);
    if (std::fwrite(s.data(), 1, s.size(), f.f) != s.size())
        return wfail(AM_ERR_INVALID_ARG, std::string("write failed: ") + path);
    return AM_OK;
}

am_status am_write_metadata_json(const char *path, const am_run_metadata *m) {
    if (!path || !m) return wfail(AM_ERR_INVALID_ARG, "null path or metadata");
    auto str = [](const char *v) { return std::string(v ? v : ""); };
    std::string s = "{\n";
    s += "  \"case\": \"" + str(m->case_name) + "\",\n";
    s += "  \"mode\": \"" + str(m->mode) + "\",\n";
    s += "  \"provenance\": \"" + str(m->provenance) + "\",\n";
    s += "  \"resolution_mm\": " + g6(m->resolution_mm) + ",\n";
    s += "  \"domain_shape\": [" + std::to_string(m->nx) + ", " + std::to_string(m->ny) + ", " +
         std::to_string(m->nz) + "],\n";
    s += "  \"n_elements\": " + std::to_string(m->n_elements) + ",\n";
    s += "  \"n_design\": " + std::to_string(m->n_design) + ",\n";
    s += "  \"n_fixed\": " + std::to_string(m->n_fixed) + ",\n";
    s += "  \"n_void\": " + std::to_string(m->n_void) + ",\n";
    s += "  \"volume_fraction_target\": " + g6(m->volume_fraction_target) + ",\n";
    if (m->has_history) {
        s += "  \"volume_fraction_final\": " + g6(m->volume_fraction_final) + ",\n";
        s += "  \"compliance_final\": " + g6(m->compliance_final) + ",\n";
    }
    s += "  \"iterations\": " + std::to_string(m->iterations) + ",\n";
    s += std::string("  \"converged\": ") + (m->converged ? "true" : "false") + ",\n";
    s += "  \"elapsed_time_s\": " + g6(m->elapsed_time_s) + ",\n";
    s += "  \"openmp_threads\": " + std::to_string(m->threads) + ",\n";
    s += "  \"simp_config\": {\n";
    s += "    \"filter_radius\": " + g6(m->filter_radius) + ",\n";
    s += "    \"E_min\": " + g6(m->E_min) + ",\n";
    s += "    \"penalty\": " + g6(m->penalty) + ",\n";
    s += "    \"move_limit\": " + g6(m->move_limit) + "\n";
    s += "  }\n}\n";
    File f(path, "wb");
    if (!f.f) return wfail(AM_ERR_INVALID_ARG, std::string("cannot open ") + path);
    if (std::fwrite(s.data(), 1, s.size(), f.f) != s.size())
        return wfail(AM_ERR_INVALID_ARG, std::string("write failed: ") + path);
    return AM_OK;
}

}  // extern "C"
