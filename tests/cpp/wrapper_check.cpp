// Compiled check of the header-only C++ wrapper (include/am_gpu.hpp): the
// reference's TopologyOptimizer interface over the C ABI.
//
//   wrapper_check cpu   argument and device errors map to the reference's
//                       exception types (runs without a GPU)
//   wrapper_check gpu   a 24x12x6 cantilever through run() with and without a
//                       callback and through runIteration(), against the FP64
//                       CPU oracle (liboracle.so)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/am_gpu.hpp"
#include "../../oracle/oracle.h"

namespace gt = am::gpu::topopt;
namespace gf = am::gpu::fem;

static int failures = 0;
#define EXPECT(cond, what)                                          \
    do {                                                            \
        if (!(cond)) {                                              \
            std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, what); \
            ++failures;                                             \
        }                                                           \
    } while (0)

template <class E, class F>
static bool throws(F f) {
    try {
        f();
    } catch (const E &) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

static int cpu_checks() {
    gt::SIMPConfig cfg;
    cfg.verbose = false;
    EXPECT(throws<std::invalid_argument>([&] { gt::TopologyOptimizer t(0, 4, 4, 1.0, gf::MaterialProperties(1.0, 0.3), cfg); }),
           "a zero dimension is std::invalid_argument");
    EXPECT(throws<std::invalid_argument>([&] { gt::TopologyOptimizer t(4, 4, 4, -1.0, gf::MaterialProperties(1.0, 0.3), cfg); }),
           "a negative element size is std::invalid_argument");
    if (!am_is_available())
        EXPECT(throws<std::runtime_error>([&] { gt::TopologyOptimizer t(4, 4, 4, 1.0, gf::MaterialProperties(1.0, 0.3), cfg); }),
               "no device is std::runtime_error");
    EXPECT(std::string(am_status_string(AM_ERR_TIMEOUT)) == "AM_ERR_TIMEOUT", "status names");
    std::printf("sizeof(am_simp_config) %zu sizeof(am_iteration_result) %zu sizeof(am_solve_stats) %zu\n",
                sizeof(am_simp_config), sizeof(am_iteration_result), sizeof(am_solve_stats));
    return failures;
}

static void cantilever(int nx, int ny, int nz, std::vector<double> &F, std::vector<int64_t> &fixed) {
    const int64_t N = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    F.assign((size_t)N, 0.0);
    fixed.clear();
    for (int j = 0; j <= ny; ++j)
        for (int k = 0; k <= nz; ++k)
            for (int d = 0; d < 3; ++d) fixed.push_back(3 * ((int64_t)j * (nz + 1) + k) + d);
    for (int j = 0; j <= ny; ++j) {
        const int64_t n = ((int64_t)nx * (ny + 1) + j) * (nz + 1) + nz / 2;
        F[(size_t)(3 * n + 2)] = -1.0 / (ny + 1);
    }
}

static int gpu_checks() {
    const int nx = 24, ny = 12, nz = 6, iters = 8;
    std::vector<double> F;
    std::vector<int64_t> fixed;
    cantilever(nx, ny, nz, F, fixed);
    gt::SIMPConfig cfg;
    cfg.verbose = false;
    cfg.volume_fraction = 0.3;
    cfg.filter_radius = 1.5;
    cfg.E_min = 1e-9;
    cfg.max_iterations = iters;
    cfg.convergence_tol = 0.0;
    cfg.cg_tol = 1e-10;
    gt::TopologyOptimizer opt(nx, ny, nz, 1.0, gf::MaterialProperties(1.0, 0.3), cfg);
    EXPECT(opt.numElements() == (int64_t)nx * ny * nz && opt.numDofs() == (int64_t)F.size(), "sizes");

    // the FP64 oracle: uniform start, so both layouts coincide
    const int64_t nel = (int64_t)nx * ny * nz;
    std::vector<double> rho0((size_t)nel, 0.3), rho_ref((size_t)nel), c_ref(iters), v_ref(iters), d_ref(iters);
    std::vector<int> cg(iters);
    int conv = 0;
    orc_simp_params prm{};
    prm.volume_fraction = 0.3;
    prm.penalty = 3.0;
    prm.filter_radius = 1.5;
    prm.move_limit = 0.2;
    prm.rho_min = 0.01;
    prm.E_min = 1e-9;
    prm.convergence_tol = 0.0;
    prm.max_iterations = iters;
    prm.cg_tol = 1e-12;
    prm.cg_maxit = 100000;
    prm.warm_start = 1;
    const int n_ref = orc_simp_cpp(nx, ny, nz, 1.0, 1.0, 0.3, &prm, rho0.data(), F.data(), fixed.data(),
                                   (int64_t)fixed.size(), rho_ref.data(), c_ref.data(), v_ref.data(), d_ref.data(),
                                   cg.data(), &conv);
    EXPECT(n_ref == iters, "oracle ran");
    // oracle densities are C-order (x, y, z), the wrapper's x fastest
    auto xfast = [&](const std::vector<double> &c) {
        std::vector<double> o((size_t)nel);
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k)
                    o[(size_t)(((int64_t)k * ny + j) * nx + i)] = c[(size_t)(((int64_t)i * ny + j) * nz + k)];
        return o;
    };
    const std::vector<double> ref_x = xfast(rho_ref);

    auto compare = [&](const gt::OptimizationResult &r, const char *what) {
        EXPECT(r.iterations == iters && (int)r.compliance_history.size() == iters, what);
        double cmax = 0.0, dmax = 0.0;
        for (int i = 0; i < iters && i < (int)r.compliance_history.size(); ++i)
            cmax = std::fmax(cmax, std::fabs(r.compliance_history[i] - c_ref[i]) / c_ref[i]);
        for (int64_t e = 0; e < nel; ++e) dmax = std::fmax(dmax, std::fabs(r.final_density[(size_t)e] - ref_x[(size_t)e]));
        std::printf("%s: compliance rel err %.2e, density max-abs %.2e\n", what, cmax, dmax);
        EXPECT(cmax <= 1e-6, "compliance within 1e-6 of the oracle");
        EXPECT(dmax <= 1e-4, "densities within 1e-4 of the oracle");
    };

    // run() in one device call
    const gt::OptimizationResult a = opt.run(std::vector<double>(), F, fixed);  // wrong size -> vf everywhere
    compare(a, "run");
    // run() with a callback that sees every iteration
    int seen = 0;
    const gt::OptimizationResult b =
        opt.run(std::vector<double>((size_t)nel, 0.3), F, fixed,
                [&](int it, const std::vector<double> &d, const gt::IterationResult &r) {
                    EXPECT(it == seen && d.size() == (size_t)nel && r.compliance > 0.0, "callback arguments");
                    ++seen;
                    return true;
                });
    EXPECT(seen == iters, "callback every iteration");
    compare(b, "run+callback");
    // a callback that stops early
    const gt::OptimizationResult c = opt.run(std::vector<double>((size_t)nel, 0.3), F, fixed,
                                             [](int it, const std::vector<double> &, const gt::IterationResult &) {
                                                 return it < 2;
                                             });
    EXPECT(c.iterations == 3 && !c.converged, "callback stop");
    // runIteration continues the loop on the returned density
    std::vector<double> rho((size_t)nel, 0.3);
    std::vector<double> hist;
    for (int i = 0; i < iters; ++i) hist.push_back(opt.runIteration(rho, F, fixed).compliance);
    gt::OptimizationResult d;
    d.iterations = iters;
    d.compliance_history = hist;
    d.final_density = rho;
    compare(d, "runIteration");
    // the engine knobs: host-driven loop and FP64 residuals give the oracle's answers too
    opt.setDeviceLoop(false);
    opt.setResidualArithmetic(AM_RESID_FP64);
    compare(opt.run(std::vector<double>((size_t)nel, 0.3), F, fixed), "run (host loop, FP64 residuals)");
    opt.setDeviceLoop(true);
    opt.setResidualArithmetic(AM_RESID_DOUBLE_FLOAT);
    EXPECT(throws<std::invalid_argument>([&] { opt.setResidualArithmetic(9); }),
           "an unknown residual mode is std::invalid_argument");
    // solve(): reference tolerance semantics
    auto sol = opt.solve(std::vector<double>((size_t)nel, 0.5), F, fixed);
    EXPECT(sol.second.converged && sol.second.residual <= 1e-10, "solve converged");
    EXPECT(sol.first.size() == F.size(), "solve size");
    // error mapping on a live device
    std::vector<int64_t> bad = fixed;
    bad.push_back((int64_t)F.size() + 7);
    EXPECT(throws<std::out_of_range>([&] { opt.solve(std::vector<double>((size_t)nel, 0.5), F, bad); }),
           "a DOF outside the grid is std::out_of_range");
    EXPECT(throws<std::invalid_argument>([&] { opt.solve(std::vector<double>((size_t)nel, 0.5), std::vector<double>(5), fixed); }),
           "a force vector of the wrong size is std::invalid_argument");
    return failures;
}

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "cpu";
    const int f = mode == "gpu" ? gpu_checks() : cpu_checks();
    std::printf("%s checks: %d failure(s)\n", mode.c_str(), f);
    return f == 0 ? 0 : 1;
}
