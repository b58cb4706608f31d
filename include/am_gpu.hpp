/*
 * am_gpu.hpp -- header-only C++ wrapper of the C ABI (am_gpu.h) with the class
 * and struct names of the reference's C++ engine, so a caller of
 *
 *   am::topopt::TopologyOptimizer   cpp_engine/include/am/topology_optimizer.hpp:120-279
 *   am::topopt::SIMPConfig          topology_optimizer.hpp:49-59
 *   am::topopt::IterationResult     topology_optimizer.hpp:65-74
 *   am::topopt::OptimizationResult  topology_optimizer.hpp:80-87
 *   am::topopt::IterationCallback   topology_optimizer.hpp:98-102
 *   am::fem::SolveStats             cpp_engine/include/am/linear_solver.hpp:48-56
 *   am::fem::MaterialProperties     cpp_engine/include/am/element_kernel.hpp:61-76
 *
 * switches by changing its include and namespace (am::gpu::topopt / am::gpu::fem).
 * Status codes become the reference's exceptions: AM_ERR_INVALID_ARG and
 * AM_ERR_SIZE_MISMATCH std::invalid_argument (global_assembler.cpp:73-83,
 * linear_solver.cpp:59-63), AM_ERR_DOF_OUT_OF_RANGE std::out_of_range
 * (linear_solver.cpp:69-73), AM_ERR_OOM std::bad_alloc, every other failure
 * std::runtime_error.  A solve that does not reach its tolerance is not an
 * exception, as in the reference (linear_solver.cpp:148-152, 175-180): it shows
 * in the statistics.
 *
 * Densities are the reference optimizer's vectors: element (ix, iy, iz) at
 * iz*nx*ny + iy*nx + ix (topology_optimizer.hpp:218-232).  Forces are any
 * contiguous container of doubles with data() and size() (std::vector, or the
 * reference's Eigen::VectorXd without including Eigen here) in the reference DOF
 * order 3*(i*(ny+1)*(nz+1) + j*(nz+1) + k) + d.  Device memory lives in the
 * object; one object is used from one host thread at a time.
 */
#ifndef AM_GPU_HPP
#define AM_GPU_HPP

#include <chrono>
#include <cstdint>
#include <cstring>
#include <functional>
#include <iostream>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "am_gpu.h"

namespace am {
namespace gpu {

namespace detail {

[[noreturn]] inline void raise(am_status s, const char *where) {
    std::string msg = std::string(where) + ": " + am_status_string(s);
    const char *d = am_last_error();
    if (d && *d) msg += std::string(": ") + d;
    switch (s) {
        case AM_ERR_INVALID_ARG:
        case AM_ERR_SIZE_MISMATCH: throw std::invalid_argument(msg);
        case AM_ERR_DOF_OUT_OF_RANGE: throw std::out_of_range(msg);
        case AM_ERR_OOM: throw std::bad_alloc();
        default: throw std::runtime_error(msg);
    }
}

inline void check(am_status s, const char *where) {
    if (s != AM_OK) raise(s, where);
}

}  // namespace detail

namespace fem {

/* Isotropic material (element_kernel.hpp:61-76); rho is carried for parity and unused. */
struct MaterialProperties {
    double E, nu, rho;
    static constexpr double DEFAULT_E = 113.8e9;
    static constexpr double DEFAULT_NU = 0.342;
    static constexpr double DEFAULT_RHO = 4430.0;
    MaterialProperties(double E_ = DEFAULT_E, double nu_ = DEFAULT_NU, double rho_ = DEFAULT_RHO)
        : E(E_), nu(nu_), rho(rho_) {}
};

/* linear_solver.hpp:48-56, plus the FP32/FP64 split of the mixed solver. */
struct SolveStats {
    int iterations = 0;          /* PCG iterations (inner ones in mixed precision) */
    double residual = 0.0;       /* final ||f - K u|| / ||f||, FP64 */
    double solve_time_s = 0.0;
    double bc_time_s = 0.0;      /* constraints are applied by masking: always 0 */
    bool converged = false;
    double max_displacement = 0.0;
    double min_displacement = 0.0;
    int outer_iterations = 0;    /* FP64 residual replacements / outer flexible-CG steps */
};

}  // namespace fem

namespace topopt {

/* SIMPConfig (topology_optimizer.hpp:49-59) with the reference's defaults, plus
 * the solver choices of this engine.  cg_tol defaults to the tolerance the
 * reference optimizer gives its solver (topology_optimizer.cpp:36). */
struct SIMPConfig {
    double volume_fraction = 0.25;
    double penalty = 3.0;
    double filter_radius = 2.0;
    double move_limit = 0.2;
    double rho_min = 0.01;
    double E_min = 1e-6;
    int max_iterations = 100;
    double convergence_tol = 0.01;
    bool verbose = true;
    /* GPU solver */
    int precision = AM_PREC_MIXED;          /* AM_PREC_MIXED or AM_PREC_FP64 */
    int preconditioner = AM_PRECOND_JACOBI; /* AM_PRECOND_JACOBI / _MG / _LEARNED */
    double cg_tol = 1e-6;
    int cg_max_iterations = 200000;
    bool warm_start = true;
    /* true: the element stiffness scales read the density vector with the
     * reference assembler's z-fastest index (global_assembler.hpp:162-164), as the
     * reference engine does, to replay its runs */
    bool reference_assembly_index = false;
};

/* topology_optimizer.hpp:65-74 */
struct IterationResult {
    double compliance = 0.0;
    double volume_fraction = 0.0;
    double max_density_change = 0.0;
    int solver_iterations = 0;
    double assembly_time_s = 0.0;
    double solve_time_s = 0.0;
    double sensitivity_time_s = 0.0;
    double update_time_s = 0.0;
    double solver_residual = 0.0;  /* FP64 relative residual of the accepted solve */
};

/* topology_optimizer.hpp:80-87 */
struct OptimizationResult {
    std::vector<double> final_density;
    std::vector<double> compliance_history;
    std::vector<double> volume_history;
    int iterations = 0;
    bool converged = false;
    double elapsed_time_s = 0.0;
};

/* topology_optimizer.hpp:98-102: false stops the run after this iteration. */
using IterationCallback =
    std::function<bool(int iteration, const std::vector<double> &density, const IterationResult &result)>;

/* TopologyOptimizer (topology_optimizer.hpp:120-279) on one GPU. */
class TopologyOptimizer {
public:
    TopologyOptimizer(int nx, int ny, int nz, double element_size, const fem::MaterialProperties &material,
                      const SIMPConfig &config = SIMPConfig())
        : nx_(nx), ny_(ny), nz_(nz), config_(config) {
        detail::check(am_problem_create(nx, ny, nz, element_size, material.E, material.nu, nullptr,
                                        AM_LAYOUT_XFASTEST, &p_),
                      "TopologyOptimizer");
        n_elements_ = (int64_t)nx * ny * nz;
        n_dofs_ = 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    }
    ~TopologyOptimizer() {
        if (p_) am_problem_destroy(p_);
    }
    TopologyOptimizer(const TopologyOptimizer &) = delete;
    TopologyOptimizer &operator=(const TopologyOptimizer &) = delete;
    TopologyOptimizer(TopologyOptimizer &&o) noexcept { *this = std::move(o); }
    TopologyOptimizer &operator=(TopologyOptimizer &&o) noexcept {
        if (this != &o) {
            if (p_) am_problem_destroy(p_);
            p_ = o.p_;
            o.p_ = nullptr;
            nx_ = o.nx_; ny_ = o.ny_; nz_ = o.nz_;
            n_elements_ = o.n_elements_;
            n_dofs_ = o.n_dofs_;
            config_ = o.config_;
            forces_ = std::move(o.forces_);
            fixed_ = std::move(o.fixed_);
            begun_ = o.begun_;
            last_density_ = std::move(o.last_density_);
        }
        return *this;
    }

    /* Engine knobs with no reference counterpart: who drives an inner solve's loop
     * (am_problem_set_device_loop) and the arithmetic of the mixed solvers'
     * residuals (am_problem_set_residual_arithmetic: AM_RESID_DOUBLE_FLOAT or
     * AM_RESID_FP64). */
    void setDeviceLoop(bool on) { detail::check(am_problem_set_device_loop(p_, on ? 1 : 0), "setDeviceLoop"); }
    void setResidualArithmetic(int mode) {
        detail::check(am_problem_set_residual_arithmetic(p_, mode), "setResidualArithmetic");
    }

    /* One iteration (runIteration, topology_optimizer.cpp:294-384) on `density`,
     * which is updated in place.  The first call starts the loop on the device
     * (design mask from this density, as run() does); later calls continue it
     * when `density` is what the previous call returned, and restart it from
     * `density` otherwise. */
    template <class Vec>
    IterationResult runIteration(std::vector<double> &density, const Vec &forces,
                                 const std::vector<int64_t> &fixed_dofs) {
        if (density.size() != (size_t)n_elements_)
            throw std::invalid_argument("runIteration: density has " + std::to_string(density.size()) +
                                        " entries, the grid " + std::to_string(n_elements_));
        set_loads(forces, fixed_dofs);
        if (!begun_ || density != last_density_) {
            const am_simp_config c = to_c(config_, config_.max_iterations > 0 ? config_.max_iterations : 1);
            detail::check(am_simp_begin(p_, &c, density.data()), "runIteration");
            begun_ = true;
        }
        am_iteration_result r{};
        detail::check(am_simp_step(p_, &r), "runIteration");
        detail::check(am_simp_get_density(p_, density.data()), "runIteration");
        last_density_ = density;
        return from_c(r);
    }

    /* The whole loop (run, topology_optimizer.cpp:391-520): stops after
     * max_iterations, when max |change| < convergence_tol, or when the callback
     * returns false.  Like the reference, a density of the wrong size is replaced
     * by volume_fraction everywhere.  Without a callback the loop runs in one
     * call on the device (am_simp_run); with one, the density is read back every
     * iteration for it. */
    template <class Vec>
    OptimizationResult run(std::vector<double> initial_density, const Vec &forces,
                           const std::vector<int64_t> &fixed_dofs, IterationCallback callback = nullptr) {
        const auto t0 = std::chrono::steady_clock::now();
        if (initial_density.size() != (size_t)n_elements_) initial_density.assign((size_t)n_elements_, config_.volume_fraction);
        set_loads(forces, fixed_dofs);
        OptimizationResult out;
        const int m = config_.max_iterations > 0 ? config_.max_iterations : 0;
        if (m == 0) {
            out.final_density = std::move(initial_density);
            return out;
        }
        const am_simp_config c = to_c(config_, m);
        if (!callback) {
            out.final_density.assign((size_t)n_elements_, 0.0);
            out.compliance_history.assign((size_t)m, 0.0);
            out.volume_history.assign((size_t)m, 0.0);
            int its = 0, conv = 0;
            detail::check(am_simp_run(p_, &c, initial_density.data(), out.final_density.data(),
                                      out.compliance_history.data(), out.volume_history.data(), nullptr, &its,
                                      &conv),
                          "run");
            out.compliance_history.resize((size_t)its);
            out.volume_history.resize((size_t)its);
            out.iterations = its;
            out.converged = conv != 0;
        } else {
            std::vector<double> density = std::move(initial_density);
            detail::check(am_simp_begin(p_, &c, density.data()), "run");
            for (int it = 0; it < m; ++it) {
                am_iteration_result r{};
                detail::check(am_simp_step(p_, &r), "run");
                detail::check(am_simp_get_density(p_, density.data()), "run");
                const IterationResult ir = from_c(r);
                out.compliance_history.push_back(ir.compliance);
                out.volume_history.push_back(ir.volume_fraction);
                out.iterations = it + 1;
                if (!callback(it, density, ir)) break;
                if (ir.max_density_change < config_.convergence_tol) {
                    out.converged = true;
                    break;
                }
            }
            out.final_density = std::move(density);
        }
        begun_ = false;
        out.elapsed_time_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (config_.verbose)
            std::cout << "SIMP (GB300): " << out.iterations << " iterations, compliance "
                      << (out.compliance_history.empty() ? 0.0 : out.compliance_history.back()) << ", "
                      << out.elapsed_time_s << " s" << std::endl;
        return out;
    }

    /* K(density) u = forces with the constrained and orphan DOFs eliminated
     * (LinearSolver::solveWithBCs, linear_solver.cpp:186-203) to config().cg_tol. */
    template <class Vec>
    std::pair<std::vector<double>, fem::SolveStats> solve(const std::vector<double> &density, const Vec &forces,
                                                         const std::vector<int64_t> &fixed_dofs) {
        if (density.size() != (size_t)n_elements_) throw std::invalid_argument("solve: density size mismatch");
        set_loads(forces, fixed_dofs);
        const am_simp_config c = to_c(config_, 1);
        std::vector<double> u((size_t)n_dofs_, 0.0);
        am_solve_stats s{};
        detail::check(am_solve(p_, &c, density.data(), 0, u.data(), &s), "solve");
        fem::SolveStats st;
        st.iterations = s.iterations;
        st.residual = s.residual;
        st.solve_time_s = s.solve_time_s;
        st.converged = s.converged != 0;
        st.max_displacement = s.max_displacement;
        st.min_displacement = s.min_displacement;
        st.outer_iterations = s.outer_iterations;
        return {std::move(u), st};
    }

    int nx() const { return nx_; }
    int ny() const { return ny_; }
    int nz() const { return nz_; }
    int64_t numElements() const { return n_elements_; }
    int64_t numDofs() const { return n_dofs_; }
    const SIMPConfig &config() const { return config_; }
    SIMPConfig &config() { return config_; }
    am_problem *handle() { return p_; }

private:
    static am_simp_config to_c(const SIMPConfig &s, int max_iterations) {
        am_simp_config c;
        am_simp_config_default(&c, AM_VARIANT_CPP);
        c.volume_fraction = s.volume_fraction;
        c.penalty = s.penalty;
        c.filter_radius = s.filter_radius;
        c.move_limit = s.move_limit;
        c.rho_min = s.rho_min;
        c.E_min = s.E_min;
        c.convergence_tol = s.convergence_tol;
        c.max_iterations = max_iterations;
        c.precision = s.precision;
        c.preconditioner = s.preconditioner;
        c.cg_tol = s.cg_tol;
        c.cg_max_iterations = s.cg_max_iterations;
        c.warm_start = s.warm_start ? 1 : 0;
        c.cpp_assembly_index = s.reference_assembly_index ? 1 : 0;
        c.layout = AM_LAYOUT_XFASTEST;
        c.verbose = 0;
        return c;
    }
    static IterationResult from_c(const am_iteration_result &r) {
        IterationResult o;
        o.compliance = r.compliance;
        o.volume_fraction = r.volume_fraction;
        o.max_density_change = r.max_density_change;
        o.solver_iterations = r.solver_iterations;
        o.assembly_time_s = r.assembly_time_s;
        o.solve_time_s = r.solve_time_s;
        o.sensitivity_time_s = r.sensitivity_time_s;
        o.update_time_s = r.update_time_s;
        o.solver_residual = r.solver_residual;
        return o;
    }
    // uploads the load case when it differs from the one on the device
    template <class Vec>
    void set_loads(const Vec &forces, const std::vector<int64_t> &fixed) {
        const size_t n = (size_t)forces.size();
        if (n != (size_t)n_dofs_)
            throw std::invalid_argument("force vector has " + std::to_string(n) + " entries, the grid " +
                                        std::to_string(n_dofs_) + " DOFs");
        const double *f = forces.data();
        if (forces_.size() == n && fixed_ == fixed && std::memcmp(forces_.data(), f, n * sizeof(double)) == 0)
            return;
        const int64_t nf = (int64_t)fixed.size();
        detail::check(am_problem_set_loads(p_, 1, f, fixed.data(), &nf), "set_loads");
        forces_.assign(f, f + n);
        fixed_ = fixed;
        begun_ = false;
    }

    am_problem *p_ = nullptr;
    int nx_ = 0, ny_ = 0, nz_ = 0;
    int64_t n_elements_ = 0, n_dofs_ = 0;
    SIMPConfig config_;
    std::vector<double> forces_;
    std::vector<int64_t> fixed_;
    bool begun_ = false;
    std::vector<double> last_density_;
};

}  // namespace topopt
}  // namespace gpu
}  // namespace am

#endif  // AM_GPU_HPP
