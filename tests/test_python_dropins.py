"""The Python surface a caller of the reference uses, end to end:

* ``core`` input types (VoxelDomain, LoadCase, BoundaryCondition, PointLoad,
  DistributedLoad; src/am/core/geometry.py:16-76, loads.py:23-156) build the
  reference's own force vectors and constrained-DOF lists (golden fixtures);
* ``numerical.topopt.SIMPOptimizer`` (topopt.py:84-411) reproduces the
  reference's recorded SIMP histories from those inputs;
* ``numerical.fem`` solves and element compliances match the reference's
  direct solve with orphan DOFs (fem.py:251-383);
* ``cpp.CPPTopologyOptimizer`` (the notebook's missing binding, cells 23-24)
  replays the reference C++ engine's recorded run data/cpp_test_run with the
  engine's assembly index, and agrees with the FP64 oracle with the consistent
  one."""
import numpy as np
import pytest

import oracle as O
from am_ml_suite_gb300 import _native as nat
from am_ml_suite_gb300.core import BoundaryCondition, DistributedLoad, LoadCase, PointLoad, VoxelDomain


def _simp_py_inputs(golden):
    shape = tuple(int(v) for v in golden["simp_py_shape"])
    nx, ny, nz = shape
    base = [j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)]
    load_node = nx * (ny + 1) * (nz + 1) + (ny // 2) * (nz + 1) + nz // 2
    lc = LoadCase(name="cantilever", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                  point_loads=[PointLoad(node_index=load_node, force_vector=np.array([0.0, 0.0, -1.0]))])
    lc2 = LoadCase(name="side", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                   distributed_loads=[DistributedLoad(node_indices=np.array([load_node, load_node - 1]),
                                                      total_force=np.array([0.0, 0.5, 0.0]))])
    dom = VoxelDomain(grid=np.zeros(shape, np.int8), resolution_mm=1000.0)
    return shape, dom, lc, lc2


def test_core_types_build_the_reference_loads(golden):
    shape, dom, lc, lc2 = _simp_py_inputs(golden)
    N = 3 * int(np.prod(np.array(shape) + 1))
    assert np.array_equal(lc.get_force_vector(N), golden["simp_py_F"])
    assert np.array_equal(lc.get_constrained_dofs(), golden["simp_py_fixed"])
    assert np.array_equal(lc2.get_force_vector(N), golden["simp_py2_F2"])
    assert dom.n_elements == int(np.prod(shape)) and dom.n_design == dom.n_elements


@pytest.mark.gpu
def test_simp_optimizer_reproduces_reference_history(golden):
    from am_ml_suite_gb300.numerical.fem import MaterialProperties
    from am_ml_suite_gb300.numerical.topopt import SIMPOptimizer, SIMPParams

    shape, dom, lc, lc2 = _simp_py_inputs(golden)
    mat = MaterialProperties(E=1.0, nu=0.3)
    seen = []
    prm = SIMPParams(volume_fraction=0.3, filter_radius=1.5, max_iterations=5, convergence_tol=0.0, cg_tol=1e-11)
    res = SIMPOptimizer(dom, [lc], mat, prm, verbose=False).run(callback=lambda i, d, c: seen.append((i, c)))
    assert res.iterations == 5 and not res.converged
    assert np.allclose(res.compliance_history, golden["simp_py_compliance"], rtol=1e-8)
    assert np.allclose(res.volume_history, golden["simp_py_volume"], rtol=1e-10)
    assert res.density.shape == shape
    assert np.abs(res.density - golden["simp_py_density"]).max() < 1e-8
    assert [i for i, _ in seen] == list(range(5))
    # two load cases (topopt.py:309-360)
    prm = SIMPParams(volume_fraction=0.35, filter_radius=1.5, max_iterations=3, convergence_tol=0.0, cg_tol=1e-11)
    res = SIMPOptimizer(dom, [lc, lc2], mat, prm, verbose=False).run()
    assert np.allclose(res.compliance_history, golden["simp_py2_compliance"], rtol=1e-8)
    assert np.abs(res.density - golden["simp_py2_density"]).max() < 1e-8


@pytest.mark.gpu
def test_fem_functions_match_reference_direct_solve(golden):
    from am_ml_suite_gb300.numerical import fem

    mat = fem.MaterialProperties(E=1.0, nu=0.3)
    grid, rho = golden["solve_grid"], golden["solve_rho"]
    u = fem.solve_fem(grid, rho, golden["solve_F"], golden["solve_fixed"], 1.0, mat, tol=1e-12)
    ref = golden["solve_u"]
    assert np.linalg.norm(u - ref) / np.linalg.norm(ref) <= 1e-9
    c, ce = fem.compute_element_compliance(u, grid, rho, 1.0, mat)
    assert c == pytest.approx(float(golden["solve_c"]), rel=1e-9)
    assert np.abs(ce - golden["solve_ce"]).max() <= 1e-9 * np.abs(golden["solve_ce"]).max()
    ke = fem.get_element_stiffness_matrix(1.0, mat)
    assert np.abs(ke - golden["ke_E1_nu03_h1"]).max() < 1e-15
    with pytest.raises(ValueError):
        fem.solve_fem(grid, rho, np.full_like(golden["solve_F"], np.nan), golden["solve_fixed"], 1.0, mat)


def _xfast(c_order, shape):
    return np.asarray(c_order).reshape(shape).transpose(2, 1, 0).ravel()


@pytest.mark.gpu
def test_cpp_surface_replays_the_reference_engine_run(golden):
    """data/cpp_test_run: am_topopt at 4 mm (30x15x20 bracket), Ti6Al4V, vf 0.25,
    filter 3.5, move 0.1, rho_min 1e-4, E_min 1e-6, 5 iterations.  With the
    engine's assembly index the run is the reference's own: compliance history
    to its printed digits, final densities to 1e-6."""
    from am_ml_suite_gb300 import cpp

    g = golden["cpprun_grid"]
    shape = g.shape
    rho0 = _xfast(np.where(g == 0, 0.25, np.where(g == 1, 1.0, 1e-4)), shape)
    cfg = cpp.SIMPConfig(volume_fraction=0.25, max_iterations=5, filter_radius=3.5, E_min=1e-6, move_limit=0.1,
                         rho_min=1e-4, convergence_tol=0.01, cg_tol=1e-10, verbose=False, precision=nat.PREC_FP64,
                         reference_assembly_index=True)
    opt = cpp.CPPTopologyOptimizer(*shape, 0.004, cpp.MaterialProperties(), cfg)
    assert cpp.is_available() and cpp.get_max_threads() > 0
    res = opt.run(list(rho0), golden["cpprun_F"], golden["cpprun_fixed"])
    assert res.iterations == 5
    assert np.allclose(res.compliance_history, golden["cpprun_compliance"], rtol=2e-6)
    assert np.allclose(res.volume_history, golden["cpprun_volume"], rtol=4e-6)
    # the reference writes the x-fastest vector as a C-order (nx, ny, nz) array
    dens = np.asarray(res.final_density).reshape(shape[2], shape[1], shape[0]).transpose(2, 1, 0)
    assert np.abs(dens - golden["cpprun_density"]).max() < 1e-6


@pytest.mark.gpu
def test_cpp_surface_consistent_index_matches_oracle(golden):
    from am_ml_suite_gb300 import cpp

    g = golden["cpprun_grid"]
    shape = g.shape
    rho0_c = np.where(g == 0, 0.25, np.where(g == 1, 1.0, 1e-4))
    prm = O.make_params(volume_fraction=0.25, max_iterations=4, filter_radius=3.5, E_min=1e-6, move_limit=0.1,
                        rho_min=1e-4, convergence_tol=0.0, cg_tol=1e-12, warm_start=1)
    ref = O.simp_cpp(shape, 0.004, 113.8e9, 0.342, prm, rho0_c, golden["cpprun_F"], golden["cpprun_fixed"])
    cfg = cpp.SIMPConfig(volume_fraction=0.25, max_iterations=4, filter_radius=3.5, E_min=1e-6, move_limit=0.1,
                         rho_min=1e-4, convergence_tol=0.0, cg_tol=1e-10, verbose=False)
    opt = cpp.CPPTopologyOptimizer(*shape, 0.004, cpp.MaterialProperties(), cfg)
    calls = []
    res = opt.run(_xfast(rho0_c, shape), golden["cpprun_F"], golden["cpprun_fixed"],
                  callback=lambda it, d, r: calls.append(it) or True)
    assert calls == [0, 1, 2, 3]
    rel = np.abs(np.array(res.compliance_history) - ref["compliance"]) / ref["compliance"]
    assert rel.max() <= 1e-6, rel
    assert np.abs(np.asarray(res.final_density) - _xfast(ref["density"], shape)).max() <= 1e-4
    # run_iteration updates the caller's list in place
    dens = list(_xfast(rho0_c, shape))
    r = opt.run_iteration(dens, golden["cpprun_F"], golden["cpprun_fixed"])
    assert r.compliance == pytest.approx(float(ref["compliance"][0]), rel=1e-6)
    assert np.abs(np.asarray(dens) - _xfast(rho0_c, shape)).max() > 0.0
