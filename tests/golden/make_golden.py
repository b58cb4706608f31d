"""Generate the golden fixtures that pin the oracle to the reference.

Run once in a container where the reference project is checked out:

    python tests/golden/make_golden.py /path/to/reference

It imports the reference's own Python package (``src.am.numerical``,
``src.am.core``) and records its outputs, and copies the recorded outputs of
the reference's C++ engine run (``data/cpp_test_run``) together with the
inputs of that run (restated from ``cpp_engine/src/am_topopt.cpp:98-334``:
bracket grid, eyelet load vector, base constraint).  The fixtures are written
next to this file as ``.npz``; tests never need the reference checkout.
"""
from __future__ import annotations

import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def cpp_bracket(res, sx=120.0, sy=60.0, sz=80.0, base_t=5.0, hole_d=8.0, hole_off=15.0,
                eye_d=12.0, eye_off=4.0, eye_zoff=15.0, eye_h=20.0):
    """BracketDomain of am_topopt.cpp:98-239 as a physical (nx,ny,nz) int8 grid."""
    nx, ny, nz = int(sx / res), int(sy / res), int(sz / res)
    g = np.zeros((nx, ny, nz), np.int8)
    base_z = max(1, int(base_t / res))
    g[:, :, 0:min(base_z, nz)] = 1

    def cyl(cx, cy, z0, rad, h, val):
        for i in range(max(0, int(cx - rad - 1)), min(nx, int(cx + rad + 2))):
            for j in range(max(0, int(cy - rad - 1)), min(ny, int(cy + rad + 2))):
                di, dj = i - cx, j - cy
                if di * di + dj * dj <= rad * rad:
                    for k in range(z0, min(nz, z0 + h)):
                        if val == -1:
                            g[i, j, k] = -1
                        elif g[i, j, k] != -1:
                            g[i, j, k] = 1

    hr = hole_d / 2 / res
    hox, hoy = int(hole_off / res), int(hole_off / res)
    for hx, hy in [(hox, hoy), (nx - hox, hoy), (hox, ny - hoy), (nx - hox, ny - hoy)]:
        cyl(hx, hy, 0, hr, base_z, -1)
    ezo = int(eye_zoff / res)
    eh = max(1, int(eye_h / res))
    ezc = nz - ezo
    ex, ey = nx // 2, ny // 2
    z_start = max(0, ezc - eh // 2)
    z_end = min(nz, z_start + eh)
    if z_end - z_start > 0:
        cyl(ex, ey, z_start, (eye_d / 2 + eye_off) / res, z_end - z_start, 1)
        cyl(ex, ey, z_start, eye_d / 2 / res, z_end - z_start, -1)
    if z_start > base_z:
        cyl(ex, ey, base_z, (eye_d / 2 + eye_off) / res, z_start - base_z, 1)
    return g


def cpp_force(nx, ny, nz, res, load=15000.0, eye_d=12.0, eye_off=4.0, eye_zoff=15.0, eye_h=20.0):
    """createForceVector of am_topopt.cpp:248-314."""
    F = np.zeros(3 * (nx + 1) * (ny + 1) * (nz + 1))
    ezo = int(eye_zoff / res)
    eh = max(1, int(eye_h / res))
    z_start = max(0, nz - ezo - eh // 2)
    z_end = min(nz, z_start + eh)
    ez = max(1, min(nz - 1, (z_start + z_end) // 2))
    ex, ey = nx // 2, ny // 2
    ir = eye_d / 2 + res * 1.25
    orr = eye_d / 2 + eye_off
    if ir >= orr:
        ir = eye_d / 2 + eye_off * 0.5
    ir /= res
    orr /= res
    nodes = []
    s = int(orr) + 2
    for i in range(max(0, ex - s), min(nx, ex + s) + 1):
        for j in range(max(0, ey - s), min(ny, ey + s) + 1):
            d = math.sqrt((i - ex) ** 2 + (j - ey) ** 2)
            if ir < d <= orr:
                nodes.append(i * (ny + 1) * (nz + 1) + j * (nz + 1) + ez)
    if not nodes:
        nodes.append(ex * (ny + 1) * (nz + 1) + ey * (nz + 1) + ez)
    for n in nodes:
        F[3 * n + 2] = -load / len(nodes)
    return F


def cpp_fixed(nx, ny, nz):
    """createFixedDofs of am_topopt.cpp:319-334 (all nodes with k = 0)."""
    out = []
    for i in range(nx + 1):
        for j in range(ny + 1):
            n = i * (ny + 1) * (nz + 1) + j * (nz + 1)
            out += [3 * n, 3 * n + 1, 3 * n + 2]
    return np.array(out, np.int64)


def main(ref):
    sys.path.insert(0, ref)
    from src.am.core.geometry import VoxelDomain, create_bracket_domain
    from src.am.core.loads import (DOF, BoundaryCondition, DistributedLoad, LoadCase, PointLoad,
                                   create_brk_a_01_static_case_1)
    from src.am.numerical import fem
    from src.am.numerical.topopt import SIMPOptimizer, SIMPParams

    mat1 = fem.MaterialProperties(E=1.0, nu=0.3)
    out = {}

    # --- A1 element stiffness (fem.py:43-135)
    out["ke_E1_nu03_h1"] = fem.get_element_stiffness_matrix(1.0, mat1)
    out["ke_ti_h2mm"] = fem.get_element_stiffness_matrix(0.002, fem.MaterialProperties())

    # --- A2 DOF map (fem.py:138-172)
    shape = (5, 4, 3)
    out["dofs_shape"] = np.array(shape)
    out["dofs_elems"] = np.array([(0, 0, 0), (1, 2, 0), (4, 3, 2), (2, 1, 1)])
    out["dofs"] = np.stack([fem.get_element_dof_indices(tuple(e), shape) for e in out["dofs_elems"]])

    # --- A3py assembled K and K*u on a mixed grid (fem.py:175-248)
    rng = np.random.default_rng(0)
    shape = (6, 5, 4)
    grid = rng.integers(-1, 2, size=shape).astype(np.int8)
    grid[0] = 0
    rho = rng.uniform(0.01, 1.0, size=shape)
    K = fem.assemble_global_stiffness(grid, rho, 1.0, mat1, 3.0, 1e-9)
    u = rng.normal(size=K.shape[0])
    out.update(ku_shape=np.array(shape), ku_grid=grid, ku_rho=rho, ku_u=u, ku_y=K @ u,
               ku_nnz=np.array(K.nnz))

    # --- A4py solve + compliance on a cantilever with void (orphan DOFs), fem.py:251-383
    shape = (7, 3, 4)
    grid = np.zeros(shape, np.int8)
    grid[3:5, :, 2:] = -1          # void block -> orphan nodes in its interior/top
    grid[6, :, :] = 1              # solid end cap
    rho = rng.uniform(0.2, 1.0, size=shape)
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    base = [j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)]
    lc = LoadCase(name="t", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                  point_loads=[PointLoad(node_index=nx * (ny + 1) * (nz + 1) + 1 * (nz + 1) + 2,
                                         force_vector=np.array([0.1, 0.2, -1.0]))])
    F = lc.get_force_vector(N)
    fixed = lc.get_constrained_dofs()
    K = fem.assemble_global_stiffness(grid, rho, 1.0, mat1, 3.0, 1e-9)
    usol = fem.solve_fem(K, F, fixed, method="direct")
    c, ce = fem.compute_element_compliance(usol, grid, rho, 1.0, mat1, 3.0, 1e-9)
    out.update(solve_shape=np.array(shape), solve_grid=grid, solve_rho=rho, solve_F=F,
               solve_fixed=fixed, solve_u=usol, solve_c=np.array(c), solve_ce=ce)

    # --- A6/A7py/A8py on the optimizer object (topopt.py:135-264)
    shape = (7, 5, 4)
    dom = VoxelDomain(grid=np.zeros(shape, np.int8), resolution_mm=1000.0)
    dom.grid[0, 0, :] = 1
    dom.grid[6, 4, 3] = -1
    for r in (1.5, 2.5):
        opt = SIMPOptimizer(dom, [lc], mat1, SIMPParams(filter_radius=r), verbose=False)
        x = rng.uniform(0.0, 1.0, size=shape)
        out[f"filter_py_r{r}_x"] = x
        out[f"filter_py_r{r}_y"] = opt._apply_filter(x)
    opt = SIMPOptimizer(dom, [lc], mat1, SIMPParams(volume_fraction=0.3, move_limit=0.2), verbose=False)
    dens = rng.uniform(0.05, 0.9, size=shape)
    dc = -rng.uniform(0.0, 5.0, size=shape) * dens
    out.update(oc_py_shape=np.array(shape), oc_py_grid=dom.grid, oc_py_rho=dens, oc_py_dc=dc,
               oc_py_out=opt._oc_update(dens, dc, np.ones_like(dens)))
    # sensitivities on a solved field of the same grid size
    n = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    uu = rng.normal(size=3 * n)
    out.update(sens_u=uu, sens_rho=dens, sens_dc=opt._compute_sensitivities(dens, uu))

    # --- A9py: 8x4x4 Python SIMP, 5 iterations (topopt.py:266-411)
    shape = (8, 4, 4)
    nx, ny, nz = shape
    dom = VoxelDomain(grid=np.zeros(shape, np.int8), resolution_mm=1000.0)
    base = [j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)]
    load_node = nx * (ny + 1) * (nz + 1) + (ny // 2) * (nz + 1) + nz // 2
    lc = LoadCase(name="cantilever", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                  point_loads=[PointLoad(node_index=load_node, force_vector=np.array([0.0, 0.0, -1.0]))])
    prm = SIMPParams(volume_fraction=0.3, filter_radius=1.5, max_iterations=5, convergence_tol=0.0)
    res = SIMPOptimizer(dom, [lc], mat1, prm, verbose=False).run()
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    out.update(simp_py_shape=np.array(shape), simp_py_F=lc.get_force_vector(N),
               simp_py_fixed=lc.get_constrained_dofs(), simp_py_density=res.density,
               simp_py_compliance=np.array(res.compliance_history),
               simp_py_volume=np.array(res.volume_history))

    # --- two load cases (multi-load-case sum, topopt.py:309-360), 3 iterations
    lc2 = LoadCase(name="side", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                   distributed_loads=[DistributedLoad(node_indices=np.array([load_node, load_node - 1]),
                                                      total_force=np.array([0.0, 0.5, 0.0]))])
    prm = SIMPParams(volume_fraction=0.35, filter_radius=1.5, max_iterations=3, convergence_tol=0.0)
    res = SIMPOptimizer(dom, [lc, lc2], mat1, prm, verbose=False).run()
    out.update(simp_py2_F2=lc2.get_force_vector(N), simp_py2_density=res.density,
               simp_py2_compliance=np.array(res.compliance_history),
               simp_py2_volume=np.array(res.volume_history))

    # --- cfg-1 geometry at uniform rho = 0.3 (48x24x12, clamp i=0, -1 z line load)
    shape = (48, 24, 12)
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    base = [j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)]
    line = [nx * (ny + 1) * (nz + 1) + j * (nz + 1) + nz // 2 for j in range(ny + 1)]
    lc = LoadCase(name="cfg1", boundary_conditions=[BoundaryCondition(node_indices=np.array(base))],
                  distributed_loads=[DistributedLoad(node_indices=np.array(line),
                                                     total_force=np.array([0.0, 0.0, -1.0]))])
    grid = np.zeros(shape, np.int8)
    t0 = time.time()
    K = fem.assemble_global_stiffness(grid, np.full(shape, 0.3), 1.0, mat1, 3.0, 1e-9)
    F = lc.get_force_vector(N)
    usol = fem.solve_fem(K, F, lc.get_constrained_dofs(), method="direct")
    print(f"cfg1 uniform solve {time.time() - t0:.1f}s")
    out.update(cfg1_F=F, cfg1_fixed=lc.get_constrained_dofs(), cfg1_nnz=np.array(K.nnz),
               cfg1_compliance=np.array(float(F @ usol)), cfg1_u_norm=np.array(np.linalg.norm(usol)),
               cfg1_u_loadnodes=usol[3 * np.array(line) + 2])

    # --- notebook C++ debug run (visualize_results.ipynb cell 23): inputs + printed outputs.
    res_mm = 12.0
    dom = create_bracket_domain(size_mm=(120, 60, 80), resolution_mm=res_mm)
    lc = create_brk_a_01_static_case_1(dom.shape, res_mm)
    nx, ny, nz = dom.shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    out.update(nb_grid=dom.grid, nb_F=lc.get_force_vector(N), nb_fixed=lc.get_constrained_dofs(),
               nb_compliance=np.array([1.440006209452606, 2.5182595401031365, 1.971215740189977]),
               nb_volume=np.array([0.3135, 0.29999973003107716, 0.2999996582296991]))

    # --- reference C++ engine run data/cpp_test_run (am_topopt --resolution 4 --iterations 5)
    g = cpp_bracket(4.0)
    nx, ny, nz = g.shape
    hist = np.loadtxt(os.path.join(ref, "data/cpp_test_run/history.csv"), delimiter=",", skiprows=1)
    out.update(cpprun_grid=g, cpprun_F=cpp_force(nx, ny, nz, 4.0), cpprun_fixed=cpp_fixed(nx, ny, nz),
               cpprun_compliance=hist[:, 1], cpprun_volume=hist[:, 2],
               cpprun_density=np.load(os.path.join(ref, "data/cpp_test_run/density_field.npy")))

    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_golden.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
