"""Multigrid-preconditioned solves (AM_PRECOND_MG) through the C ABI against the
FP64 oracle: displacement within 1e-6 of a tight oracle solve, far fewer
iterations than Jacobi PCG, SIMP histories within the SIMP tolerances
(compliance 1e-6 relative, densities 1e-4), and grids that do not coarsen solve
on the Jacobi path."""
import numpy as np
import pytest

import oracle as O
from am_ml_suite_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _cantilever(shape):
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    fixed = (3 * base[:, None] + np.arange(3)).ravel()
    F = np.zeros(N)
    line = [nx * (ny + 1) * (nz + 1) + j * (nz + 1) + nz // 2 for j in range(ny + 1)]
    F[3 * np.array(line) + 2] = -1.0 / len(line)
    return F, fixed


def _smooth_density(shape, seed):
    """A SIMP-like field: a smooth random blend clipped to [0.01, 1], with void
    pockets (rho < rho_min: skipped by the C++ rule, orphaning their nodes)."""
    rng = np.random.default_rng(seed)
    x, y, z = np.meshgrid(*[np.linspace(0, 1, n) for n in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(6):
        k = rng.uniform(1, 4, size=3)
        f += rng.normal() * np.cos(np.pi * (k[0] * x + rng.random())) * np.cos(np.pi * (k[1] * y + rng.random())) \
            * np.cos(np.pi * (k[2] * z + rng.random()))
    rho = np.clip(0.5 + 0.5 * f / np.abs(f).max(), 0.01, 1.0)
    rho[f < -0.8 * np.abs(f).max()] = 1e-3
    return rho


@pytest.mark.parametrize("shape", [(32, 16, 16), (24, 12, 8), (48, 24, 24)])
def test_mg_solve_matches_oracle_in_few_iterations(shape):
    rho = _smooth_density(shape, sum(shape))
    F, fixed = _cantilever(shape)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    base = dict(E_min=1e-9, rho_min=0.01, cg_tol=1e-8, warm_start=0)
    u_mg, st_mg = p.solve(nat.default_config(nat.VARIANT_CPP, preconditioner=nat.PRECOND_MG, **base), rho)
    u_j, st_j = p.solve(nat.default_config(nat.VARIANT_CPP, **base), rho)
    s = O.scales(0, rho.ravel(), None, 3.0, 1e-9, 0.01, 1.0)
    ref, _, _ = O.pcg(shape, O.ke(), s, fixed, F, tol=1e-13)
    assert st_mg.converged and st_mg.residual <= 1e-8
    assert np.linalg.norm(u_mg - ref) / np.linalg.norm(ref) <= 1e-6
    assert np.linalg.norm(u_j - ref) / np.linalg.norm(ref) <= 1e-6
    # one V-cycle per outer iteration: far fewer than Jacobi PCG's iterations
    assert st_mg.iterations == st_mg.outer_iterations
    assert 5 * st_mg.iterations < st_j.iterations, (st_mg.iterations, st_j.iterations)


def test_mg_simp_matches_oracle():
    shape = (32, 16, 8)
    F, fixed = _cantilever(shape)
    iters = 8
    prm = O.make_params(volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                        convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12, warm_start=1)
    ref = O.simp_cpp(shape, 1.0, 1.0, 0.3, prm, np.full(shape, 0.3), F, fixed)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    cfg = nat.default_config(nat.VARIANT_CPP, volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01,
                             E_min=1e-9, convergence_tol=0.0, max_iterations=iters, cg_tol=1e-10,
                             preconditioner=nat.PRECOND_MG)
    r = p.simp_run(cfg, np.full(shape, 0.3))
    rel = np.abs(r["compliance"] - ref["compliance"]) / ref["compliance"]
    assert rel.max() <= 1e-6, rel
    assert np.abs(r["density"] - ref["density"].ravel()).max() <= 1e-4


def test_mg_on_a_rough_density_falls_back_to_jacobi():
    """White-noise densities (contrast 1e6 between neighbours): the averaged coarse
    grids do not represent the operator, the V-cycle stops helping and the solve
    continues on Jacobi-PCG inner solves to the same answer."""
    shape = (32, 16, 16)
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.01, 1.0, size=shape)
    F, fixed = _cantilever(shape)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    u, st = p.solve(nat.default_config(nat.VARIANT_CPP, preconditioner=nat.PRECOND_MG, E_min=1e-9, rho_min=0.01,
                                       cg_tol=1e-8, warm_start=0), rho)
    s = O.scales(0, rho.ravel(), None, 3.0, 1e-9, 0.01, 1.0)
    ref, _, _ = O.pcg(shape, O.ke(), s, fixed, F, tol=1e-13)
    assert st.converged and st.residual <= 1e-8
    assert np.linalg.norm(u - ref) / np.linalg.norm(ref) <= 1e-6


def test_mg_on_a_grid_that_does_not_coarsen_uses_jacobi():
    shape = (7, 5, 3)
    F, fixed = _cantilever(shape)
    rho = np.full(shape, 0.5)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    u, st = p.solve(nat.default_config(nat.VARIANT_CPP, preconditioner=nat.PRECOND_MG, cg_tol=1e-9,
                                       warm_start=0), rho)
    s = O.scales(0, rho.ravel(), None, 3.0, 1e-6, 0.01, 1.0)
    ref, _, _ = O.pcg(shape, O.ke(), s, fixed, F, tol=1e-13)
    assert st.converged
    assert np.linalg.norm(u - ref) / np.linalg.norm(ref) <= 1e-6


def _floating_pad(shape):
    """A passive solid column (grid = 1, full height) inside a two-element ring of
    near-void design material (rho 0.011: 1e-6 of the pad's stiffness), the rest at
    0.5: the pad's rigid-body motions are near-null modes of K."""
    nx, ny, nz = shape
    grid = np.zeros(shape, dtype=np.int8)
    x0, y0 = 3 * nx // 4 - 2, ny // 2 - 2
    grid[x0:x0 + 4, y0:y0 + 4, :] = 1
    rho = np.full(shape, 0.5)
    rho[x0 - 2:x0 + 6, y0 - 2:y0 + 6, :] = 0.011
    rho[grid == 1] = 1.0
    return grid, rho


def test_mg_deflation_of_a_floating_pad_matches_oracle():
    shape = (48, 24, 24)
    grid, rho = _floating_pad(shape)
    F, fixed = _cantilever(shape)
    p = nat.Problem(shape, 1.0, 1.0, 0.3, grid=grid)
    p.set_loads([F], [fixed])
    base = dict(E_min=1e-9, rho_min=0.01, cg_tol=1e-8, warm_start=0, preconditioner=nat.PRECOND_MG)
    u_d, st_d = p.solve(nat.default_config(nat.VARIANT_CPP, mg_deflation=1, **base), rho)
    u_0, st_0 = p.solve(nat.default_config(nat.VARIANT_CPP, mg_deflation=0, **base), rho)
    s = O.scales(0, rho.ravel(), grid.ravel(), 3.0, 1e-9, 0.01, 1.0)
    ref, _, _ = O.pcg(shape, O.ke(), s, fixed, F, tol=1e-13)
    for u, st in ((u_d, st_d), (u_0, st_0)):
        assert st.converged and st.residual <= 1e-8
        assert np.linalg.norm(u - ref) / np.linalg.norm(ref) <= 1e-6
    # the balanced V-cycle carries the whole solve (no Jacobi fallback) and needs
    # no more iterations than the V-cycle alone
    assert st_d.iterations == st_d.outer_iterations, (st_d.iterations, st_d.outer_iterations)
    assert st_d.iterations <= st_0.iterations, (st_d.iterations, st_0.iterations)


def test_mg_deflation_simp_with_passive_pads_matches_oracle():
    """SIMP with two passive solid columns (rho0 = 1: outside the design mask) and
    the balanced V-cycle: compliance history and densities as the FP64 oracle."""
    shape = (32, 16, 8)
    F, fixed = _cantilever(shape)
    rho0 = np.full(shape, 0.3)
    rho0[22:25, 2:5, :] = 1.0
    rho0[22:25, 11:14, :] = 1.0
    iters = 8
    prm = O.make_params(volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                        convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12, warm_start=1)
    ref = O.simp_cpp(shape, 1.0, 1.0, 0.3, prm, rho0, F, fixed)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    cfg = nat.default_config(nat.VARIANT_CPP, volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01,
                             E_min=1e-9, convergence_tol=0.0, max_iterations=iters, cg_tol=1e-10,
                             preconditioner=nat.PRECOND_MG, mg_deflation=1)
    r = p.simp_run(cfg, rho0)
    rel = np.abs(r["compliance"] - ref["compliance"]) / ref["compliance"]
    assert rel.max() <= 1e-6, rel
    assert np.abs(r["density"] - ref["density"].ravel()).max() <= 1e-4


def test_mg_deflation_simp_py_with_passive_pads_matches_oracle():
    """The Python variant with two passive solid columns marked in the grid (grid = 1:
    scale 1 whatever the density): the balanced V-cycle against the FP64 oracle."""
    shape = (32, 16, 8)
    F, fixed = _cantilever(shape)
    grid = np.zeros(shape, np.int8)
    grid[22:25, 2:5, :] = 1
    grid[22:25, 11:14, :] = 1
    iters = 6
    prm = O.make_params(volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                        convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12)
    ref = O.simp_py(shape, 1.0, 1.0, 0.3, prm, grid, [F], [fixed])
    p = nat.Problem(shape, 1.0, 1.0, 0.3, grid=grid)
    p.set_loads([F], [fixed])
    cfg = nat.default_config(nat.VARIANT_PY, volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01,
                             E_min=1e-9, convergence_tol=0.0, max_iterations=iters, cg_tol=1e-10,
                             preconditioner=nat.PRECOND_MG, mg_deflation=1)
    r = p.simp_run(cfg)
    rel = np.abs(r["compliance"] - ref["compliance"]) / ref["compliance"]
    assert rel.max() <= 1e-6, rel
    assert np.abs(r["density"] - ref["density"].ravel()).max() <= 1e-4
