"""BRK-A-01 set-up on the device (am_bracket_build; core.create_bracket_domain,
create_brk_a_01_static_case_1/2) against the reference's own outputs: the voxel
grid cell for cell, the eyelet load ring node for node in the reference's order,
the force vectors bit for bit and the base constraints, at six resolutions
(tests/golden/bracket_golden.npz, made by importing the reference), plus the
C++ driver's x-fastest grid and force vector (the restated am_topopt run in
reference_golden.npz)."""
import os

import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat
from am_ml_suite_gb300 import core

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bracket_golden.npz"))
RES = [float(r) for r in GOLD["resolutions"]]


@pytest.mark.parametrize("r", RES)
def test_bracket_grid_matches_reference(r):
    dom = core.create_bracket_domain(resolution_mm=r)
    ref = GOLD[f"r{r:g}_grid"]
    assert dom.shape == ref.shape
    assert np.array_equal(dom.grid, ref)
    assert dom.n_fixed == int((ref == 1).sum()) and dom.n_design == int((ref == 0).sum())


@pytest.mark.parametrize("r", RES)
def test_brk_load_cases_match_reference(r):
    key = f"r{r:g}"
    shape = GOLD[f"{key}_grid"].shape
    N = 3 * int(np.prod(np.array(shape) + 1))
    c1 = core.create_brk_a_01_static_case_1(shape, r)
    assert np.array_equal(c1.distributed_loads[0].node_indices, GOLD[f"{key}_ring"])
    assert np.array_equal(c1.get_constrained_dofs(), GOLD[f"{key}_fixed"])
    for c, lc in ((1, c1), (2, core.create_brk_a_01_static_case_2(shape, r))):
        assert np.array_equal(lc.distributed_loads[0].total_force, GOLD[f"{key}_c{c}_total"])
        F = lc.get_force_vector(N)
        idx = np.flatnonzero(F)
        assert np.array_equal(idx, GOLD[f"{key}_c{c}_F_idx"])
        assert np.array_equal(F[idx], GOLD[f"{key}_c{c}_F_val"])
        # the force vector formed on the device
        Fd = core.bracket_force_vector(shape, r, GOLD[f"{key}_c{c}_total"])
        assert np.array_equal(Fd, F)
    assert np.array_equal(core.bracket_fixed_dofs(shape, r), GOLD[f"{key}_fixed"])


def test_cpp_driver_layout_and_load(golden):
    """am_topopt's BracketDomain stores the same grid x-fastest; its force vector
    puts -15000 / n on the z component of every ring node (am_topopt.cpp:248-314)."""
    import ctypes

    g = golden["cpprun_grid"]  # C-order (nx, ny, nz) of the 4 mm run
    p = nat.BracketParams()
    nat.load().am_bracket_params_default(p, 4.0)
    assert (p.nx, p.ny, p.nz) == g.shape
    xf = np.zeros(g.size, np.int8)
    nat.check(nat.load().am_bracket_build(p, None, nat.LAYOUT_XFASTEST, nat.ptr(xf, nat._i8p), None, None, None,
                                          None, None, 0), "am_bracket_build")
    assert np.array_equal(xf, g.transpose(2, 1, 0).ravel())
    F = core.bracket_force_vector(g.shape, 4.0, [0.0, 0.0, -15000.0])
    assert np.array_equal(F, golden["cpprun_F"])
    assert np.array_equal(core.bracket_fixed_dofs(g.shape, 4.0), golden["cpprun_fixed"])
    # the notebook's 12 mm Python set-up
    dom = core.create_bracket_domain(size_mm=(120, 60, 80), resolution_mm=12.0)
    assert np.array_equal(dom.grid, golden["nb_grid"])
    lc = core.create_brk_a_01_static_case_1(dom.shape, 12.0)
    assert np.array_equal(lc.get_force_vector(golden["nb_F"].size), golden["nb_F"])
    assert np.array_equal(lc.get_constrained_dofs(), golden["nb_fixed"])
    # a ring buffer that is too small is refused
    small = np.zeros(1, np.int64)
    n = ctypes.c_int64(0)
    st = nat.load().am_bracket_build(p, None, nat.LAYOUT_ZFASTEST, None, None, None, None, nat.ptr(small, nat._i64p),
                                     ctypes.byref(n), 1)
    assert nat.STATUS[st] == "AM_ERR_SIZE_MISMATCH"


def test_bracket_simp_runs_on_device_setup():
    """The set-up feeds the Python SIMP drop-in directly: a 4 mm BRK-A-01 run,
    3 iterations, compliance positive and volume at the target."""
    from am_ml_suite_gb300.numerical.fem import MaterialProperties
    from am_ml_suite_gb300.numerical.topopt import SIMPOptimizer, SIMPParams

    dom = core.create_bracket_domain(resolution_mm=4.0)
    lc = core.create_brk_a_01_static_case_1(dom.shape, 4.0)
    prm = SIMPParams(volume_fraction=0.3, filter_radius=1.5, max_iterations=3, convergence_tol=0.0,
                     precision=nat.PREC_MIXED, cg_tol=1e-6)
    res = SIMPOptimizer(dom, [lc], MaterialProperties(), prm, verbose=False).run()
    assert res.iterations == 3 and all(c > 0 for c in res.compliance_history)
    assert abs(res.volume_history[-1] - 0.3) < 1e-3
