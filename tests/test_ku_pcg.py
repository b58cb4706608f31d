"""Parity of the FP32 inner-PCG K*u step -- the kernel every inner iteration of a
mixed-precision solve runs -- through the C ABI (am_ku_pcg_step).

The step: p = D^-1 r + beta p_prev, q = mask(K p), p.q, with D the Jacobi
diagonal and mask zeroing the fixed and orphan DOFs.  Checked against
  * the FP64 oracle: p within 1e-6 of max|p| (FP32 inputs and product), q against
    the oracle's K applied to the returned p within 2e-6 of max|q| (the FP32 K*u
    tolerance), masked DOFs exactly 0, p.q against numpy's dot of the returned
    vectors within 1e-6 of sum |p||q| (a node's three products are summed in
    FP32, the nodes in double-float);
  * the staged kernel without a CTA-wide barrier per plane (impl 4) and the
    register-direct kernel (impl 2): p and q bitwise equal, p.q equal to the
    impl-4 kernel's;
  * the staged kernel on 7-warp tiles (13 node rows, am_problem_set_ku_plan): p
    bitwise equal; q within one FP32 rounding of each node's sum (a node's
    contributions from the element rows above and below it are added in an order
    that depends on its row within a warp, so nodes whose row position differs
    between 13- and 15-row tiles round differently), exactly 0 on masked DOFs; p.q
    within rounding.
Shapes span several 28-column, 15-row and z-chunk tiles, odd remainders and a
single element.
"""
import numpy as np
import pytest

import oracle as O
from am_ml_suite_gb300 import _native as nat

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (7, 5, 4), (27, 14, 6), (28, 15, 9), (33, 9, 10), (57, 31, 21), (48, 24, 12)]


def _cantilever_fixed(shape):
    nx, ny, nz = shape
    base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    return (3 * base[:, None] + np.arange(3)).ravel()


def _node_diag(shape, s, ke00):
    nx, ny, nz = shape
    se = s.reshape(shape)
    acc = np.zeros((nx + 1, ny + 1, nz + 1))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                acc[dx:dx + nx, dy:dy + ny, dz:dz + nz] += se
    return (ke00 * acc).ravel()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("beta", [0.0, 0.37])
def test_pcg_step_matches_oracle_and_previous_kernel(shape, beta):
    nx, ny, nz = shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    N = 3 * nn
    rng = np.random.default_rng(sum(shape) + int(100 * beta))
    rho = rng.uniform(0.05, 1.0, size=shape)
    rho[rng.random(shape) < 0.15] = 1e-3  # below rho_min: skipped (C++ rule), orphaning some nodes
    fixed = _cantilever_fixed(shape)
    F = np.zeros(N)
    F[-1] = -1.0
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([F], [fixed])
    cfg = nat.default_config(nat.VARIANT_CPP, E_min=1e-9, rho_min=0.01)
    r = rng.normal(size=N)
    p_prev = rng.normal(size=N)

    p3, q3, pq3 = p.ku_pcg_step(cfg, rho, r, p_prev, beta, impl=3)
    p2, q2, pq2 = p.ku_pcg_step(cfg, rho, r, p_prev, beta, impl=2)
    p4, q4, pq4 = p.ku_pcg_step(cfg, rho, r, p_prev, beta, impl=4)
    assert np.array_equal(p3, p2) and np.array_equal(p4, p2)
    assert np.array_equal(q3, q2) and np.array_equal(q4, q2)
    # the barrier-per-plane and the barrier-free staged kernels sum in the same order
    assert pq3 == pq4

    s = O.scales(0, rho.ravel(), None, 3.0, 1e-9, 0.01, 1.0)
    ke = O.ke()
    d = _node_diag(shape, s, ke[0, 0])
    orphan = np.abs(d) < 1e-15
    dinv = np.where(orphan, 0.0, 1.0 / np.where(orphan, 1.0, d))
    p_ref = (dinv[:, None] * r.reshape(-1, 3) + beta * p_prev.reshape(-1, 3)).ravel()
    assert np.abs(p3 - p_ref).max() <= 1e-6 * np.abs(p_ref).max()

    mask = np.zeros((nn, 3), bool)
    mask[orphan] = True
    mask.reshape(-1)[fixed] = True
    mask = mask.ravel()
    q_ref = O.ku(shape, ke, s, p3)
    q_ref[mask] = 0.0
    assert np.all(q3[mask] == 0.0)
    assert np.abs(q3 - q_ref).max() <= 2e-6 * np.abs(q_ref).max()

    assert abs(pq3 - p3 @ q3) <= 1e-6 * (np.abs(p3) @ np.abs(q3))
    assert abs(pq3 - pq2) <= 1e-6 * (np.abs(p3) @ np.abs(q3))

    p.set_ku_plan(7)
    assert p.ku_plan()["warps"] == 7
    p7, q7, pq7 = p.ku_pcg_step(cfg, rho, r, p_prev, beta, impl=3)
    assert np.array_equal(p7, p2)
    assert np.all(q7[mask] == 0.0)
    assert np.abs(q7 - q2).max() <= 1e-6 * np.abs(q2).max()
    assert np.abs(q7 - q_ref).max() <= 2e-6 * np.abs(q_ref).max()
    assert abs(pq7 - pq3) <= 1e-6 * (np.abs(p3) @ np.abs(q3))
    p.set_ku_plan(0)
    assert p.ku_plan()["warps"] == 8  # small grids keep the 8-warp tiles


def test_ku_plan_tile_height_by_grid():
    """The staged K*u's plan: one wave of tiles with the longest z chunks, on the
    tile height whose one wave fills more CTA slots -- 7-warp tiles on the
    256x128x128 cantilever (10 x 10 columns x 3 chunks of 43 planes = 300 tiles),
    8-warp tiles on the 192x96x96 bracket (7 x 7 x 6 chunks of 17 = 294); the plan
    is computed when the problem is created, before any vector is allocated."""
    p = nat.Problem((256, 128, 128))
    assert p.ku_plan() == {"warps": 7, "tiles": 300, "z_chunk": 43}
    p.set_ku_plan(8)
    assert p.ku_plan() == {"warps": 8, "tiles": 270, "z_chunk": 43}
    p.close()
    p = nat.Problem((192, 96, 96))
    assert p.ku_plan() == {"warps": 8, "tiles": 294, "z_chunk": 17}
    with pytest.raises(nat.AmError):
        p.set_ku_plan(6)
    p.close()


def test_pcg_step_rejects_bad_arguments():
    shape = (4, 3, 2)
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    N = p.N
    p.set_loads([np.zeros(N)], [_cantilever_fixed(shape)])
    cfg = nat.default_config(nat.VARIANT_CPP)
    rho = np.full(shape, 0.5)
    with pytest.raises(nat.AmError):
        p.ku_pcg_step(cfg, rho, np.zeros(N), np.zeros(N), 0.5, impl=7)
    with pytest.raises(nat.AmError):
        p.ku_pcg_step(cfg, rho, np.zeros(N), np.zeros(N), float("nan"))
    with pytest.raises(nat.AmError):
        p.ku_pcg_step(cfg, rho, np.zeros(N), np.zeros(N), 0.5, load_case=3)
