"""Batched SIMP (am_batch_*): independent C++-variant problems of uneven sizes
solved together, checked problem by problem against the FP64 oracle and the
single-problem engine."""
import numpy as np
import pytest

import oracle as O
from am_ml_suite_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _point_load_case(shape, rng):
    """Clamped x = 0 face, one unit load at a random node of the x = max face in a
    random unit direction (the batched-cantilever workload)."""
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    fixed = (3 * base[:, None] + np.arange(3)).ravel()
    j, k = int(rng.integers(0, ny + 1)), int(rng.integers(0, nz + 1))
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    F = np.zeros(N)
    node = nx * (ny + 1) * (nz + 1) + j * (nz + 1) + k
    F[3 * node:3 * node + 3] = d
    return F, fixed


def _batch(shapes, seed=0):
    rng = np.random.default_rng(seed)
    loads = [_point_load_case(s, rng) for s in shapes]
    b = nat.Batch(shapes)
    b.set_loads([F for F, _ in loads], [fx for _, fx in loads])
    return b, loads


def _cfg(iters, vf=0.3, rmin=1.5, tol=1e-9, conv=0.0):
    return nat.default_config(nat.VARIANT_CPP, volume_fraction=vf, filter_radius=rmin, move_limit=0.2,
                              rho_min=0.01, E_min=1e-9, convergence_tol=conv, max_iterations=iters,
                              cg_tol=tol)


SHAPES = [(12, 6, 4), (17, 8, 6), (9, 5, 7), (20, 4, 3)]


def test_batch_matches_oracle_per_problem():
    """Per-iteration compliance <= 1e-6 relative and densities <= 1e-4 against the
    oracle's FP64 SIMP of each problem (solves to 1e-12), with per-problem volume
    fractions and filter radii."""
    iters = 6
    b, loads = _batch(SHAPES, seed=1)
    params = [(0.3, 1.5), (0.4, 2.0), (0.25, 1.2), (0.5, 2.5)]
    cfgs = [_cfg(iters, vf, r) for vf, r in params]
    res = b.simp_run(cfgs)
    for shape, (F, fixed), (vf, r), out in zip(SHAPES, loads, params, res):
        prm = O.make_params(volume_fraction=vf, filter_radius=r, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                            convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12, warm_start=1)
        ref = O.simp_cpp(shape, 1.0, 1.0, 0.3, prm, np.full(shape, vf), F, fixed)
        assert out["iterations"] == iters
        rel = np.abs(out["compliance"] - ref["compliance"]) / ref["compliance"]
        assert rel.max() <= 1e-6, (shape, rel)
        assert np.abs(out["density"] - ref["density"].ravel()).max() <= 1e-4, shape
        assert np.allclose(out["volume"], ref["volume"], rtol=0, atol=1e-9)
        assert out["pcg_iterations"] > 0


def test_batch_matches_single_problem_engine():
    iters = 4
    b, loads = _batch(SHAPES[:3], seed=2)
    res = b.simp_run([_cfg(iters) for _ in SHAPES[:3]])
    for shape, (F, fixed), out in zip(SHAPES[:3], loads, res):
        p = nat.Problem(shape)
        p.set_loads([F], [fixed])
        single = p.simp_run(_cfg(iters), np.full(shape, 0.3))
        rel = np.abs(out["compliance"] - single["compliance"]) / single["compliance"]
        assert rel.max() <= 1e-6
        assert np.abs(out["density"] - single["density"]).max() <= 1e-4


def test_batch_autotune_keeps_results():
    iters = 3
    b, _ = _batch(SHAPES, seed=3)
    before = b.simp_run([_cfg(iters) for _ in SHAPES])
    plan = b.autotune(reps=2)
    assert plan["warps"] in (4, 8) and plan["z_chunk"] in (0, 8, 16) and plan["ctas_per_sm"] in (1, 2, 4)
    assert plan["ms"] > 0
    after = b.simp_run([_cfg(iters) for _ in SHAPES])
    for x, y in zip(before, after):
        assert np.allclose(x["compliance"], y["compliance"], rtol=1e-7, atol=0)
        assert np.abs(x["density"] - y["density"]).max() <= 1e-6


def test_batch_per_problem_iteration_limits_and_convergence():
    b, _ = _batch(SHAPES[:3], seed=4)
    cfgs = [_cfg(3), _cfg(5), _cfg(0)]
    res = b.simp_run(cfgs)
    assert [r["iterations"] for r in res] == [3, 5, 0]
    assert res[2]["pcg_iterations"] == 0
    assert np.allclose(res[2]["density"], 0.3)  # untouched initial density
    # a loose convergence tolerance stops a problem early
    b2, _ = _batch(SHAPES[:2], seed=4)
    out = b2.simp_run([_cfg(20, conv=0.5), _cfg(2)])
    assert out[0]["converged"] and out[0]["iterations"] < 20
    assert not out[1]["converged"] and out[1]["iterations"] == 2


def test_batch_errors():
    with pytest.raises(nat.AmError) as e:
        nat.Batch([(4, 4, 0)])
    assert e.value.name == "AM_ERR_INVALID_ARG"
    b = nat.Batch([(4, 3, 2), (3, 3, 3)])
    with pytest.raises(nat.AmError) as e:
        b.simp_run([_cfg(1), _cfg(1)])
    assert e.value.name == "AM_ERR_INVALID_ARG"  # loads not set
    F0 = np.zeros(b.N[0])
    F1 = np.zeros(b.N[1])
    with pytest.raises(nat.AmError) as e:
        b.set_loads([F0, F1], [np.array([0]), np.array([b.N[1] + 3])])
    assert e.value.name == "AM_ERR_DOF_OUT_OF_RANGE"
    b.set_loads([F0, F1], [np.array([0]), np.array([1])])
    py = nat.default_config(nat.VARIANT_PY, max_iterations=1)
    with pytest.raises(nat.AmError) as e:
        b.simp_run([_cfg(1), py])
    assert e.value.name == "AM_ERR_INVALID_ARG"


def test_batch_step_api_matches_run():
    iters = 3
    b, _ = _batch(SHAPES[:3], seed=5)
    cfgs = [_cfg(iters), _cfg(2), _cfg(iters)]
    run = b.simp_run(cfgs)
    b.simp_begin(cfgs)
    hist = []
    for k, expect_active in zip(range(iters), (3, 2, 0)):
        c, v, d, active = b.simp_step()
        hist.append(c)
        assert active == expect_active
    assert np.isnan(hist[2][1])  # problem 1 stopped after 2 iterations
    dens = b.densities()
    for p, r in enumerate(run):
        got = np.array([h[p] for h in hist[:r["iterations"]]])
        assert np.allclose(got, r["compliance"], rtol=1e-12, atol=0)
        assert np.array_equal(dens[p], r["density"])
        assert b.pcg_iterations[p] == r["pcg_iterations"]


def test_batch_device_loop_matches_host_loop():
    """The batch's FP32 PCG rounds driven by the device-side graph loop (default)
    and chunk by chunk from the host run the same kernels in the same order:
    identical compliance histories, densities and PCG iteration counts."""
    out = []
    for on in (True, False):
        b, _ = _batch(SHAPES, seed=9)
        b.set_device_loop(on)
        res = b.simp_run([_cfg(4, tol=1e-7) for _ in SHAPES])
        out.append((res, [r["pcg_iterations"] for r in res]))
        b.close()
    (dev, it_dev), (host, it_host) = out
    assert it_dev == it_host and min(it_dev) > 0
    for a, h in zip(dev, host):
        assert np.array_equal(a["compliance"], h["compliance"])
        assert np.array_equal(a["density"], h["density"])


def test_batch_per_problem_tile_heights():
    """Plan warps = 0: each problem computes its K*u with the tile height (7 or 15
    node rows) that overhangs its grid least -- here a 7-row and a 15-row problem
    land in different kernels -- and every problem still matches the FP64 oracle;
    the plan is pinned and invalid plans are refused."""
    shapes = [(12, 6, 4), (17, 14, 6), (9, 5, 7), (20, 13, 3)]
    iters = 4
    b, loads = _batch(shapes, seed=11)
    b.set_plan(0, 0, 2)
    res = b.simp_run([_cfg(iters) for _ in shapes])
    for (shape, (F, fixed)), r in zip(zip(shapes, loads), res):
        prm = O.make_params(volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                            convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12, warm_start=1)
        ref = O.simp_cpp(shape, 1.0, 1.0, 0.3, prm, np.full(shape, 0.3), F, fixed)
        assert np.allclose(r["compliance"], ref["compliance"], rtol=1e-6, atol=0)
        assert np.abs(r["density"] - ref["density"].ravel()).max() <= 1e-4
    with pytest.raises(nat.AmError):
        b.set_plan(6)
    with pytest.raises(nat.AmError):
        b.set_plan(8, 0, 7)


def test_batch_axis_order_and_layouts():
    """Each problem is stored in the axis order whose K*u tiles overhang it least:
    (6, 40, 9) keeps its 40-element axis in the 30-column tile direction and its
    6-element axis as the marching axis, (9, 5, 7) swaps y and z, (20, 4, 3) keeps
    the caller's order.  Loads, constraints, non-uniform initial densities (both
    density layouts) and the results cross the boundary in the caller's order:
    every problem matches the FP64 oracle of its unpermuted grid."""
    shapes = [(6, 40, 9), (9, 5, 7), (20, 4, 3)]
    b, loads = _batch(shapes, seed=5)
    assert [b.axes(i) for i in range(3)] == [(1, 2, 0), (0, 2, 1), (0, 1, 2)]
    iters = 4
    rng = np.random.default_rng(6)
    rho0 = [rng.uniform(0.2, 0.5, size=s) for s in shapes]
    layouts = [nat.LAYOUT_ZFASTEST, nat.LAYOUT_XFASTEST, nat.LAYOUT_XFASTEST]
    cfgs = [_cfg(iters) for _ in shapes]
    for c, lay in zip(cfgs, layouts):
        c.layout = lay
    host = [r.ravel() if lay == nat.LAYOUT_ZFASTEST else r.ravel(order="F") for r, lay in zip(rho0, layouts)]
    res = b.simp_run(cfgs, host)
    for shape, (F, fixed), r0, lay, out in zip(shapes, loads, rho0, layouts, res):
        prm = O.make_params(volume_fraction=0.3, filter_radius=1.5, move_limit=0.2, rho_min=0.01, E_min=1e-9,
                            convergence_tol=0.0, max_iterations=iters, cg_tol=1e-12, warm_start=1)
        ref = O.simp_cpp(shape, 1.0, 1.0, 0.3, prm, r0, F, fixed)
        assert np.allclose(out["compliance"], ref["compliance"], rtol=1e-6, atol=0), shape
        got = out["density"].reshape(shape) if lay == nat.LAYOUT_ZFASTEST else \
            out["density"].reshape(shape, order="F")
        assert np.abs(got - ref["density"].reshape(shape)).max() <= 1e-4, shape
    with pytest.raises(nat.AmError):
        b.axes(3)


def test_batch_staged_ku_matches_warp_row_ku():
    """The batch's FP32 PCG K*u on the tensor-copy staged kernel (default, one CTA
    per 28 x 15-node tile of a problem, tensor maps in device memory) and on the
    warp-row kernel compute the same p and q; their p.q sums run over different
    tiles, so two batches solved to rel-res 1e-9 agree to rounding: compliance
    within 1e-7, densities within 1e-6."""
    out = []
    for staged in (True, False):
        b, _ = _batch(SHAPES, seed=13)
        b.set_staged(staged)
        out.append(b.simp_run([_cfg(4) for _ in SHAPES]))
        b.close()
    for x, y in zip(*out):
        assert x["pcg_iterations"] > 0 and y["pcg_iterations"] > 0
        assert np.allclose(x["compliance"], y["compliance"], rtol=1e-7, atol=0)
        assert np.abs(x["density"] - y["density"]).max() <= 1e-6


def test_batch_bench_ku_restores_state():
    """am_batch_bench_ku times the PCG K*u of either kernel between SIMP steps and
    leaves the solver state as it found it: the steps after it are bitwise those of
    an uninterrupted run."""
    ref, _ = _batch(SHAPES, seed=17)
    cfgs = [_cfg(4, tol=1e-7) for _ in SHAPES]
    ref.simp_begin(cfgs)
    hist_ref = [ref.simp_step()[0] for _ in range(4)]
    b, _ = _batch(SHAPES, seed=17)
    b.simp_begin(cfgs)
    hist = [b.simp_step()[0] for _ in range(2)]
    assert b.bench_ku(reps=3) > 0
    b.set_staged(False)
    assert b.bench_ku(reps=3) > 0
    b.set_staged(True)
    hist += [b.simp_step()[0] for _ in range(2)]
    for h, r in zip(hist, hist_ref):
        assert np.array_equal(h, r)
    for p in range(len(SHAPES)):
        assert np.array_equal(b.densities()[p], ref.densities()[p])
