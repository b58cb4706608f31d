"""Device-side safety paths, exercised without a fault: a bounded copy wait on a
barrier that nothing completes gives up after its limit and reports it (the
solver's copy stages then end the solve with an error instead of spinning)."""
import pytest

from am_ml_suite_gb300 import _native as nat


@pytest.mark.gpu
@pytest.mark.parametrize("limit_ms", [2.0, 10.0])
def test_bounded_copy_wait_gives_up(limit_ms):
    timed_out, waited = nat.selftest_copy_wait(limit_ms)
    assert timed_out
    assert limit_ms <= waited < limit_ms + 50.0


def test_copy_wait_limits_are_checked():
    with pytest.raises(nat.AmError):
        nat.selftest_copy_wait(0.0)
    with pytest.raises(nat.AmError):
        nat.selftest_copy_wait(1000.0)


@pytest.mark.gpu
def test_copy_timeout_status_of_a_solve():
    """A PCG kernel that reports a copy wait that ran out ends the solve with
    AM_ERR_TIMEOUT (the flag is planted on the host; no wait runs out), and the
    problem solves normally afterwards."""
    import numpy as np

    shape = (12, 6, 6)
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    fixed = (3 * base[:, None] + np.arange(3)).ravel()
    F = np.zeros(N)
    F[3 * (nx * (ny + 1) * (nz + 1)) + 2] = -1.0
    p = nat.Problem(shape)
    p.set_loads([F], [fixed])
    rho = np.full(shape, 0.5)
    cfg = nat.default_config(nat.VARIANT_CPP, precision=nat.PREC_MIXED, cg_tol=1e-8)
    st = p.selftest_solve_timeout(cfg, rho)
    assert nat.STATUS[st] == "AM_ERR_TIMEOUT"
    assert b"timed out" in nat.load().am_last_error()
    u, stats = p.solve(cfg, rho)
    assert stats.converged and stats.residual <= 1e-8
    p.close()
